"""PirParams: the reference's parameter derivation (src/pir.cpp:9-112,
src/includes/pir.h:18-86) over the presets of src/includes/database_constants.h.

Host logic only (no GPU needed).  Prime selection follows SEAL's
``CoeffModulus::Create`` (the largest primes below 2^bits that are 1 mod 2N,
handed out in descending order) and ``utils::generate_prime``
(utils.cpp:82-95).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Dict, List, Sequence

POLY_DEGREE = 2048


def is_prime(n: int) -> bool:
    if n < 2:
        return False
    small = (2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37)
    for b in small:
        if n == b:
            return True
        if n % b == 0:
            return False
    d, s = n - 1, 0
    while d % 2 == 0:
        d //= 2
        s += 1
    for b in small:
        x = pow(b, d, n)
        if x in (1, n - 1):
            continue
        for _ in range(s - 1):
            x = x * x % n
            if x == n - 1:
                break
        else:
            return False
    return True


def generate_prime(bit_width: int) -> int:
    """utils::generate_prime: smallest prime reached by ++, |= 1 from 2^(bits-1)."""
    if bit_width < 2:
        raise ValueError("Bit width must be at least 2.")
    c = 1 << (bit_width - 1)
    while True:
        c += 1
        c |= 1
        if is_prime(c):
            return c


def coeff_modulus_create(n: int, bit_sizes: Sequence[int]) -> List[int]:
    """SEAL CoeffModulus::Create(n, bit_sizes) (called at pir.cpp:23,40)."""
    out = []
    for i, b in enumerate(bit_sizes):
        rank = sum(1 for j in range(i) if bit_sizes[j] == b)
        step = 2 * n
        v = (1 << b) - step + 1
        found = 0
        while True:
            if v <= (1 << (b - 1)):
                raise ValueError(f"not enough {b}-bit primes for N={n}")
            if is_prime(v):
                if found == rank:
                    break
                found += 1
            v -= step
        out.append(v)
    return out


def next_pow_of_2(n: int) -> int:
    p = 1
    while p < n:
        p <<= 1
    return p


def roundup_div(a: int, b: int) -> int:
    if b == 0:
        raise ValueError("roundup_div division by zero")
    return (a + b - 1) // b


# The N = 2048 presets of database_constants.h (the active one is
# "2^16 * 4KB = 256MB (quick test)", database_constants.h:215-223).
PRESETS: Dict[str, dict] = {
    "quick_test_256MB": dict(max_fst_dim=256, num_entries=1 << 16),
    "512MB": dict(max_fst_dim=512, num_entries=1 << 17),
    "1GB": dict(max_fst_dim=512, num_entries=1 << 18),
    "8GB_best_throughput": dict(max_fst_dim=512, num_entries=1 << 21),
}

# The N = 4096 presets with two ciphertext primes (CoeffMods = {60, 60, 60},
# database_constants.h:13-172) share these ciphertext parameters; the
# "2^14 * 24KB = 384MB" preset (database_constants.h:92-101) is the one the
# tests and the benchmark use.
RNS4096 = dict(poly_degree=4096, gsw_l=4, gsw_l_key=8, plain_mod_bits=46, small_q_width=57,
               coeff_mods=(60, 60, 60))
PRESETS["n4096_384MB"] = dict(max_fst_dim=256, num_entries=1 << 14, **RNS4096)
PRESETS["n4096_1GB"] = dict(max_fst_dim=256, num_entries=1 << 20, entry_size_cfg=1024, **RNS4096)

# Workloads used by the tests and the benchmark (sizes as named).
WORKLOADS: Dict[str, dict] = {
    # 256 x 2^4 = 4096 plaintexts (CPU-runnable reference case)
    "db4096": dict(max_fst_dim=256, num_entries=4096),
    # 512 x 2^6 = 32,768 plaintexts, 537 MB NTT form (small profiling case, > L2)
    "db32768": dict(max_fst_dim=512, num_entries=1 << 15),
    # 128 x 2^9 = 65,536 plaintexts, 1.07 GB NTT form: the scan's tile and
    # work split of the 262,144-plaintext case at a quarter of the size
    # (profiling case)
    "db65536": dict(max_fst_dim=128, num_entries=1 << 16),
    # 512 x 2^9 = 262,144 plaintexts, ~1 GB raw entries, 4.29 GB NTT form
    "db262144": dict(max_fst_dim=512, num_entries=1 << 18),
    # 1024 x 2^11 = 2,097,152 plaintexts, ~8 GB raw entries, 34.4 GB NTT form
    "db2097152": dict(max_fst_dim=1024, num_entries=1 << 21),
    # N = 4096 with two ciphertext primes: 256 x 2^2 = 1024 plaintexts of
    # 23,040-byte entries (parity-test case)
    "rns1024": dict(max_fst_dim=256, num_entries=1024, **RNS4096),
    # 256 x 2^6 = 16,384 plaintexts: the "2^14 * 24KB = 384MB" preset,
    # 1.07 GB in NTT form over the two primes
    "rns16384": dict(max_fst_dim=256, num_entries=1 << 14, **RNS4096),
}


@dataclass
class PirParams:
    """PirParams::PirParams (pir.cpp:29-95)."""

    num_entries: int = 1 << 16
    max_fst_dim: int = 256
    entry_size_cfg: int = 0          # 0: largest entry that fits a plaintext
    gsw_l: int = 5                   # DatabaseConstants::GSW_L
    gsw_l_key: int = 10              # DatabaseConstants::GSW_L_KEY
    plain_mod_bits: int = 16         # DatabaseConstants::PlainMod
    small_q_width: int = 27          # DatabaseConstants::SmallQWidth
    coeff_mods: Sequence[int] = (60, 60)
    poly_degree: int = POLY_DEGREE
    dims: List[int] = field(default_factory=list, init=False)

    def __post_init__(self):
        n = self.poly_degree
        self.plain_mod = generate_prime(self.plain_mod_bits)              # pir.cpp:18
        self.coeff_modulus = coeff_modulus_create(n, list(self.coeff_mods))  # pir.cpp:22-23
        self.small_q = coeff_modulus_create(n, [self.small_q_width, self.coeff_mods[-1]])[0]
        bits_per_coeff = self.plain_mod.bit_length() - 1
        self.entry_size = (self.entry_size_cfg if self.entry_size_cfg
                           else bits_per_coeff * n // 8)                     # pir.cpp:34-38
        logq = sum(q.bit_length() for q in self.coeff_modulus[:-1])
        self.base_log2 = (logq + self.gsw_l - 1) // self.gsw_l              # pir.cpp:53
        self.base_log2_key = (logq + self.gsw_l_key - 1) // self.gsw_l_key  # pir.cpp:54
        if self.get_num_entries_per_plaintext() == 0:
            raise ValueError("Number of entries per plaintext is 0, possibly due to too large "
                             "entry size")
        num_pt_required = roundup_div(self.num_entries, self.get_num_entries_per_plaintext())
        other = roundup_div(next_pow_of_2(num_pt_required), self.max_fst_dim)  # pir.cpp:70
        first = roundup_div(num_pt_required, other)                            # pir.cpp:72
        self.num_pt = first * other
        self.num_entries = self.num_pt * self.get_num_entries_per_plaintext()
        ndim = 1 + int(math.log2(other))                                       # pir.cpp:89
        self.dims = [first] + [2] * (ndim - 1)
        if not 1 <= self.get_rns_mod_cnt() <= 2:
            raise ValueError("one or two ciphertext primes (CoeffMods of length 2 or 3) are "
                             "supported")
        if n not in (1024, 2048, 4096):
            raise ValueError("poly_degree must be 1024, 2048 or 4096")

    @classmethod
    def preset(cls, name: str, **kw) -> "PirParams":
        d = dict(WORKLOADS.get(name) or PRESETS[name])
        d.update(kw)
        return cls(**d)

    # ---- getters (pir.h:29-68)
    def get_num_bits_per_coeff(self) -> int:
        return self.plain_mod.bit_length() - 1

    def get_num_bits_per_plaintext(self) -> int:
        return self.get_num_bits_per_coeff() * self.poly_degree

    def get_num_entries_per_plaintext(self) -> int:
        return self.get_num_bits_per_plaintext() // (self.entry_size * 8)

    def get_num_entries(self) -> int:
        return self.num_entries

    def get_num_pt(self) -> int:
        return self.num_pt

    def get_entry_size(self) -> int:
        return self.entry_size

    def get_dims(self) -> List[int]:
        return list(self.dims)

    def get_l(self) -> int:
        return self.gsw_l

    def get_l_key(self) -> int:
        return self.gsw_l_key

    def get_small_q(self) -> int:
        return self.small_q

    def get_base_log2(self) -> int:
        return self.base_log2

    def get_base_log2_key(self) -> int:
        return self.base_log2_key

    def get_fst_dim_sz(self) -> int:
        return self.dims[0]

    def get_other_dim_sz(self) -> int:
        return self.num_pt // self.dims[0]

    def get_rns_mod_cnt(self) -> int:
        return len(self.coeff_modulus) - 1

    def get_coeff_val_cnt(self) -> int:
        return self.poly_degree * self.get_rns_mod_cnt()

    def get_plain_mod(self) -> int:
        return self.plain_mod

    def get_coeff_modulus(self) -> List[int]:
        return list(self.coeff_modulus[:-1])

    def get_expan_height(self) -> int:
        return math.ceil(math.log2(self.dims[0] + self.gsw_l * (len(self.dims) - 1)))

    def get_DBSize_MB(self) -> float:
        return self.num_entries * self.entry_size / 1024 / 1024

    def is_multi_modulus(self) -> bool:
        """True for parameter sets served by the multi-modulus path
        (opir_ctx_create_rns): more than one ciphertext prime, or N != 2048."""
        return self.get_rns_mod_cnt() > 1 or self.poly_degree != POLY_DEGREE

    def get_physical_storage_MB(self) -> float:
        return self.get_coeff_val_cnt() * self.num_pt * 8 / 1024 / 1024

    def small_q_width_bits(self) -> int:
        return math.ceil(math.log2(self.small_q))

    def response_bytes(self) -> int:
        return (2 * self.poly_degree * self.small_q_width_bits() + 7) // 8
