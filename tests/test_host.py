"""Host-side logic (no GPU): parameter derivation, the C ABI library loads
and exports every symbol include/onionpir_gpu.h declares, synthetic entries."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    text = open(os.path.join(ROOT, "include", "onionpir_gpu.h")).read()
    return sorted(set(re.findall(r"\b(opir_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(gpu_lib):
    from onionpirv2_gb300 import _capi
    syms = header_symbols()
    assert len(syms) >= 20
    assert sorted(_capi.EXPORTS) == syms
    lib = ctypes.CDLL(_capi.LIB)
    for s in syms:
        assert hasattr(lib, s), s


def test_ctypes_structs_match_the_c_header(tmp_path):
    """Every ctypes mirror of an include/onionpir_gpu.h struct has the C
    layout: size and each field's offset, from a program gcc compiles
    against the header."""
    import shutil
    import subprocess
    from onionpirv2_gb300 import _capi
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    mirrors = {"opir_params": _capi.OpirParams, "opir_db_shape": _capi.OpirDbShape,
               "opir_serve_config": _capi.OpirServeConfig,
               "opir_serve_stats": _capi.OpirServeStats,
               "opir_tune_report": _capi.OpirTuneReport,
               "opir_rns_params": _capi.OpirRnsParams}
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "onionpir_gpu.h"',
             "int main(void) {"]
    for cname, cls in mirrors.items():
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in cls._fields_:
            lines.append(f'  printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                   check=True, capture_output=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {tuple(line.split()[:2]): int(line.split()[2]) for line in out if line.strip()}
    for cname, cls in mirrors.items():
        assert got[(cname, "size")] == ctypes.sizeof(cls), cname
        for fname, _ in cls._fields_:
            assert got[(cname, fname)] == getattr(cls, fname).offset, (cname, fname)


def test_ctx_create_without_gpu_fails_cleanly(gpu_lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from onionpirv2_gb300 import PirParams, PirServer, OpirError
    with pytest.raises(OpirError):
        PirServer(PirParams(num_entries=4096, max_fst_dim=256))


@pytest.mark.parametrize("name", ["db4096", "db32768", "db262144", "db2097152",
                                  "quick_test_256MB", "1GB"])
def test_params_match_oracle(oracle_lib, name):
    from onionpirv2_gb300 import PirParams
    p = PirParams.preset(name)
    o = oracle_lib.Oracle(p.num_entries, p.max_fst_dim)
    P = o.P
    assert p.coeff_modulus == [P.q, P.p]
    assert (p.plain_mod, p.small_q, p.small_q_width_bits()) == (P.t, P.small_q, P.small_q_width)
    assert (p.base_log2, p.base_log2_key) == (P.base_log2, P.base_log2_key)
    assert (p.get_fst_dim_sz(), p.get_other_dim_sz(), len(p.get_dims())) == (P.n1, P.n_rest, P.ndim)
    assert p.get_num_pt() == P.num_pt and p.get_entry_size() == P.entry_size
    assert p.get_expan_height() == P.h
    assert p.response_bytes() == o.response_bytes()


def test_workload_shapes():
    from onionpirv2_gb300 import PirParams
    p = PirParams.preset("db262144")
    assert (p.get_fst_dim_sz(), p.get_other_dim_sz(), p.get_num_pt()) == (512, 512, 262144)
    assert p.get_physical_storage_MB() * 1024 * 1024 == 4294967296
    p = PirParams.preset("db2097152")
    assert (p.get_fst_dim_sz(), p.get_other_dim_sz()) == (1024, 2048)
    assert len(p.get_dims()) == 12 and p.get_expan_height() == 11
    # the active preset of database_constants.h:215-223
    p = PirParams.preset("quick_test_256MB")
    assert p.get_dims() == [256] + [2] * 8


def test_entry_too_large_rejected():
    from onionpirv2_gb300 import PirParams
    with pytest.raises(ValueError):
        PirParams(num_entries=16, max_fst_dim=4, entry_size_cfg=10**6)


def test_synthetic_entries_match_oracle(oracle_lib):
    from onionpirv2_gb300 import synthetic_entries
    o = oracle_lib.Oracle(4096, 256)
    for first, count in ((0, 3), (4000, 5)):
        assert np.array_equal(synthetic_entries(77, first, count, o.P.entry_size),
                              o.gen_entries(77, first, count))
    e = synthetic_entries(5, 0x0102030405060708, 1, 3840)[0]
    assert list(e[:8]) == [1, 2, 3, 4, 5, 6, 7, 8]
