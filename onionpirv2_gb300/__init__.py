"""onionpirv2_gb300 -- GB300-native (sm_103a) OnionPIRv2 server query path.

The CUDA library (``_build/libopir_gb300.so``, C ABI in
``include/onionpir_gpu.h``) runs query expansion, RGSW reconstruction, the
first-dimension database scan, RGSW folding, modulus switching and response
packing.  This package mirrors the reference's PirParams / PirServer
interface on top of it, and its PirClient (CPU, ``_build/libopir_client.so``,
C ABI in ``include/onionpir_client.h``).
"""
from .params import PirParams, PRESETS, WORKLOADS  # noqa: F401
from .server import PirServer, synthetic_entries  # noqa: F401
from ._capi import OpirError, UnknownClientError  # noqa: F401
from .client import PirClient  # noqa: F401

__all__ = ["PirParams", "PirServer", "PirClient", "PRESETS", "WORKLOADS", "OpirError", "UnknownClientError",
           "synthetic_entries"]
