"""GB300-native Cassandra molecular-energy hot path.

The product is libcassgpu.so (CUDA, sm_103a) behind the C-ABI of
include/cassandra_gb300.h.  This package loads it, mirrors the reference's
data model (species, boxes, molecules) and drives it.  There is no CPU
fallback: if the library cannot be loaded, every call raises.
"""
from __future__ import annotations

import ctypes
import os

from . import abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libcassgpu.so")
_LIB = None
_FNS = None


def load_library() -> ctypes.CDLL:
    """dlopen libcassgpu.so (built by cassandra_gb300.build); raises if absent."""
    global _LIB, _FNS
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with `python -m cassandra_gb300.build`")
        _LIB = ctypes.CDLL(LIB_PATH)
        _FNS = abi.bind(_LIB, "cass_")
    return _LIB


def functions() -> dict:
    load_library()
    return _FNS


def open_system(system, precision: int = abi.PREC_MIXED, device: int = 0, max_kvectors: int = 100000) -> abi.Context:
    """Create a GPU context loaded with `system` (cassandra_gb300.system.System)."""
    return system.open(functions(), precision=precision, device=device, max_kvectors=max_kvectors)


def open_trajectory(xyz_path: str, h_path: str | None, natoms, nmols=None, box=None) -> abi.Trajectory:
    """Open a pregenerated trajectory (.xyz and, optionally, .H) for cass_load_next_frame."""
    return abi.Trajectory(functions(), xyz_path, h_path, natoms, nmols, box)


def header_functions() -> list:
    """Names of the entry points declared in include/cassandra_gb300.h."""
    import re
    hdr = os.path.join(HERE, "..", "include", "cassandra_gb300.h")
    with open(hdr) as f:
        text = f.read()
    return sorted(set(re.findall(r"^(?:int|const char\*)\s+(cass_\w+)\s*\(", text, re.M)))
