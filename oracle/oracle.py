"""Loader for the CPU FP64 oracle (test infrastructure only).

Imported by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg,
never by the product package.  The oracle implements the entry points of
include/cassandra_gb300.h under the ``orc_`` prefix, so the same
cassandra_gb300.abi.Context drives it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from cassandra_gb300 import abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liborc.so")
_lib = None
_fns = None


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "cass_oracle.cpp")
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(src):
        subprocess.check_call(["make", "-s", "-C", HERE, "liborc.so"])
    return LIB


def lib() -> C.CDLL:
    global _lib, _fns
    if _lib is None:
        build()
        _lib = C.CDLL(LIB)
        _fns = abi.bind(_lib, "orc_")
        _lib.orc_rng_stream.argtypes = [C.c_uint64, C.c_int64, C.c_int64, C.c_int32, C.POINTER(C.c_double)]
        _lib.orc_rng_reference.argtypes = [C.c_int64, C.c_int64, C.c_int32, C.POINTER(C.c_double)]
        _lib.orc_num_threads.restype = C.c_int
        _lib.orc_set_num_threads.restype = C.c_int
        _lib.orc_set_num_threads.argtypes = [C.c_int]
    return _lib


def fns() -> dict:
    lib()
    return _fns


def open_system(system, max_kvectors: int = 100000) -> abi.Context:
    """Open an oracle context loaded with `system` (a cassandra_gb300.system.System)."""
    return system.open(fns(), precision=abi.PREC_FP64, max_kvectors=max_kvectors)


def rng_stream(seed: int, ibox: int, ins: int, n: int) -> np.ndarray:
    out = np.zeros(n)
    lib().orc_rng_stream(C.c_uint64(seed & (2**64 - 1)), ibox, ins, n, out.ctypes.data_as(C.POINTER(C.c_double)))
    return out


def rng_reference(i1: int, i3: int, n: int) -> np.ndarray:
    out = np.zeros(n)
    lib().orc_rng_reference(i1, i3, n, out.ctypes.data_as(C.POINTER(C.c_double)))
    return out


def num_threads() -> int:
    return int(lib().orc_num_threads())


def set_num_threads(n: int) -> int:
    """OpenMP threads of the oracle's parallel loops (n < 1: every host processor)."""
    return int(lib().orc_set_num_threads(int(n)))
