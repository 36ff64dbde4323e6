"""The C-ABI library builds for sm_103a, loads, and exports every entry point
declared in include/cassandra_gb300.h (no GPU needed: nothing is computed)."""
import ctypes

import cassandra_gb300 as cg
from cassandra_gb300 import abi, build


def test_library_exports_header():
    build.build()
    lib = cg.load_library()
    names = cg.header_functions()
    assert len(names) >= 17
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert lib.cass_abi_version() == 2


def test_bindings_cover_header():
    names = {n[len("cass_"):] for n in cg.header_functions()}
    assert names == set(abi.SIGNATURES)


def test_struct_layouts():
    assert ctypes.sizeof(abi.CassEnergy) == 14 * 8
    assert ctypes.sizeof(abi.CassWidomResult) == 40
    assert ctypes.sizeof(abi.CassWidomTrace) == 48
    assert ctypes.sizeof(abi.CassMCParams) == 8 + 2 * 4 + 2 * 8
    assert ctypes.sizeof(abi.CassMCResult) == 14 * 8 + 5 * 8
    assert ctypes.sizeof(abi.CassStats) == 2 * 8 + 5 * 8 + 4 * 4 + 8 + 8 + 2 * 4
    assert ctypes.sizeof(abi.CassBoxDesc) == 3 * 8 + 2 * 4 + 6 * 8 + 2 * 4 + 3 * 8
    assert ctypes.sizeof(abi.CassFrame) == 4 + 4 + 8 + 9 * 8 + 8 + 8 + 4 + 4


def test_errors_are_status_codes_without_a_device():
    """With no usable GPU, ctx_create returns a status (never aborts)."""
    import torch
    if torch.cuda.is_available():
        return
    fns = cg.functions()
    cfg = abi.CassConfig(1, 1, 1, abi.PREC_MIXED, 0, 100, None)
    h = ctypes.c_void_p()
    rc = fns["ctx_create"](ctypes.byref(cfg), ctypes.byref(h))
    assert rc in (abi.CASS_EINVAL, abi.CASS_ECUDA)
    assert fns["last_error"]()
    rc = fns["mol_inter_energy"](None, 1, 1, 0, None, None, None)
    assert rc == abi.CASS_EINVAL
