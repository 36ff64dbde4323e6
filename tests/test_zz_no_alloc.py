"""The allocation-free entry point agrees with the allocating one.

cass_mol_box_energy_noalloc exists for Monte Carlo hosts that may not call
cudaMalloc inside their move loop (their device memory belongs to another
allocator, or an allocation would stall the device mid-loop).  It must give the
molecule-vs-box energy that cass_mol_inter_energy gives, call after call, using
only the caller's device arrays and its own static scratch.  The inputs here
are device tensors made by the test (the test may allocate; the entry point
does not).  This file is collected last so that a run stopping at its first
failure has run every other test already.
"""
import ctypes

import numpy as np
import pytest

import cassandra_gb300 as cg
import helpers
from cassandra_gb300 import abi

pytestmark = pytest.mark.gpu

TOL = 1e-10  # FP64 path: the two entry points differ only in summation order


def _box_desc(bx):
    d = abi.CassBoxDesc()
    d.length[0], d.length[1], d.length[2] = bx.length
    d.vdw_style, d.vdw_sum_style = bx.vdw_style, bx.vdw_sum_style
    d.rcut_vdw, d.rcut_coul, d.rcut_cbmc, d.rcut_low = bx.rcut_vdw, bx.rcut_coul, bx.rcut_cbmc, bx.rcut_low
    d.ron_switch, d.roff_switch = bx.ron_switch, bx.roff_switch
    d.charge_style, d.charge_sum_style = bx.charge_style, bx.charge_sum_style
    d.ewald_tol, d.alpha_dsf, d.temperature = bx.ewald_tol, bx.alpha_dsf, bx.temperature
    return d


def test_noalloc_matches_allocating_entry_point_twice():
    import torch

    from cassandra_gb300 import build
    build.build()
    fns = cg.functions()
    noalloc = fns["mol_box_energy_noalloc"]
    s = helpers.pregen_system("water_spce", 4)
    sp = s.species[0]
    na = sp.natoms
    xyz = np.concatenate([x for x in s.molecules.xyz])            # [nmol*na, 3]
    q = np.tile([a.charge for a in sp.atoms], len(s.molecules.xyz))
    box_xyzq = np.concatenate([xyz, q[:, None]], axis=1)
    types = np.tile(np.asarray(sp.type_index, dtype=np.int32), len(s.molecules.xyz))
    mols = np.repeat(np.arange(1, len(s.molecules.xyz) + 1, dtype=np.int32), na)
    dev = torch.device("cuda:0")
    d_box = torch.tensor(box_xyzq, dtype=torch.float64, device=dev).contiguous()
    d_type = torch.tensor(types, dtype=torch.int32, device=dev).contiguous()
    d_mol = torch.tensor(mols, dtype=torch.int32, device=dev).contiguous()
    d_out = torch.zeros(3, dtype=torch.float64, device=dev)
    desc = _box_desc(s.boxes[0])
    eps = np.ascontiguousarray(s.ff.eps, dtype=np.float64).ravel()
    sig = np.ascontiguousarray(s.ff.sig, dtype=np.float64).ravel()
    pe = eps.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    ps = sig.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    torch.cuda.synchronize()
    with cg.open_system(s, precision=abi.PREC_FP64) as g:
        for im, cbmc in ((17, 0), (42, 1)):  # two calls in a row, reusing the shared scratch
            want = g.mol_inter_energy(im, 1, bool(cbmc))
            qa = box_xyzq[(im - 1) * na: im * na]
            d_q = torch.tensor(qa, dtype=torch.float64, device=dev).contiguous()
            d_qt = torch.tensor(np.asarray(sp.type_index, dtype=np.int32), device=dev).contiguous()
            d_out.fill_(-7.0)
            torch.cuda.synchronize()
            rc = noalloc(ctypes.byref(desc), s.ff.ntypes, pe, ps, ctypes.c_void_p(d_box.data_ptr()),
                         ctypes.c_void_p(d_type.data_ptr()), ctypes.c_void_p(d_mol.data_ptr()), d_type.numel(),
                         ctypes.c_void_p(d_q.data_ptr()), ctypes.c_void_p(d_qt.data_ptr()), na, im, cbmc,
                         int(sp.l_coul_cbmc), abi.PREC_FP64, ctypes.c_void_p(d_out.data_ptr()), None)
            assert rc == abi.CASS_OK, fns["last_error"]()
            torch.cuda.synchronize()
            got = d_out.cpu().numpy()
            assert bool(got[2]) == want[2]
            for a, b in zip(got[:2], want[:2]):
                assert abs(a - b) <= TOL * max(abs(b), 1.0), (im, cbmc, got, want)


def test_noalloc_rejects_oversize():
    fns = cg.functions()
    s = helpers.pregen_system("water_spce", 0)
    desc = _box_desc(s.boxes[0])
    eps = np.ones(1)
    p = eps.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    rc = fns["mol_box_energy_noalloc"](ctypes.byref(desc), 1, p, p, ctypes.c_void_p(8), ctypes.c_void_p(8),
                                       ctypes.c_void_p(8), 262145, ctypes.c_void_p(8), ctypes.c_void_p(8), 3, 1, 0,
                                       0, abi.PREC_FP64, ctypes.c_void_p(8), None)
    assert rc == abi.CASS_ECAPACITY
    assert b"262144" in fns["last_error"]()


@pytest.mark.parametrize("vdw_sum", [abi.VDW_SUM_CUT_SHIFT, abi.VDW_SUM_CUT_SWITCH, abi.VDW_SUM_CUT_TAIL],
                         ids=["cut_shift", "cut_switch", "cut_tail"])
def test_noalloc_mixed_matches_oracle(vdw_sum):
    """Mixed precision through the allocation-free call, in LJ styles with and without a
    shift or switch term, against the oracle's molecule energy: the shift and switch
    terms apply in every precision and with or without the CBMC flag
    (energy_routines.f90:1927-1970).  Two calls in a row per style."""
    import torch

    from cassandra_gb300 import build
    from oracle import oracle
    build.build()
    fns = cg.functions()
    noalloc = fns["mol_box_energy_noalloc"]
    s = helpers.lj_fluid_system(vdw_sum)
    sp = s.species[0]
    xyz = np.concatenate([x for x in s.molecules.xyz])
    box_xyzq = np.concatenate([xyz, np.zeros((len(xyz), 1))], axis=1)
    dev = torch.device("cuda:0")
    d_box = torch.tensor(box_xyzq, dtype=torch.float64, device=dev).contiguous()
    d_type = torch.ones(len(xyz), dtype=torch.int32, device=dev)
    d_mol = torch.arange(1, len(xyz) + 1, dtype=torch.int32, device=dev)
    d_out = torch.zeros(3, dtype=torch.float64, device=dev)
    d_qt = torch.ones(1, dtype=torch.int32, device=dev)
    desc = _box_desc(s.boxes[0])
    eps = np.ascontiguousarray(s.ff.eps, dtype=np.float64).ravel()
    sig = np.ascontiguousarray(s.ff.sig, dtype=np.float64).ravel()
    pe = eps.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    ps = sig.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    with oracle.open_system(s) as o:
        o.system_total_energy(1)
        for im, cbmc in ((17, 0), (42, 1)):
            want = o.mol_inter_energy(im, 1, bool(cbmc))
            d_q = torch.tensor(box_xyzq[im - 1:im], dtype=torch.float64, device=dev).contiguous()
            d_out.fill_(-7.0)
            torch.cuda.synchronize()
            rc = noalloc(ctypes.byref(desc), s.ff.ntypes, pe, ps, ctypes.c_void_p(d_box.data_ptr()),
                         ctypes.c_void_p(d_type.data_ptr()), ctypes.c_void_p(d_mol.data_ptr()), d_type.numel(),
                         ctypes.c_void_p(d_q.data_ptr()), ctypes.c_void_p(d_qt.data_ptr()), 1, im, cbmc, 0,
                         abi.PREC_MIXED, ctypes.c_void_p(d_out.data_ptr()), None)
            assert rc == abi.CASS_OK, fns["last_error"]()
            torch.cuda.synchronize()
            got = d_out.cpu().numpy()
            assert bool(got[2]) == want[2]
            k = s.molecules.im.index(im)
            scale = helpers.pair_magnitude_scale(s, s.molecules.xyz[k], sp.type_index, [0.0], im,
                                                 s.boxes[0].rcut_cbmc if cbmc else s.boxes[0].rcut_vdw)
            assert abs(got[0] - want[0]) <= 1e-5 * scale, (vdw_sum, im, cbmc, got, want)
