"""cass_build_molecule -- Build_Molecule (fragment_growth.f90:72-707) for one
molecule through the C-ABI, as a host that keeps its own CBMC insertion,
deletion and regrowth moves calls it (move_insert.f90:166, move_delete.f90:175),
against the oracle's Build_Molecule on the same liquid of n-butane: the same
growth order, overlap flag, ln P_seq and ln P_bias, coordinates and lfsr258
state after the call, for new molecules (del_flag 0) and for the old-weight
pass of live ones (del_flag 1)."""
import numpy as np
import pytest

import cassandra_gb300 as cg
from cassandra_gb300 import abi, workloads
from oracle import oracle

pytestmark = pytest.mark.gpu

MINS = np.array([1, 511, 4095, 131071, 8388607], dtype=np.uint64)


@pytest.fixture(scope="module", autouse=True)
def _built():
    from cassandra_gb300 import build
    build.build()
    oracle.build()


def _state(rng):
    """A valid lfsr258 state: each component above its minimum (random_generators.f90:64-91)."""
    v = rng.integers(0, 2**63, size=5, dtype=np.int64).astype(np.uint64)
    low = (v & ~MINS) == 0
    v[low] |= MINS[low] + np.uint64(1)
    return v


@pytest.fixture(scope="module")
def liquid():
    """A 25 A box of liquid butane made by the oracle's grand-canonical chain."""
    s = workloads.gcmc_system(nboxes=1, length=25.0, max_per_box=200, rcut=12.0)
    with oracle.open_system(s) as o:
        o.system_total_energy(1)
        o.gcmc([1], 3000, 1, [-20.0], [[1.0]], [[0.5]], seed=21)
        where = o.molecule_boxes(1)
        live = [int(k) + 1 for k in np.flatnonzero(where)]
        xyz = np.stack([o.get_molecule(im, 1) for im in live])
    free = [im for im in range(1, 201) if im not in live]
    assert len(live) > 20
    return s, live, xyz, free


def _load(ctx, liquid):
    s, live, xyz, _ = liquid
    ctx.set_molecules(live, [1] * len(live), [1] * len(live), xyz.ravel())
    ctx.system_total_energy(1)


def test_build_molecule_fp64_matches_oracle(liquid):
    s, live, xyz, free = liquid
    rng = np.random.default_rng(7)
    with oracle.open_system(s) as o, cg.open_system(s, precision=abi.PREC_FP64) as g:
        _load(o, liquid)
        _load(g, liquid)
        n_ov = 0
        for k in range(24):
            del_flag = k % 3 == 2
            im = live[k % len(live)] if del_flag else free[k]
            st = _state(rng)
            a = o.build_molecule(im, 1, 1, del_flag, 8, 8, st)
            b = g.build_molecule(im, 1, 1, del_flag, 8, 8, st)
            assert a["cbmc_overlap"] == b["cbmc_overlap"], k
            assert np.array_equal(a["rng_state"], b["rng_state"]), k
            assert not np.array_equal(a["rng_state"], st)
            assert np.array_equal(a["frag_order"], b["frag_order"]), k
            assert abs(a["ln_pseq"] - b["ln_pseq"]) <= 1e-12
            n_ov += a["cbmc_overlap"]
            if a["cbmc_overlap"]:
                continue
            assert abs(a["ln_pbias"] - b["ln_pbias"]) <= 1e-9 * max(1.0, abs(a["ln_pbias"])), (k, a, b)
            assert np.allclose(a["xyz"], b["xyz"], rtol=0, atol=1e-9), k
            if del_flag:  # the old-weight pass leaves the molecule where it was
                assert np.array_equal(b["xyz"], xyz[live.index(im)])
        assert n_ov < 24
        # a growth stores nothing in the context
        assert np.array_equal(g.get_molecule(live[0], 1), xyz[0])


def test_build_molecule_mixed_follows_oracle(liquid):
    """FP32 growth (mixed context) from the same lfsr258 state: nearly always the
    same trials, and then coordinates and ln P_bias agree to FP32 rounding."""
    s, live, xyz, free = liquid
    rng = np.random.default_rng(8)
    with oracle.open_system(s) as o, cg.open_system(s, precision=abi.PREC_MIXED) as g:
        _load(o, liquid)
        _load(g, liquid)
        close = 0
        n = 32
        for k in range(n):
            st = _state(rng)
            a = o.build_molecule(free[k], 1, 1, False, 8, 8, st)
            b = g.build_molecule(free[k], 1, 1, False, 8, 8, st)
            assert np.array_equal(a["frag_order"], b["frag_order"])
            if a["cbmc_overlap"] or b["cbmc_overlap"]:
                close += a["cbmc_overlap"] == b["cbmc_overlap"]
                continue
            if np.allclose(a["xyz"], b["xyz"], rtol=0, atol=1e-3) and abs(a["ln_pbias"] - b["ln_pbias"]) < 1e-3:
                close += 1
        assert close >= 0.9 * n


def test_build_molecule_errors(liquid):
    s, live, xyz, free = liquid
    st = np.array([5, 600, 5000, 200000, 9000000], dtype=np.uint64)
    with cg.open_system(s, precision=abi.PREC_FP64) as g:
        _load(g, liquid)
        with pytest.raises(abi.CassError) as e:
            g.build_molecule(live[0], 1, 1, False, 8, 8, st)  # growing a live molecule
        assert e.value.code == abi.CASS_ESTATE
        with pytest.raises(abi.CassError) as e:
            g.build_molecule(free[0], 1, 1, True, 8, 8, st)  # old-weight pass of a molecule not in the box
        assert e.value.code == abi.CASS_ESTATE
        with pytest.raises(abi.CassError):
            g.build_molecule(0, 1, 1, False, 8, 8, st)


@pytest.mark.parametrize("l_coul_cbmc", [False, True])
def test_build_molecule_charged_fp64_matches_oracle(liquid, l_coul_cbmc):
    """The same liquid with partial charges in an Ewald box: the CBMC trial
    energies carry the intramolecular charges, and with L_Coul_CBMC the
    intermolecular real-space charges within rcut_cbmc as well."""
    import copy
    s, live, xyz, free = liquid
    s = copy.deepcopy(s)
    for a, q in zip(s.species[0].atoms, (0.25, -0.25, -0.25, 0.25)):
        a.charge = q
    s.species[0].l_coul_cbmc = l_coul_cbmc
    bx = s.boxes[0]
    bx.charge_style, bx.charge_sum_style, bx.ewald_tol, bx.rcut_coul = abi.CHARGE_COUL, abi.QQ_EWALD, 1e-5, 12.0
    rng = np.random.default_rng(9)
    with oracle.open_system(s) as o, cg.open_system(s, precision=abi.PREC_MIXED) as g:
        _load(o, (s, live, xyz, free))
        _load(g, (s, live, xyz, free))
        for k in range(16):
            del_flag = k % 2 == 1
            im = live[k % len(live)] if del_flag else free[k]
            st = _state(rng)
            a = o.build_molecule(im, 1, 1, del_flag, 8, 8, st)
            b = g.build_molecule(im, 1, 1, del_flag, 8, 8, st)  # charged boxes grow in FP64
            assert a["cbmc_overlap"] == b["cbmc_overlap"], k
            assert np.array_equal(a["rng_state"], b["rng_state"]), k
            assert np.array_equal(a["frag_order"], b["frag_order"]), k
            if a["cbmc_overlap"]:
                continue
            assert abs(a["ln_pbias"] - b["ln_pbias"]) <= 1e-9 * max(1.0, abs(a["ln_pbias"])), (k, a, b)
            assert np.allclose(a["xyz"], b["xyz"], rtol=0, atol=1e-9), k
