"""The CPU oracle's grand-canonical chains (move_insert.f90, move_delete.f90,
move_regrow.f90): energy bookkeeping against a recomputed system energy, and
the ideal-chain limit <N> = V exp(beta mu) <W> / Lambda^3 with <W> from Widom
insertions of the same oracle."""
import math

import numpy as np
import pytest

from cassandra_gb300 import abi, workloads
from oracle import oracle

KBOLTZ = 0.8314472
H_PLANK = 39.9031268605


def test_gcmc_bookkeeping_all_moves():
    s = workloads.gcmc_system(nboxes=2, length=25.0, max_per_box=300)
    with oracle.open_system(s) as o:
        for b in (1, 2):
            o.system_total_energy(b)
        r = o.gcmc([1, 2], 3000, 1, [-22.0, -26.0], [[1.0], [1.0]], [[0.5], [0.5]], seed=3)
        where = o.molecule_boxes(1)
        assert where.shape == (600,)
        for k, x in enumerate(r):
            assert int((where == k + 1).sum()) == x["n_molecules"]
            for kind in ("translate", "rotate", "insert", "delete", "regrow"):
                assert x[f"n_{kind}"] > 0
            assert x["n_insert_accepted"] > 0 and x["n_regrow_accepted"] > 0
            e, ov = o.system_total_energy(k + 1)
            assert not ov
            for comp in ("total", "inter_vdw", "angle", "dihedral", "lrc"):
                assert abs(x["energy"][comp] - e[comp]) <= 1e-9 * (abs(e["inter_vdw"]) + 1.0), comp


def test_gcmc_ewald_bookkeeping():
    """Water in Ewald boxes: insertions and deletions change the reciprocal sum
    by the molecule's structure factor and the self energy by the molecule's
    (move_insert.f90:274-291, move_delete.f90:261-277); the chain's running
    energy equals a recomputation of its final state in every component."""
    s = workloads.water_gcmc_system(nboxes=2)
    with oracle.open_system(s) as o:
        for b in (1, 2):
            o.system_total_energy(b)
        r = o.gcmc([1, 2], 4000, 1, [-30.0, -34.0], [[0.5], [0.5]], [[0.4], [0.4]], seed=7, kappa_ins=8,
                   kappa_dih=0, cuts=(0.2, 0.4, 0.7, 1.0, 1.0))
        for k, x in enumerate(r):
            assert x["n_insert_accepted"] > 0 and x["n_delete_accepted"] > 0, x
            e, ov = o.system_total_energy(k + 1)
            assert not ov
            scale = abs(e["inter_vdw"]) + abs(e["inter_q"]) + abs(e["reciprocal"]) + abs(e["self"])
            for comp in ("total", "inter_vdw", "inter_q", "intra_q", "reciprocal", "self"):
                assert abs(x["energy"][comp] - e[comp]) <= 1e-9 * scale, (comp, x["energy"][comp], e[comp])


def test_gcmc_ideal_chain_matches_widom():
    s = workloads.gcmc_system(nboxes=2, length=30.0, max_per_box=400, eps_scale=0.0, rcut_low=1e-3)
    T = s.boxes[0].temperature
    beta = 1.0 / (KBOLTZ * T)
    mw = sum(a.mass for a in s.species[0].atoms)
    lam = H_PLANK * math.sqrt(beta / (2 * math.pi * mw))
    V = s.boxes[0].volume
    with oracle.open_system(s) as o:
        for b in (1, 2):
            o.system_total_energy(b)
        _, tr = o.widom_insert(1, [1, 2], 20000, 12, 12, seed=5, trace=True)
        w = tr["widom_var"].mean()
        target = 20.0
        mu = math.log(target * lam ** 3 / (V * w)) / beta * 0.01
        r = o.gcmc([1, 2], 100000, 1, [mu, mu], [[1.0], [1.0]], [[0.5], [0.5]], seed=3,
                   cuts=(0.0, 0.0, 0.5, 1.0, 1.0))
    mean_n = np.mean([x["sum_n_molecules"] / 100000 for x in r])
    assert abs(mean_n - target) < 0.5, mean_n


def test_gcmc_deterministic():
    s = workloads.gcmc_system(nboxes=1, length=25.0, max_per_box=200)
    out = []
    for _ in range(2):
        with oracle.open_system(s) as o:
            o.system_total_energy(1)
            out.append(o.gcmc([1], 500, 1, [-24.0], [[1.0]], [[0.5]], seed=9))
    assert out[0] == out[1]


def test_gcmc_charged_butane_bookkeeping():
    """Partially charged butane in Ewald boxes, with and without L_Coul_CBMC:
    insertions, deletions and regrowths (the reciprocal sum of a regrown
    molecule, move_regrow.f90:338-354) keep the running energy equal to a
    recomputation in every component."""
    s = workloads.gcmc_system(nboxes=2, length=25.0, max_per_box=300, rcut=12.0)
    for a, q in zip(s.species[0].atoms, (0.25, -0.25, -0.25, 0.25)):
        a.charge = q
    for bx in s.boxes:
        bx.charge_style, bx.charge_sum_style, bx.ewald_tol, bx.rcut_coul = abi.CHARGE_COUL, abi.QQ_EWALD, 1e-5, 12.0
    for l_coul_cbmc in (False, True):
        s.species[0].l_coul_cbmc = l_coul_cbmc
        with oracle.open_system(s) as o:
            for b in (1, 2):
                o.system_total_energy(b)
            r = o.gcmc([1, 2], 600, 1, [-22.0, -26.0], [[1.0], [1.0]], [[0.5], [0.5]], seed=5)
            for k, x in enumerate(r):
                assert x["n_insert_accepted"] > 0 and x["n_regrow_accepted"] > 0, x
                e, ov = o.system_total_energy(k + 1)
                assert not ov
                scale = abs(e["inter_vdw"]) + abs(e["inter_q"]) + abs(e["reciprocal"]) + abs(e["self"])
                for comp in ("total", "inter_vdw", "inter_q", "intra_q", "reciprocal", "self", "dihedral"):
                    assert abs(x["energy"][comp] - e[comp]) <= 1e-9 * scale, (comp, x["energy"][comp], e[comp])


def test_gcmc_charges_need_ewald():
    """Grand-canonical moves and per-call growth in a charged box whose charges
    use another sum than Ewald are refused (CASS_EUNSUPPORTED), as the device
    path refuses them."""
    s = workloads.water_gcmc_system(nboxes=1)
    s.boxes[0].charge_sum_style = abi.QQ_DSF
    with oracle.open_system(s) as o:
        o.system_total_energy(1)
        with pytest.raises(abi.CassError) as e:
            o.gcmc([1], 10, 1, [-30.0], [[0.5]], [[0.4]], seed=1, kappa_ins=8, kappa_dih=0,
                   cuts=(0.2, 0.4, 0.7, 1.0, 1.0))
        assert e.value.code == abi.CASS_EUNSUPPORTED
        st = np.array([5, 600, 5000, 200000, 9000000], dtype=np.uint64)
        with pytest.raises(abi.CassError) as e:
            o.build_molecule(100, 1, 1, False, 8, 0, st)
        assert e.value.code == abi.CASS_EUNSUPPORTED
