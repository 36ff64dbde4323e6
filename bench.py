"""Benchmark: batched CBMC Widom insertion (trial energies/s) on GB300.

Workload: n-butane (4-site united atom, 2 CBMC fragments) inserted into 64
frozen LJ boxes of uneven size (N uniform in 200..4000, rho* = 0.6, sigma 3.73 A,
eps/k 148 K, 14 A cut_tail, rcut_cbmc 6.5 A, T 150 K) with kappa_ins = 12 and
kappa_dih = 12, i.e. 24 trial energies per insertion; one step = 10^6
insertions (15,625 per box) in one batched call.  Synthetic, seeded inputs.

value : trial energies/s of the mixed-precision path, device time (CUDA events
        around each step on the library's stream), inputs resident in HBM,
        L2 flushed between steps.
e2e   : the same metric through the public API with host buffers: upload the
        frame, system energies of every box, Widom batch, results back.
Also reported: the plain-FP64 GPU path on the same workload, the roofline of
the Widom kernel, and the CPU FP64 oracle (OpenMP, all host cores) on a
bounded sample; NVT MC sweeps/s (500 LJ spheres, 256 waters), grand-canonical
butane moves/s in 16 boxes with densities against FP64 reruns, and the
configuration gradient of 4096 waters.  `--impl reference` times the CPU restatement of the
reference's algorithm (the reference itself is Fortran and cannot be built
here) on the same workload.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "CBMC/Widom trial energies/s and MC sweeps/s vs plain FP64 GPU at stated error"
WIDOM_PROFILE = "k_widom_f32_butane_16boxes.md"
UNIT = "trial energies/s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--boxes", type=int, default=64)
    p.add_argument("--insertions", type=int, default=1_000_000, help="insertions per step, all boxes")
    p.add_argument("--kappa", type=int, default=12)
    p.add_argument("--seed", type=int, default=2024)
    p.add_argument("--fp64-steps", type=int, default=2)
    p.add_argument("--cpu-seconds", type=float, default=15.0, help="target CPU-baseline sample length")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-mc", action="store_true", help="skip the MC-sweep leg")
    p.add_argument("--no-grad", action="store_true", help="skip the configuration-gradient leg")
    p.add_argument("--no-gcmc", action="store_true", help="skip the grand-canonical leg")
    p.add_argument("--no-npt", action="store_true", help="skip the NPT / fluctuation-formula leg")
    p.add_argument("--no-pregen", action="store_true", help="skip the trajectory-fed Widom leg")
    p.add_argument("--gcmc-eq-steps", type=int, default=150000)
    p.add_argument("--gcmc-blocks", type=int, default=8)
    p.add_argument("--gcmc-block-steps", type=int, default=15000)
    p.add_argument("--pregen-frames", type=int, default=4)
    p.add_argument("--npt-chains", type=int, default=64)
    p.add_argument("--npt-eq-blocks", type=int, default=300)
    p.add_argument("--npt-blocks", type=int, default=32, help="production blocks (configurations per chain)")
    p.add_argument("--profile-case", choices=["mixed", "fp64", "mc"], default=None,
                   help="only the small case a kernel profile uses: the Widom kernel on 16 of the benchmark boxes, "
                        "16,000 (mixed) or 4,096 (FP64) insertions per box, fixed cell edge, three launches; or (mc) "
                        "single MC chains: FP64 water-256 (warm-up and 2 sweeps), then mixed LJ-500 (warm-up and 20 "
                        "sweeps)")
    return p.parse_args()


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def build_workload(args, rank):
    """Rank r's shard of the job: its own `args.boxes` boxes (seed offset by the rank),
    so that the per-rank work stays fixed as ranks are added (weak scaling)."""
    from cassandra_gb300 import workloads
    return workloads.widom_batch_system(nboxes=args.boxes, seed=args.seed + 1000 * rank, nconfig=1000)


def cpu_baseline(system, args, per_box_cap=None, threads=0, seconds=None):
    """CPU FP64 oracle (restatement of the reference's Widom loop), OpenMP over
    insertions on `threads` host threads (0: all)."""
    from oracle import oracle
    boxes = list(range(1, len(system.boxes) + 1))
    secs = args.cpu_seconds if seconds is None else seconds
    nthr = oracle.set_num_threads(threads)
    try:
        with oracle.open_system(system) as o:
            for b in boxes:
                o.system_total_energy(b)
            # calibrate on a small sample, then size the run to ~secs
            t0 = time.perf_counter()
            o.widom_insert(2, boxes, 8 if nthr > 1 else 1, args.kappa, args.kappa, seed=1)
            dt = max(time.perf_counter() - t0, 1e-3)
            per = dt / ((8 if nthr > 1 else 1) * len(boxes))
            n = max(1, int(secs / (per * len(boxes))))
            if per_box_cap:
                n = min(n, per_box_cap)
            t0 = time.perf_counter()
            res = o.widom_insert(2, boxes, n, args.kappa, args.kappa, seed=99)
            dt = time.perf_counter() - t0
    finally:
        oracle.set_num_threads(0)
    trials = sum(r["n_trials"] for r in res)
    return {"value": trials / dt, "unit": UNIT, "cores": nthr, "kind": "port",
            "sample": f"{len(boxes)} boxes x {n} insertions ({trials} trial energies) in {dt:.2f} s, "
                      f"FP64 C++ oracle, OpenMP over insertions, {nthr} thread(s)"}


def mc_leg(cg, abi, dev, with_cpu: bool) -> dict:
    """NVT MC sweeps/s: the 500-sphere LJ box (translation) and the 256-water
    Ewald box (translate/rotate 50/50), one chain and many independent chains."""
    from cassandra_gb300 import workloads

    def chains(system, boxes, nsweeps, precision, prob_translate, recompute=False):
        ns = len(system.species)
        with cg.open_system(system, precision=precision, device=dev) as g:
            for b in boxes:
                g.system_total_energy(b)
            md, mr = [[0.8] * ns] * len(boxes), [[0.4] * ns] * len(boxes)
            g.mc_sweeps(boxes, 1, md, mr, seed=1, prob_translate=prob_translate)  # warm-up
            res, _, _ = g.mc_sweeps(boxes, nsweeps, md, mr, seed=2, prob_translate=prob_translate)
            st = g.stats()
            out = {"chains": len(boxes), "sweeps": nsweeps, "kernel_ms": st["mc_ms"],
                   "sweeps_per_s": nsweeps * len(boxes) / (st["mc_ms"] / 1e3),
                   "moves_per_s": st["mc_moves"] / (st["mc_ms"] / 1e3),
                   "acceptance": sum(r["n_translate_accepted"] + r["n_rotate_accepted"] for r in res) /
                   max(1, sum(r["n_translate"] + r["n_rotate"] for r in res))}
            if recompute:  # the running FP64 bookkeeping against an FP64 recomputation of the final frame
                m = system.molecules
                xyz = np.concatenate([g.get_molecule(im, is_).ravel() for im, is_ in zip(m.im, m.is_)])
                with cg.open_system(system, precision=abi.PREC_FP64, device=dev) as f:
                    f.set_molecules(m.im, m.is_, m.ibox, xyz)
                    e, _ = f.system_total_energy(boxes[0])
                scale = abs(e["inter_vdw"]) + abs(e["inter_q"]) + abs(e["reciprocal"])
                out["bookkeeping_rel_err"] = abs(res[0]["energy"]["total"] - e["total"]) / scale
            return out

    def cpu(system, nsweeps, prob_translate):
        from oracle import oracle
        ns = len(system.species)
        with oracle.open_system(system) as o:
            o.system_total_energy(1)
            t0 = time.perf_counter()
            o.mc_sweeps([1], nsweeps, [[0.8] * ns], [[0.4] * ns], seed=2, prob_translate=prob_translate)
            dt = time.perf_counter() - t0
        return {"sweeps_per_s": nsweeps / dt, "cores": 1, "kind": "port",
                "sample": f"{nsweeps} sweeps of one chain, FP64 C++ oracle, one thread"}

    out = {}
    c0 = workloads.lj_nvt_system(nboxes=1)
    c0r = workloads.lj_nvt_system(nboxes=304, seed=7)
    out["lj500_translate"] = {
        "workload": "500 LJ spheres, sigma 3.73 A, eps/k 148 K, 35 A box, T 150 K, 14 A cut_tail, translation",
        "mixed_1chain": chains(c0, [1], 100, abi.PREC_MIXED, 1.0, recompute=True),
        "fp64_1chain": chains(c0, [1], 20, abi.PREC_FP64, 1.0),
        "mixed_304chains": chains(c0r, list(range(1, 305)), 20, abi.PREC_MIXED, 1.0),
        "fp64_304chains": chains(c0r, list(range(1, 305)), 2, abi.PREC_FP64, 1.0)}
    c1 = workloads.water_nvt_system(nboxes=1)
    c1r = workloads.water_nvt_system(nboxes=152, seed=5)
    out["water256_translate_rotate"] = {
        "workload": "256 rigid 3-site waters, 19.7 A box, T 298 K, 9.8 A LJ + Ewald real space, tol 1e-5 "
                    "(959 k-vectors), translate/rotate 50/50",
        "mixed_1chain": chains(c1, [1], 20, abi.PREC_MIXED, 0.5, recompute=True),
        "fp64_1chain": chains(c1, [1], 2, abi.PREC_FP64, 0.5),
        "mixed_152chains": chains(c1r, list(range(1, 153)), 4, abi.PREC_MIXED, 0.5)}
    if with_cpu:
        out["lj500_translate"]["cpu_baseline"] = cpu(c0, 20, 1.0)
        out["water256_translate_rotate"]["cpu_baseline"] = cpu(c1, 4, 0.5)
    return out


BUTANE_MW = 2 * 15.035 + 2 * 14.027  # g/mol, united-atom CH3-CH2-CH2-CH3
AVOGADRO = 6.02214076e23


def blocking_se(x):
    """Standard error of the mean of the rows of x [samples, series] with pairwise
    blocking: the largest standard error over the levels that keep 4 or more blocks."""
    y = np.asarray(x, dtype=np.float64)
    best = np.zeros(y.shape[1])
    while len(y) >= 4:
        best = np.maximum(best, y.std(axis=0, ddof=1) / np.sqrt(len(y)))
        m = len(y) // 2 * 2
        y = 0.5 * (y[0:m:2] + y[1:m:2])
    return best


def gcmc_leg(cg, abi, dev, with_cpu: bool, eq_steps: int = 150000, blocks: int = 8,
             block_steps: int = 15000) -> dict:
    """Grand-canonical butane in 16 boxes of 40 A at 300 K, mu evenly spaced over
    [-30, -20] kJ/mol, insert/delete 40 %, translate/rotate 40 %, regrow 20 %.
    Each precision equilibrates from empty boxes, then runs `blocks` production
    calls whose per-call <N> are block averages; densities of the mixed chains are
    compared with FP64 reruns of the same boxes through those block errors."""
    from cassandra_gb300 import workloads

    nb = 16
    mu = list(np.linspace(-30.0, -20.0, nb))
    cuts = (0.2, 0.4, 0.6, 0.8, 1.0)

    def chains(precision, boxes_mu, eq, nblk, nstep, seed):
        n = len(boxes_mu)
        s = workloads.gcmc_system(nboxes=n, length=40.0, max_per_box=800)
        boxes = list(range(1, n + 1))
        md, mr = [[1.0]] * n, [[0.5]] * n
        g = cg.open_system(s, precision=precision, device=dev)
        for b in boxes:
            g.system_total_energy(b)
        g.gcmc(boxes, eq, 1, boxes_mu, md, mr, seed=seed, cuts=cuts)
        eq_ms = g.stats()["mc_ms"]
        cluster = g.stats()["gcmc_cluster"]
        means, ms, last = [], 0.0, None
        for k in range(nblk):
            last = g.gcmc(boxes, nstep, 1, boxes_mu, md, mr, seed=seed + 1 + k, cuts=cuts)
            ms += g.stats()["mc_ms"]
            means.append([r["sum_n_molecules"] / nstep for r in last])
        means = np.array(means)  # [sub-blocks, boxes]
        mean_n = means.mean(axis=0)
        se = blocking_se(means) if nblk > 1 else np.zeros(n)
        acc = {k: sum(r[f"n_{k}_accepted"] for r in last) / max(1, sum(r[f"n_{k}"] for r in last))
               for k in ("translate", "rotate", "insert", "delete", "regrow")}
        out = {"boxes": n, "ctas_per_box": cluster, "equilibration_steps": eq, "production_steps": nblk * nstep,
               "kernel_ms": ms, "moves_per_s": n * nblk * nstep / (ms / 1e3),
               "equilibration_moves_per_s": n * eq / (eq_ms / 1e3),
               "acceptance_last_block": acc, "mean_n": mean_n, "se_n": se}
        return out, g, s

    def density(n):
        return float(n * BUTANE_MW / AVOGADRO / (40.0 ** 3 * 1e-24))

    # production as many short sub-blocks, whose means are blocked pairwise until
    # few remain; the error of a box is the largest standard error over those
    # levels (Flyvbjerg and Petersen, J. Chem. Phys. 91, 461 (1989)), so the
    # correlation between successive sub-blocks is accounted for
    nsub = max(blocks, 64)
    sub_steps = max(1, blocks * block_steps // nsub)
    mixed, gm, sysm = chains(abi.PREC_MIXED, mu, eq_steps, nsub, sub_steps, seed=11)
    fp64, gf, _ = chains(abi.PREC_FP64, mu, eq_steps, nsub, sub_steps, seed=911)
    gf.close()
    z = (mixed["mean_n"] - fp64["mean_n"]) / np.sqrt(np.maximum(mixed["se_n"] ** 2 + fp64["se_n"] ** 2, 1e-12))
    from scipy import stats as _st
    pvals = 2.0 * _st.t.sf(np.abs(z), 3)
    dn = mixed["mean_n"] - fp64["mean_n"]
    dse = float(dn.std(ddof=1) / np.sqrt(len(dn))) if len(dn) > 1 else float("nan")
    pooled = {"mean_diff_n": float(dn.mean()), "se": dse, "z": float(dn.mean() / dse) if dse > 0 else None,
              "mean_diff_rel": float(dn.mean() / fp64["mean_n"].mean())}
    per_box = [{"mu_kjmol": round(float(m), 4), "mean_n_mixed": float(a), "se_mixed": float(sa),
                "mean_n_fp64": float(b), "se_fp64": float(sb), "density_g_cm3_mixed": density(a),
                "density_g_cm3_fp64": density(b), "z": float(zz), "p": float(pp)}
               for m, a, sa, b, sb, zz, pp in zip(mu, mixed["mean_n"], mixed["se_n"], fp64["mean_n"], fp64["se_n"], z,
                                                  pvals)]
    for d in (mixed, fp64):
        del d["mean_n"], d["se_n"]
    out = {"workload": "GCMC of united-atom n-butane (CBMC kappa_ins 12, kappa_dih 12) in 16 boxes of 40 A at "
                       "300 K, mu evenly spaced over [-30, -20] kJ/mol, 14 A cut_tail; insert/delete 40 %, "
                       "translate/rotate 40 %, regrow 20 %; one CTA per box, all boxes in one launch",
           "mixed": mixed, "fp64": fp64, "mixed_over_fp64": mixed["moves_per_s"] / fp64["moves_per_s"],
           "density_check": {"max_abs_z": float(np.max(np.abs(z))), "rms_z": float(np.sqrt(np.mean(z ** 2))),
               "boxes_p_below_0.01": int(np.sum(pvals < 0.01)), "min_p": float(np.min(pvals)),
               "p_note": "two-sided p of each box's z under a Student t with 3 degrees of freedom (the top "
                         "blocking level keeps 4 blocks, so each standard error is itself uncertain)",
               "mean_abs_rel_diff_n": float(
               np.mean([abs(p["mean_n_mixed"] / max(p["mean_n_fp64"], 1e-9) - 1) for p in per_box])),
               "pooled": pooled,
               "note": f"z = (<N>_mixed - <N>_fp64) / combined standard error; each chain's error from "
                       f"{nsub} sub-block means of {sub_steps} steps blocked pairwise down to 4 blocks, the "
                       f"largest standard error over the blocking levels (Flyvbjerg-Petersen), so correlated "
                       f"sub-blocks do not shrink it.  pooled: the mean of the 16 per-box differences "
                       f"<N>_mixed - <N>_fp64 (independent chains, zero-mean when both sample the same ensembles) "
                       f"with its standard error from their spread"},
           "per_box": per_box}
    # all SMs busy: 152 boxes (the 16 chemical potentials repeated), mixed precision
    wide, gw, _ = chains(abi.PREC_MIXED, [mu[k % nb] for k in range(152)], eq_steps // 4, 1, block_steps, seed=77)
    gw.close()
    del wide["mean_n"], wide["se_n"]
    out["mixed_152boxes"] = wide
    if with_cpu:
        # the FP64 oracle from the mixed chains' equilibrated state, all boxes, all host threads
        from oracle import oracle
        where = gm.molecule_boxes(1)
        live = [int(k) + 1 for k in np.flatnonzero(where)]
        xyz = np.concatenate([gm.get_molecule(im, 1).ravel() for im in live])
        with oracle.open_system(sysm) as o:
            o.set_molecules(live, [1] * len(live), [int(where[im - 1]) for im in live], xyz)
            boxes = list(range(1, nb + 1))
            for b in boxes:
                o.system_total_energy(b)
            t0 = time.perf_counter()
            o.gcmc(boxes, 100, 1, mu, [[1.0]] * nb, [[0.5]] * nb, seed=5, cuts=cuts)
            per = max(time.perf_counter() - t0, 1e-3) / 100
            nstep = int(max(200, min(20000, 12.0 / per)))
            t0 = time.perf_counter()
            o.gcmc(boxes, nstep, 1, mu, [[1.0]] * nb, [[0.5]] * nb, seed=6, cuts=cuts)
            dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"moves_per_s": nb * nstep / dt, "cores": min(nb, oracle.num_threads()),
                               "kind": "port",
                               "sample": f"{nstep} steps of the 16 chains from the mixed chains' equilibrated "
                                         f"state, FP64 C++ oracle, boxes in parallel"}
    gm.close()
    return out


def npt_leg(cg, abi, dev, nchains: int, eq_blocks: int, prod_blocks: int) -> dict:
    """NPT sampling of 4096 rigid waters (12,288 atoms, Ewald 1e-6, 12 A) at 298 K
    and 1 bar -- mixed-precision translate/rotate sweeps on the device, volume moves
    rebuilt on the device with the host's acceptance rule -- in `nchains`
    independent chains, one configuration per chain after each block of one sweep
    and one volume move; the fluctuation formula d<rho>/d(eps_O) =
    -beta (<rho U'> - <rho><U'>) over the saved configurations, with
    U' = dU/d(eps_OO) from the running LJ energy (LJ energies are linear in eps)
    checked against the FP64 adjoint (cass_system_gradient) at the final
    configurations of four chains."""
    from cassandra_gb300 import npt, workloads
    from cassandra_gb300.autograd import fluctuation_sensitivity
    nmol, T = 4096, 298.0
    s = workloads.water_gradient_system(nboxes=nchains)
    boxes = list(range(1, nchains + 1))
    eps_oo = float(s.ff.eps[0, 0])  # internal units (eps/k times kboltz)
    mw = 15.999 + 2 * 1.008
    rho, dud = [], []
    with cg.open_system(s, precision=abi.PREC_MIXED, device=dev) as g:
        ch = npt.NPTChains(g, boxes, [nmol] * nchains, T, 1.0, 400.0, [[0.25]] * nchains, [[0.25]] * nchains,
                           seed=21)
        ch.start([b.length[0] for b in s.boxes])
        t0 = time.perf_counter()
        sweep_ms = 0.0
        for _ in range(eq_blocks):
            ch.sweeps(1, prob_translate=0.5)
            sweep_ms += g.stats()["mc_ms"]
            ch.volume_moves()
        t1 = time.perf_counter()
        for _ in range(prod_blocks):
            ch.sweeps(1, prob_translate=0.5)
            sweep_ms += g.stats()["mc_ms"]
            ch.volume_moves()
            d = ch.densities(mw)
            for k in range(nchains):
                e = ch.components[k]
                rho.append(d[k])
                dud.append((e["inter_vdw"] + e["lrc"]) / eps_oo)
        t2 = time.perf_counter()
        check = []
        for b in boxes[:4]:
            e, _, de, _, _ = g.system_gradient(b, 3 * nmol)
            k = b - 1
            check.append(abs(de[0, 0] - dud[-nchains + k]) / abs(de[0, 0]))
    rho, dud = np.array(rho), np.array(dud)
    beta = 1.0 / (0.8314472 * T)
    sens = fluctuation_sensitivity(rho, dud, beta) * 0.8314472  # per K of eps/k
    # jackknife over chains (configurations of one chain are correlated)
    per = np.arange(len(rho)) % nchains
    jk = np.array([fluctuation_sensitivity(rho[per != c], dud[per != c], beta) * 0.8314472 for c in range(nchains)])
    err = float(np.sqrt((nchains - 1) / nchains * np.sum((jk - jk.mean()) ** 2)))
    blocks = eq_blocks + prod_blocks
    return {"workload": f"NPT of 4096 rigid waters (12,288 atoms, 49.7 A start, Ewald tol 1e-6, 12 A) at 298 K and "
                        f"1 bar, {nchains} chains, blocks of one sweep (4096 translate/rotate moves) and one volume "
                        f"move per chain, mixed precision",
            "configurations": int(len(rho)), "equilibration_blocks": eq_blocks, "production_blocks": prod_blocks,
            "wall_s": t2 - t0, "production_configs_per_s": len(rho) / (t2 - t1),
            "sweeps_per_s": nchains * blocks / (sweep_ms / 1e3),
            "volume_acceptance": float(ch.n_vol_acc.sum() / max(1, ch.n_vol.sum())),
            "mean_density_g_cm3": float(rho.mean()),
            "d_rho_d_eps_O": {"value": sens, "jackknife_err": err, "unit": "g/cm^3 per K of eps_O/k",
                              "formula": "-beta (<rho dU/deps> - <rho><dU/deps>)"},
            "adjoint_check_max_rel_diff": float(max(check)),
            "note": f"{nchains} independent chains from the lattice start, {eq_blocks} equilibration blocks, then one "
                    f"configuration per chain after each of {prod_blocks} production blocks; the error is the "
                    f"jackknife over chains"}


def pregen_leg(cg, abi, system, n_per_box: int, kappa: int, nframes: int, seed: int) -> dict:
    """The headline Widom workload streamed from trajectory files, as the pregen
    driver runs it: per box an .xyz/.H trajectory of `nframes` frames (the frozen
    box with every atom displaced by N(0, 0.05 A) per frame, written to a
    temporary directory), read by the library's reader threads one frame ahead;
    per frame cass_load_next_frame and one batched Widom call, once without and
    once with the system energy of every box each frame.  The first frame of each
    pass is untimed."""
    import shutil
    import tempfile
    from cassandra_gb300 import io, pregen
    boxes = list(range(1, len(system.boxes) + 1))
    rng = np.random.default_rng(seed)
    ms = system.molecules
    xyz_all = ms.flat_xyz().reshape(-1, 3)
    td = tempfile.mkdtemp(prefix="cass_pregen_")
    try:
        t0 = time.perf_counter()
        paths = []
        for b in boxes:
            x0 = xyz_all[np.asarray(ms.ibox) == b]
            L = system.boxes[b - 1].length
            xp, hp = os.path.join(td, f"box{b}.xyz"), os.path.join(td, f"box{b}.H")
            with open(xp, "w") as fx, open(hp, "w") as fh:
                for k in range(nframes + 1):
                    x = x0 + rng.normal(scale=0.05, size=x0.shape)
                    io.write_xyz_frame(fx, x, ["LJ"] * len(x), k)
                    io.write_H_frame(fh, L, [len(x), 0])
            paths.append((xp, hp))
        t_write = time.perf_counter() - t0
        text_bytes = sum(os.path.getsize(p) for pair in paths for p in pair)

        def run(energy_every):
            with cg.open_system(system, precision=abi.PREC_MIXED) as ctx:
                trajs = [cg.open_trajectory(xp, hp, [1, 4]) for xp, hp in paths]
                try:
                    pregen.pregen_widom(ctx, trajs, [2], n_per_box, kappa, kappa, seed=seed, max_frames=1,
                                        energy_every=energy_every)
                    s0 = ctx.stats()
                    p0 = sum(t.stats()["parse_s"] for t in trajs)
                    t0 = time.perf_counter()
                    recs = pregen.pregen_widom(ctx, trajs, [2], n_per_box, kappa, kappa, seed=seed + 1,
                                               max_frames=nframes, energy_every=energy_every)
                    wall = time.perf_counter() - t0
                    s1 = ctx.stats()
                    parse = sum(t.stats()["parse_s"] for t in trajs) - p0
                finally:
                    for t in trajs:
                        t.close()
            nf = len(recs)
            trials = n_per_box * len(boxes) * 2 * kappa * nf
            return {"frames": nf, "value": trials / wall, "unit": UNIT, "frames_per_s": nf / wall,
                    "load_s_per_frame": float(np.mean([r["load_s"] for r in recs])),
                    "energy_s_per_frame": float(np.mean([r["energy_s"] for r in recs])),
                    "widom_s_per_frame": float(np.mean([r["widom_s"] for r in recs])),
                    "reader_parse_s_per_frame": parse / nf,
                    "h2d_bytes_per_frame": int((s1["h2d_bytes"] - s0["h2d_bytes"]) / nf),
                    "d2h_bytes_per_frame": int((s1["d2h_bytes"] - s0["d2h_bytes"]) / nf)}

        return {"workload": f"{len(boxes)} LJ boxes streamed from .xyz/.H trajectories, {n_per_box * len(boxes)} "
                            f"butane insertions per frame (kappa {kappa}/{kappa}), mixed precision",
                "widom_only": run(0), "with_total_energies": run(1), "reader_threads": len(paths),
                "text_mb_per_frame": text_bytes / (nframes + 1) / 1e6, "write_s": t_write,
                "note": "host wall clock per frame: load (waits for a reader only if it is behind; repack, pinned "
                        "upload, long-range correction), system energies of every box (with_total_energies: "
                        "every frame, as a pregen run printing thermo data each frame), Widom; "
                        "reader_parse_s_per_frame is summed over the reader threads and overlaps the previous "
                        "frame's device work"}
    finally:
        shutil.rmtree(td, ignore_errors=True)


def gradient_leg(cg, abi, dev) -> dict:
    """Configuration gradients/s of 4096 rigid waters with Ewald (FP64 adjoint),
    spot-checked against central differences of the FP64 GPU energy."""
    from cassandra_gb300 import workloads
    s = workloads.water_gradient_system()
    n = 3 * len(s.molecules.im)
    with cg.open_system(s, precision=abi.PREC_FP64, device=dev) as g:
        g.system_gradient(1, n)  # warm-up
        reps = 3
        t0 = time.perf_counter()
        for _ in range(reps):
            e, grad, de, ds, dq = g.system_gradient(1, n)
        dt = (time.perf_counter() - t0) / reps
        # central differences (h = 1e-6 relative) of the FP64 GPU energy
        m = s.molecules
        xyz = m.flat_xyz().copy()
        errs = []
        scale = float(np.max(np.abs(grad)))
        for idx in (5, 3 * 1000 + 1, 3 * 2047 + 7, 3 * 4095 + 8):
            h = 1e-6 * max(1.0, abs(xyz[idx]))
            x = xyz.copy()
            x[idx] += h
            g.set_molecules(m.im, m.is_, m.ibox, x)
            ep = g.system_total_energy(1)[0]["total"]
            x[idx] -= 2 * h
            g.set_molecules(m.im, m.is_, m.ibox, x)
            em = g.system_total_energy(1)[0]["total"]
            errs.append(abs((ep - em) / (2 * h) - grad.ravel()[idx]) / scale)
        g.set_molecules(m.im, m.is_, m.ibox, xyz)
    return {"workload": "4096 rigid 3-site waters (12,288 atoms), 49.7 A box, 12 A LJ + Ewald real space, tol 1e-6",
            "configs_per_s": 1.0 / dt, "ms_per_config": 1e3 * dt, "precision": "fp64",
            "outputs": "dU/dr for every atom, dU/d(eps, sigma) per type pair, dU/dq per species atom",
            "fd_check": {"coordinates": len(errs), "max_rel_err": float(max(errs)),
                         "note": "central differences h = 1e-6 relative of the FP64 GPU energy, relative to max |dU/dr|"}}


def flush_l2(torch, buf):
    buf.zero_()


def run_reference(args, rank, world):
    if rank != 0:
        return
    system = build_workload(args, rank)
    from oracle import oracle
    boxes = list(range(1, len(system.boxes) + 1))
    vals, times = [], []
    with oracle.open_system(system) as o:
        for b in boxes:
            o.system_total_energy(b)
        t0 = time.perf_counter()
        o.widom_insert(2, boxes, 4, args.kappa, args.kappa, seed=1)
        per = max(time.perf_counter() - t0, 1e-3) / (4 * len(boxes))
        n = max(4, int(args.cpu_seconds / 3.0 / (per * len(boxes))))
        for s in range(args.warmup):
            o.widom_insert(2, boxes, 2, args.kappa, args.kappa, seed=1000 + s)
        for s in range(args.steps):
            t0 = time.perf_counter()
            res = o.widom_insert(2, boxes, n, args.kappa, args.kappa, seed=s + 1)
            dt = time.perf_counter() - t0
            trials = sum(r["n_trials"] for r in res)
            vals.append(trials / dt)
            times.append(dt)
    value = float(np.sum([v * t for v, t in zip(vals, times)]) / np.sum(times))
    out = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * float(np.mean(times)),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": {"workload": "butane CBMC Widom into 64 frozen LJ boxes (N 200-4000, rho*=0.6), "
                                  "kappa_ins=12, kappa_dih=12", "boxes": len(boxes),
                      "insertions_per_step": n * len(boxes), "sample_per_box": n},
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": oracle.num_threads(), "kind": "port",
                            "sample": f"{len(boxes)} boxes x {n} insertions per step; the reference is Fortran and "
                                      f"no Fortran compiler exists here, so its C++ FP64 restatement is timed"},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def profile_case(args):
    """The small cases of the ncu captures in profiles/: three launches of the
    mixed (cells of rcut_cbmc) or FP64 (cells of rcut_cbmc / 4) Widom kernel on 16
    boxes, or four launches of the MC kernel on single chains."""
    import cassandra_gb300 as cg
    from cassandra_gb300 import abi, build, workloads
    build.build()
    if args.profile_case == "mc":
        for sysm, prec, pt, nsw in ((workloads.water_nvt_system(nboxes=1), abi.PREC_FP64, 0.5, 2),
                                    (workloads.lj_nvt_system(nboxes=1), abi.PREC_MIXED, 1.0, 20)):
            ns = len(sysm.species)
            with cg.open_system(sysm, precision=prec) as g:
                g.system_total_energy(1)
                g.mc_sweeps([1], 1, [[0.8] * ns], [[0.4] * ns], seed=1, prob_translate=pt)
                g.mc_sweeps([1], nsw, [[0.8] * ns], [[0.4] * ns], seed=2, prob_translate=pt)
                st = g.stats()
                print(json.dumps({"case": "mc", "precision": prec, "sweeps": nsw, "kernel_ms": st["mc_ms"],
                                  "sweeps_per_s": nsw / (st["mc_ms"] / 1e3), "ctas_per_chain": st["gcmc_cluster"]}))
        return
    nb = 16
    s = workloads.widom_batch_system(nboxes=nb, seed=args.seed, nconfig=1000)
    boxes = list(range(1, nb + 1))
    mixed = args.profile_case == "mixed"
    n = 16000 if mixed else 4096
    with cg.open_system(s, precision=abi.PREC_MIXED if mixed else abi.PREC_FP64) as g:
        for b in boxes:
            g.system_total_energy(b)
        g.set_widom_autotune(False)
        g.set_widom_cells(1.0 if mixed else 4.0)
        for r in range(3):
            g.widom_insert(2, boxes, n, args.kappa, args.kappa, seed=1 + r)
            st = g.stats()
            print(json.dumps({"case": args.profile_case, "insertions": nb * n, "kernel_ms": st["widom_kernel_ms"],
                              "grid": st["widom_grid_x"], "block": st["widom_block"]}))


def main():
    args = parse()
    rank, world, local = dist_info()
    if args.profile_case:
        profile_case(args)
        return
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    import torch
    import cassandra_gb300 as cg
    from cassandra_gb300 import abi, build

    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    build.build()
    dev = local
    torch.cuda.set_device(dev)
    system = build_workload(args, rank)
    boxes = list(range(1, len(system.boxes) + 1))
    n_per_box = max(1, args.insertions // len(boxes))
    trials_per_ins = args.kappa + args.kappa  # kappa_ins + (nfrag - 1) kappa_dih, butane has 2 fragments
    stream = torch.cuda.Stream(device=dev)
    l2 = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{dev}")

    def barrier():
        if dist is not None:
            dist.barrier()

    def timed_steps(ctx, steps, warmup, seed0):
        ctx.set_stream(stream.cuda_stream)
        for s in range(warmup):
            ctx.widom_insert(2, boxes, n_per_box, args.kappa, args.kappa, seed=seed0 + 1000 + s)
        st0 = ctx.stats()
        per_step, kern, allres = [], [], []
        barrier()
        torch.cuda.synchronize()
        for s in range(steps):
            with torch.cuda.stream(stream):
                flush_l2(torch, l2)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            res = ctx.widom_insert(2, boxes, n_per_box, args.kappa, args.kappa, seed=seed0 + s + rank * 7919)
            e1.record(stream)
            torch.cuda.synchronize()
            per_step.append(e0.elapsed_time(e1))
            kern.append(ctx.stats()["widom_kernel_ms"])
            allres.append(res)
        barrier()
        st1 = ctx.stats()
        timed_steps.results = allres
        return per_step, kern, res, st1["kernel_launches"] - st0["kernel_launches"]

    def mu_ex(allres):
        """Excess chemical potential per box, -kT ln <widom_var>, in kJ/mol: the mean
        over the timed steps and its standard error from their spread."""
        kT = 0.8314472 * system.boxes[0].temperature * 0.01
        per = np.array([[-kT * np.log(max(r["widom_sum"] / r["prefactor"] / r["n_insertions"], 1e-300))
                         for r in step] for step in allres])  # [steps, boxes]
        se = per.std(axis=0, ddof=1) / np.sqrt(len(per)) if len(per) > 1 else np.zeros(per.shape[1])
        return per.mean(axis=0), se

    # headline: mixed precision
    gctx = cg.open_system(system, precision=abi.PREC_MIXED, device=dev)
    for b in boxes:
        gctx.system_total_energy(b)
    clocks = ClockSampler(dev)
    clocks.start()
    t_wall0 = time.perf_counter()
    ms, kms, res, launches = timed_steps(gctx, args.steps, args.warmup, args.seed)
    t_wall = time.perf_counter() - t_wall0
    clk = clocks.stop()
    total_ms = float(np.sum(ms))
    if dist is not None:
        t = torch.tensor([total_ms], device=f"cuda:{dev}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    timed_steps_mixed_results = list(timed_steps.results)
    # per-box accumulators of every rank's boxes, merged with one small all-reduce per
    # step (each box has one owner): the job's mu_ex over all world x boxes boxes
    from cassandra_gb300 import shard
    gboxes = list(range(1, world * len(boxes) + 1))
    mine_g = [rank * len(boxes) + b for b in boxes]
    merged_steps = [shard.merge_box_results(gboxes, mine_g, r) for r in timed_steps_mixed_results]
    mu_mixed, mu_mixed_se = mu_ex(merged_steps)
    mu_cmp = None
    trials_step = n_per_box * len(boxes) * trials_per_ins
    value = trials_step * args.steps * world / (total_ms / 1000.0)
    # work counts for the roofline (one extra, untimed pass)
    gctx.set_count_pairs(True)
    gctx.widom_insert(2, boxes, n_per_box, args.kappa, args.kappa, seed=args.seed + 555)
    st = gctx.stats()
    gctx.set_count_pairs(False)
    # plain FP64 GPU path on the same workload, and the accuracy of the mixed
    # path against it (per-insertion traces of a sub-batch)
    fp64 = None
    accuracy = None
    if args.fp64_steps > 0:
        fctx = cg.open_system(system, precision=abi.PREC_FP64, device=dev)
        for b in boxes:
            fctx.system_total_energy(b)
        fms, fkms, _, _ = timed_steps(fctx, args.fp64_steps, 1, args.seed)
        mu_fp64, _ = mu_ex(timed_steps.results)
        nst = min(len(timed_steps.results), args.steps)
        mu_mixed_same, _ = mu_ex(timed_steps_mixed_results[:nst])  # rank 0's boxes, as mu_fp64
        fp64_value = trials_step * len(fms) / (float(np.sum(fms)) / 1000.0)
        fp64 = {"value": fp64_value, "unit": UNIT, "ms_per_step": float(np.mean(fms)),
                "kernel_ms": float(np.mean(fkms)), "mixed_over_fp64": value / world / fp64_value}
        mu_cmp = {"max_abs_diff_kjmol": float(np.max(np.abs(mu_mixed_same - mu_fp64))),
                  "mean_abs_diff_kjmol": float(np.mean(np.abs(mu_mixed_same - mu_fp64))),
                  "steps_compared": nst,
                  "note": "mixed and FP64 over the same timed steps (the same seeds, so the same insertion "
                          "streams): the difference is the precision's, not sampling noise"}
        sub = boxes[:8]
        ra, ta = fctx.widom_insert(2, sub, 2000, args.kappa, args.kappa, seed=4242, trace=True)
        rb, tb = gctx.widom_insert(2, sub, 2000, args.kappa, args.kappa, seed=4242, trace=True)
        same = (ta["overlap"] == tb["overlap"]) & (ta["selected_trial"] == tb["selected_trial"])
        ok = same & (ta["overlap"] == 0)
        err = np.abs(tb["e_inter"][ok] - ta["e_inter"][ok])
        rel = err / np.maximum(ta["e_inter_abs"][ok], 1.0)
        rel_e = err / np.maximum(np.abs(ta["e_inter"][ok]), 1e-300)
        accuracy = {"bound": "|E_mixed - E_fp64| / sum |pair energies| of the full-cutoff inter energy, every "
                             "insertion with the same status and selected trials (the FP64 GPU path equals the "
                             "FP64 oracle to 1e-14 on these traces)",
                    "same_status": float((ta["overlap"] == tb["overlap"]).mean()),
                    "same_trial_selection": float(same.mean()),
                    "e_inter_max_rel_err": float(rel.max()) if rel.size else None,
                    "e_inter_mean_rel_err": float(rel.mean()) if rel.size else None,
                    "e_inter_p999_rel_err": float(np.quantile(rel, 0.999)) if rel.size else None,
                    "frac_within_1e-5": float((rel <= 1e-5).mean()) if rel.size else None,
                    "e_inter_max_rel_err_of_abs_E": float(rel_e.max()) if rel_e.size else None,
                    "e_inter_median_rel_err_of_abs_E": float(np.median(rel_e)) if rel_e.size else None,
                    "insertions_compared": int(same.size),
                    "fp64_fixups": int(gctx.stats()["widom_fixups"]),
                    "note": "pairs whose FP32 r^2 lies within rounding of a cutoff are decided again in FP64 "
                            "(k_widom_fix, fp64_fixups insertions here), so every cutoff and overlap decision "
                            "is the FP64 one; the error left is the FP32 rounding of coordinates"}
        fctx.close()

    # roofline of the Widom kernel
    from cassandra_gb300 import system as sysmod
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    kern_ms = float(np.mean(kms))
    natoms = [sum(1 for bi in system.molecules.ibox if bi == b) for b in boxes]
    box_bytes = 0
    for b, na in zip(boxes, natoms):
        L = system.boxes[b - 1].length[0]
        nc = max(1, int(L // system.boxes[b - 1].rcut_cbmc)) ** 3
        box_bytes += st["widom_grid_x"] * (na * 16 + (nc + 1) * 4)
    alg_bytes = n_per_box * len(boxes) * 33 + box_bytes
    achieved_gbs = alg_bytes / (kern_ms / 1000.0) / 1e9
    traffic = None
    prof = os.path.join(ROOT, "profiles", WIDOM_PROFILE)
    if os.path.exists(prof):
        import re
        with open(prof) as f:
            m = re.search(r"dram_bytes_per_insertion:\s*([0-9.eE+-]+)", f.read())
        if m:
            traffic = float(m.group(1)) * n_per_box * len(boxes)
    # FP32 work of the launch: 15 ops per candidate pair visited (displacement, r^2,
    # cutoff test) + 8 per in-cutoff LJ pair; the algorithmic floor counts only the
    # in-cutoff pairs (23 ops each), which any neighbour search must evaluate
    flops = st["widom_pairs_visited"] * 15 + st["widom_pairs_in_cutoff"] * 8
    flops_alg = st["widom_pairs_in_cutoff"] * 23
    sm_count = torch.cuda.get_device_properties(dev).multi_processor_count
    fp32_peak = sm_count * 128 * 2 * float(peaks.get("sm_max_mhz", 2070.0)) * 1e6 / 1e12
    achieved_tf = flops / (kern_ms / 1000.0) / 1e12
    achieved_alg_tf = flops_alg / (kern_ms / 1000.0) / 1e12

    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "fp32 pair math / fp64 accumulation", "data": "synthetic",
           "config": {"workload": "butane CBMC Widom into 64 frozen LJ boxes (N 200-4000, rho*=0.6), "
                                  "kappa_ins=12, kappa_dih=12, 24 trial energies per insertion",
                      "boxes": len(boxes), "insertions_per_step": n_per_box * len(boxes),
                      "trial_energies_per_step": trials_step, "atoms_total": int(sum(natoms)),
                      "l2": "flushed (256 MB write) between timed steps", "precision": "mixed",
                      "parallelism": f"box shards x{world}",
                      "sharding": "each rank owns its own boxes (rank r: boxes seeded by r), per-rank work fixed; "
                                  "per-box Widom accumulators merged by one all-reduce after the timed steps"},
           "widom_launch": {"ctas_per_box": st["widom_grid_x"], "threads": st["widom_block"],
                            "smem_bytes": st["widom_smem_bytes"], "fp64_fixups": int(st["widom_fixups"]),
                            "fp64_fixup_fraction": st["widom_fixups"] / float(n_per_box * len(boxes)),
                            "note": "shape chosen by the library's launch autotuner on its first call"},
           "gpu_launches": int(launches),
           "wall_s": t_wall,
           "mu_ex_per_box": {"unit": "kJ/mol", "definition": "-kT ln <widom_var> (widom_insert.f90:445-447), "
                                                         "T = 150 K", "mixed": [round(float(v), 5) for v in mu_mixed],
                             "mixed_se": [round(float(v), 5) for v in mu_mixed_se],
                             "boxes": len(gboxes),
                             "n_atoms_per_box_rank0": [int(sum(1 for bi in system.molecules.ibox if bi == b))
                                                       for b in boxes],
                             "mixed_vs_fp64": mu_cmp},
           "fp64_gpu": fp64,
           "accuracy_vs_fp64": accuracy,
           "roofline": {"bound": "fp32", "achieved": achieved_tf, "peak": fp32_peak, "unit": "TFLOP/s",
                        "frac": achieved_tf / fp32_peak, "traffic": traffic,
                        "pairs_visited": st["widom_pairs_visited"], "pairs_in_cutoff": st["widom_pairs_in_cutoff"],
                        "in_cutoff_only": {"achieved": achieved_alg_tf, "frac": achieved_alg_tf / fp32_peak},
                        "note": "the Widom kernels (k_widom_f32, one thread per insertion, then k_widom_fix for the "
                                "insertions it queues; kernel_ms spans both); 15 FP32 ops per visited candidate pair "
                                "+ 8 per in-cutoff LJ pair, pairs counted by the kernel in an extra untimed pass; "
                                "peak is nominal (SMs x 128 FP32 lanes x 2 x max SM clock): the measured-peak file "
                                "has no FP32 figure; traffic = DRAM bytes per launch scaled from the ncu capture "
                                "in profiles/ (per insertion x insertions)"},
           "hbm_roofline": {"bound": "hbm", "achieved": achieved_gbs, "peak": hbm_peak, "unit": "GB/s",
                            "frac": achieved_gbs / hbm_peak,
                            "note": "algorithmic bytes = 33 B record per insertion + box staged once per CTA; "
                                    "peak of measured; the kernel keeps its box in shared memory, so HBM is idle"},
           "kernel_ms": kern_ms, "clocks": clk}

    # end to end through the public API with host buffers (frame upload, energies, Widom, results back)
    if not args.no_e2e:
        xyz_frames = system.molecules.flat_xyz()
        ims, iss, ibs = system.molecules.im, system.molecules.is_, system.molecules.ibox
        e2e_steps = max(1, min(args.steps, 3))
        s0 = gctx.stats()
        gctx.set_stream(stream.cuda_stream)
        t0 = time.perf_counter()
        for s in range(e2e_steps):
            gctx.set_molecules(ims, iss, ibs, xyz_frames)
            for b in boxes:
                gctx.system_total_energy(b)
            gctx.widom_insert(2, boxes, n_per_box, args.kappa, args.kappa, seed=args.seed + 77 + s)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        s1 = gctx.stats()
        out["e2e"] = {"value": trials_step * e2e_steps / dt, "unit": UNIT,
                      "h2d_bytes_per_step": int((s1["h2d_bytes"] - s0["h2d_bytes"]) / e2e_steps),
                      "d2h_bytes_per_step": int((s1["d2h_bytes"] - s0["d2h_bytes"]) / e2e_steps),
                      "steps": e2e_steps,
                      "note": "per step: set_molecules of all boxes, system_total_energy of each box, widom_insert; "
                              "host wall clock"}
    gctx.close()
    if not args.no_pregen:
        pf = pregen_leg(cg, abi, system, n_per_box, args.kappa, args.pregen_frames, args.seed + 31)
        out["pregen_feed"] = pf
        w = pf["widom_only"]
        if "e2e" in out:
            out["e2e_set_molecules"] = out.pop("e2e")
        out["e2e"] = {"value": w["value"], "unit": UNIT, "h2d_bytes_per_step": w["h2d_bytes_per_frame"],
                      "d2h_bytes_per_step": w["d2h_bytes_per_frame"], "steps": w["frames"],
                      "note": "the headline workload through the public API from trajectory files: per step "
                              "(frame) cass_load_next_frame of all 64 boxes (text parsed by reader threads into "
                              "pinned buffers, pinned upload) and one cass_widom_insert, results read back; "
                              "host wall clock"}
    # the other configurations run on one GPU only: a multi-GPU run measures the
    # sharded Widom headline and holds its GPUs no longer than that
    solo = world == 1
    if solo and not args.no_mc:
        out["mc_sweeps"] = mc_leg(cg, abi, dev, not args.no_cpu_baseline)
    if solo and not args.no_gcmc:
        out["gcmc"] = gcmc_leg(cg, abi, dev, not args.no_cpu_baseline,
                               eq_steps=args.gcmc_eq_steps, blocks=args.gcmc_blocks, block_steps=args.gcmc_block_steps)
    if solo and not args.no_grad:
        out["gradient"] = gradient_leg(cg, abi, dev)
    if solo and not args.no_npt:
        out["npt_fluctuation"] = npt_leg(cg, abi, dev, args.npt_chains, args.npt_eq_blocks, args.npt_blocks)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(system, args)
        one = cpu_baseline(system, args, threads=1, seconds=min(args.cpu_seconds, 10.0))
        out["cpu_baseline"]["one_thread"] = {"value": one["value"], "cores": one["cores"], "sample": one["sample"]}
    if rank == 0:
        print(json.dumps(out))
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
