"""The pregen driver's frame loop with Widom insertions (pregen_driver.f90:116-200
with Widom_Subdriver, widom_subdriver.f90) over the library's trajectory feed.

Per frame: cass_load_next_frame for every box (Load_Next_Frame, which also
sets up the long-range correction and the Ewald structure factors the
insertions need), every `energy_every` frames the system energy of every box
(Compute_System_Total_Energy, pregen_driver.f90:187, run by the reference at
its thermo output frequency), then one batched Widom call over all boxes for
each inserted species.  The library reads frame
k+1 on its reader threads while the device works on frame k.
"""
from __future__ import annotations

import time
from typing import Sequence


def pregen_widom(ctx, trajectories: Sequence, species: Sequence[int], n_insertions, kappa_ins: int,
                 kappa_dih: int, seed: int, max_frames: int | None = None, trace: bool = False,
                 energy_every: int = 1) -> list:
    """Runs the frame loop until a trajectory ends (or max_frames).  n_insertions
    is one count for every species or a list per species.  Returns one record
    per frame: {"frame", "energy": [per box] or None, "overlap": [per box] or None,
    "widom": {species: [per-box results]}, "trace": {species: array} (trace only),
    "load_s", "energy_s", "widom_s"}.  The seed of frame f and species is is
    seed + 1000 * f + is, so that any frame can be rerun alone."""
    nins = list(n_insertions) if isinstance(n_insertions, (list, tuple)) else [n_insertions] * len(species)
    boxes = list(range(1, len(trajectories) + 1))
    out = []
    f = 0
    while max_frames is None or f < max_frames:
        t0 = time.perf_counter()
        if ctx.load_next_frame(trajectories):
            break
        t1 = time.perf_counter()
        energies = overlaps = None
        if energy_every > 0 and f % energy_every == 0:
            energies, overlaps = [], []
            for ib in boxes:
                e, ov = ctx.system_total_energy(ib)
                energies.append(e)
                overlaps.append(ov)
        t2 = time.perf_counter()
        rec = {"frame": f, "energy": energies, "overlap": overlaps, "widom": {}, "trace": {}}
        for is_, n in zip(species, nins):
            r = ctx.widom_insert(is_, boxes, n, kappa_ins, kappa_dih, seed=seed + 1000 * f + is_, trace=trace)
            if trace:
                rec["widom"][is_], rec["trace"][is_] = r
            else:
                rec["widom"][is_] = r
        t3 = time.perf_counter()
        rec.update(load_s=t1 - t0, energy_s=t2 - t1, widom_s=t3 - t2)
        out.append(rec)
        f += 1
    return out
