"""ctypes mirror of include/cassandra_gb300.h and a thin context wrapper.

The same wrapper drives any shared library that implements the header's entry
points under a symbol prefix (``cass_`` for the CUDA library).  Arguments keep
the reference's 1-based (im, is, ibox) indices.
"""
from __future__ import annotations

import ctypes as C
from typing import Sequence

import numpy as np

CASS_OK = 0
CASS_EINVAL = -1
CASS_ECAPACITY = -2
CASS_ECUDA = -3
CASS_ETIMEDOUT = -4
CASS_ESTATE = -5
CASS_ENOMEM = -6
CASS_EUNSUPPORTED = -7

PREC_FP64 = 0
PREC_MIXED = 1

VDW_NONE, VDW_LJ, VDW_MIE = 0, 1, 2
VDW_SUM_CUT, VDW_SUM_CUT_TAIL, VDW_SUM_CUT_SHIFT, VDW_SUM_MINIMUM = 0, 1, 2, 3
VDW_SUM_CUT_SWITCH, VDW_SUM_CHARMM, VDW_SUM_CUT_SHIFT_FORCE = 4, 5, 6
CHARGE_NONE, CHARGE_COUL = 0, 1
QQ_EWALD, QQ_CUT, QQ_MINIMUM, QQ_DSF = 0, 1, 2, 3
MOVE_INSERTION, MOVE_DELETION, MOVE_TRANSLATION, MOVE_ROTATION, MOVE_INTRA = 0, 1, 2, 3, 4
BONDED_FIXED, BONDED_HARMONIC = 0, 1

_i32p = C.POINTER(C.c_int32)
_f64p = C.POINTER(C.c_double)


class CassConfig(C.Structure):
    _fields_ = [("nspecies", C.c_int32), ("ntypes", C.c_int32), ("nboxes", C.c_int32),
                ("precision", C.c_int32), ("device", C.c_int32), ("max_kvectors", C.c_int32),
                ("max_molecules", _i32p)]


class CassSpeciesDesc(C.Structure):
    _fields_ = [("natoms", C.c_int32), ("atom_type", _i32p), ("charge", _f64p), ("mass", _f64p),
                ("vdw_intra_scale", _f64p), ("charge_intra_scale", _f64p), ("bonded", _i32p),
                ("nbonds", C.c_int32), ("bond_atoms", _i32p), ("bond_kind", _i32p), ("bond_param", _f64p),
                ("nangles", C.c_int32), ("angle_atoms", _i32p), ("angle_kind", _i32p), ("angle_param", _f64p),
                ("ndihedrals", C.c_int32), ("dihedral_atoms", _i32p), ("dihedral_rb", _f64p),
                ("nimpropers", C.c_int32), ("improper_atoms", _i32p), ("improper_param", _f64p),
                ("nfragments", C.c_int32), ("frag_natoms", _i32p), ("frag_atoms", _i32p),
                ("frag_nconnect", _i32p), ("frag_connect", _i32p), ("frag_nconfig", _i32p),
                ("frag_library", _f64p), ("l_coul_cbmc", C.c_int32)]


class CassBoxDesc(C.Structure):
    _fields_ = [("length", C.c_double * 3), ("vdw_style", C.c_int32), ("vdw_sum_style", C.c_int32),
                ("rcut_vdw", C.c_double), ("rcut_coul", C.c_double), ("rcut_cbmc", C.c_double),
                ("rcut_low", C.c_double), ("ron_switch", C.c_double), ("roff_switch", C.c_double),
                ("charge_style", C.c_int32), ("charge_sum_style", C.c_int32), ("ewald_tol", C.c_double),
                ("alpha_dsf", C.c_double), ("temperature", C.c_double)]


class CassEnergy(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("total", "intra", "bond", "angle", "dihedral", "improper",
                                          "intra_vdw", "intra_q", "inter", "inter_vdw", "inter_q",
                                          "lrc", "reciprocal", "self")]

    def as_dict(self) -> dict:
        return {n: getattr(self, n) for n, _ in self._fields_}


class CassWidomResult(C.Structure):
    _fields_ = [("widom_sum", C.c_double), ("prefactor", C.c_double), ("n_insertions", C.c_int64),
                ("n_overlaps", C.c_int64), ("n_trials", C.c_int64)]


class CassWidomTrace(C.Structure):
    _fields_ = [("widom_var", C.c_double), ("ln_pbias", C.c_double), ("e_inter", C.c_double),
                ("e_first_trial_sum", C.c_double), ("e_inter_abs", C.c_double), ("selected_trial", C.c_int32),
                ("overlap", C.c_int32)]


class CassMCParams(C.Structure):
    _fields_ = [("nsweeps", C.c_int64), ("steps_per_sweep", C.c_int32), ("nupdate", C.c_int32),
                ("prob_translate", C.c_double), ("target_accept", C.c_double)]


class CassMCResult(C.Structure):
    _fields_ = [("energy", CassEnergy), ("n_translate", C.c_int64), ("n_translate_accepted", C.c_int64),
                ("n_rotate", C.c_int64), ("n_rotate_accepted", C.c_int64), ("n_overlap", C.c_int64)]

    def as_dict(self) -> dict:
        d = {n: getattr(self, n) for n, _ in self._fields_ if n != "energy"}
        d["energy"] = self.energy.as_dict()
        return d


class CassGCMCParams(C.Structure):
    _fields_ = [("nsteps", C.c_int64), ("is_exchange", C.c_int32), ("kappa_ins", C.c_int32),
                ("kappa_dih", C.c_int32), ("reserved", C.c_int32), ("cut_translate", C.c_double),
                ("cut_rotate", C.c_double), ("cut_insert", C.c_double), ("cut_delete", C.c_double),
                ("cut_regrow", C.c_double)]


class CassGCMCResult(C.Structure):
    _fields_ = [("energy", CassEnergy)] + [(n, C.c_int64) for n in (
        "n_translate", "n_translate_accepted", "n_rotate", "n_rotate_accepted", "n_insert", "n_insert_accepted",
        "n_delete", "n_delete_accepted", "n_regrow", "n_regrow_accepted", "n_molecules")] + \
        [("sum_n_molecules", C.c_double)]

    def as_dict(self) -> dict:
        d = {n: getattr(self, n) for n, _ in self._fields_ if n != "energy"}
        d["energy"] = self.energy.as_dict()
        return d


class CassCBMCOptions(C.Structure):
    _fields_ = [("energy_table_res", C.c_int32), ("sector_overlap", C.c_int32), ("rmin_u_max", C.c_double)]


class CassStats(C.Structure):
    _fields_ = [("widom_ms", C.c_double), ("widom_kernel_ms", C.c_double), ("kernel_launches", C.c_int64),
                ("h2d_bytes", C.c_int64), ("d2h_bytes", C.c_int64), ("widom_pairs_visited", C.c_int64),
                ("widom_pairs_in_cutoff", C.c_int64), ("widom_grid_x", C.c_int32), ("widom_grid_y", C.c_int32),
                ("widom_block", C.c_int32), ("widom_smem_bytes", C.c_int32), ("mc_ms", C.c_double),
                ("mc_moves", C.c_int64), ("gcmc_cluster", C.c_int32), ("widom_fixups", C.c_int32)]

    def as_dict(self) -> dict:
        return {n: getattr(self, n) for n, _ in self._fields_}


class CassFrame(C.Structure):
    _fields_ = [("status", C.c_int32), ("natoms", C.c_int32), ("index", C.c_int64), ("box", C.c_double * 9),
                ("nmols", C.POINTER(C.c_int32)), ("xyz", C.POINTER(C.c_double)), ("pinned", C.c_int32),
                ("reserved", C.c_int32)]


TRACE_DTYPE = np.dtype([("widom_var", "f8"), ("ln_pbias", "f8"), ("e_inter", "f8"),
                        ("e_first_trial_sum", "f8"), ("e_inter_abs", "f8"), ("selected_trial", "i4"),
                        ("overlap", "i4")])
assert TRACE_DTYPE.itemsize == C.sizeof(CassWidomTrace)

# entry points of the header: name -> (restype, argtypes)
SIGNATURES = {
    "abi_version": (C.c_int, []),
    "last_error": (C.c_char_p, []),
    "ctx_create": (C.c_int, [C.POINTER(CassConfig), C.POINTER(C.c_void_p)]),
    "ctx_destroy": (C.c_int, [C.c_void_p]),
    "set_nonbond_table": (C.c_int, [C.c_void_p, C.c_int32, _f64p, _f64p, _f64p, _f64p]),
    "set_species": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(CassSpeciesDesc)]),
    "set_box": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(CassBoxDesc)]),
    "set_molecules": (C.c_int, [C.c_void_p, C.c_int32, _i32p, _i32p, _i32p, _f64p]),
    "remove_molecule": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32]),
    "get_molecule": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, _f64p]),
    "get_molecule_boxes": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, _i32p]),
    "set_cbmc_options": (C.c_int, [C.c_void_p, C.POINTER(CassCBMCOptions)]),
    "volume_scale": (C.c_int, [C.c_void_p, C.c_int32, C.c_double, C.POINTER(CassEnergy), _i32p]),
    "volume_restore": (C.c_int, [C.c_void_p, C.c_int32]),
    "mol_inter_energy": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, _f64p, _f64p, _i32p]),
    "mol_intra_energy": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, _f64p, _f64p, _f64p, _i32p]),
    "system_total_energy": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.POINTER(CassEnergy), _i32p]),
    "ewald_update": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32, _f64p]),
    "ewald_restore": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32]),
    "ewald_widom": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, _f64p, _f64p]),
    "widom_insert": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, _i32p, C.c_int64, C.c_int32, C.c_int32,
                               C.c_uint64, C.POINTER(CassWidomResult), C.c_void_p]),
    "mc_sweeps": (C.c_int, [C.c_void_p, C.c_int32, _i32p, C.POINTER(CassMCParams), _f64p, _f64p, C.c_uint64,
                            C.POINTER(CassMCResult)]),
    "system_gradient": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(CassEnergy), _f64p, _f64p, _f64p, _f64p]),
    "gcmc": (C.c_int, [C.c_void_p, C.c_int32, _i32p, C.POINTER(CassGCMCParams), _f64p, _f64p, _f64p, C.c_uint64,
                       C.POINTER(CassGCMCResult)]),
    "atom_intra_energies": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32, _f64p, _i32p,
                                      C.c_int32, _f64p, _i32p]),
    "cbmc_trial_energies": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32, _i32p, C.c_int32,
                                      _f64p, C.c_int32, _f64p, _i32p]),
    # allocation-free energy entry point and run-time extensions of the GPU
    # library (no counterpart in the reference)
    "mol_box_energy_noalloc": (C.c_int, [C.POINTER(CassBoxDesc), C.c_int32, _f64p, _f64p, C.c_void_p, C.c_void_p,
                                         C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32,
                                         C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p]),
    "traj_open": (C.c_int, [C.c_char_p, C.c_char_p, C.c_int32, _i32p, _i32p, _f64p, C.POINTER(C.c_void_p)]),
    "traj_next": (C.c_int, [C.c_void_p, C.POINTER(CassFrame)]),
    "traj_stats": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_double)]),
    "traj_close": (C.c_int, [C.c_void_p]),
    "load_next_frame": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_void_p), _i32p]),
    "get_stats": (C.c_int, [C.c_void_p, C.POINTER(CassStats)]),
    "build_molecule": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                 C.POINTER(C.c_uint64), _i32p, _f64p, _f64p, _f64p, _i32p]),
    "set_count_pairs": (C.c_int, [C.c_void_p, C.c_int32]),
    "set_mc_cluster": (C.c_int, [C.c_void_p, C.c_int32]),
    "set_widom_band": (C.c_int, [C.c_void_p, C.c_double]),
    "set_widom_cells": (C.c_int, [C.c_void_p, C.c_double]),
    "set_widom_autotune": (C.c_int, [C.c_void_p, C.c_int32]),
    "set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
}
OPTIONAL = {"get_stats", "set_count_pairs", "set_mc_cluster", "set_widom_band", "set_widom_cells", "set_widom_autotune", "set_stream", "mol_box_energy_noalloc", "system_gradient", "gcmc",
            "traj_open", "traj_next", "traj_stats", "traj_close", "load_next_frame"}


class CassError(RuntimeError):
    def __init__(self, fn: str, code: int, msg: str):
        super().__init__(f"{fn} failed with status {code}: {msg}")
        self.code = code


def bind(lib: C.CDLL, prefix: str) -> dict:
    """Bind every entry point of the header under `prefix`; returns name -> function."""
    out = {}
    for name, (res, args) in SIGNATURES.items():
        if name in OPTIONAL and not hasattr(lib, prefix + name):
            continue
        f = getattr(lib, prefix + name)
        f.restype = res
        f.argtypes = args
        out[name] = f
    return out


def _i32(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.int32).ravel())


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64).ravel())


def _p(a: np.ndarray | None):
    if a is None or a.size == 0:
        return None
    ct = _i32p if a.dtype == np.int32 else _f64p
    return a.ctypes.data_as(ct)


class Context:
    """An opened context of a library implementing the header (GPU or oracle)."""

    def __init__(self, fns: dict, nspecies: int, ntypes: int, nboxes: int,
                 max_molecules: Sequence[int], precision: int = PREC_FP64,
                 device: int = 0, max_kvectors: int = 100000):
        self._f = fns
        self._keep: list = []
        mm = _i32(max_molecules)
        cfg = CassConfig(nspecies, ntypes, nboxes, precision, device, max_kvectors, _p(mm))
        h = C.c_void_p()
        self._check("ctx_create", fns["ctx_create"](C.byref(cfg), C.byref(h)))
        self._h = h
        self.nspecies, self.ntypes, self.nboxes = nspecies, ntypes, nboxes
        self.max_molecules = list(max_molecules)
        self.precision = precision
        self.natoms: dict[int, int] = {}
        self.nfrag: dict[int, int] = {}

    # -- plumbing --------------------------------------------------------
    def _check(self, fn: str, rc: int) -> None:
        if rc != CASS_OK:
            msg = self._f["last_error"]()
            raise CassError(fn, rc, msg.decode() if msg else "")

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._f["ctx_destroy"](self._h)
            self._h = None

    def __del__(self):  # pragma: no cover - best effort
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- set-up ----------------------------------------------------------
    def set_nonbond_table(self, eps, sig, mie_n=None, mie_m=None) -> None:
        nt = self.ntypes
        e, s = _f64(eps), _f64(sig)
        n = _f64(mie_n if mie_n is not None else np.zeros(nt * nt))
        m = _f64(mie_m if mie_m is not None else np.zeros(nt * nt))
        self._check("set_nonbond_table", self._f["set_nonbond_table"](self._h, nt, _p(e), _p(s), _p(n), _p(m)))

    def set_species(self, is_: int, sp) -> None:
        """`sp` is a cassandra_gb300.system.Species."""
        arrs = sp.desc_arrays()
        d = CassSpeciesDesc()
        for k, v in arrs.items():
            if isinstance(v, np.ndarray):
                setattr(d, k, _p(v))
            else:
                setattr(d, k, v)
        self._check("set_species", self._f["set_species"](self._h, is_, C.byref(d)))
        self.natoms[is_] = sp.natoms
        self.nfrag[is_] = len(sp.fragments)

    def set_box(self, ibox: int, bx) -> None:
        d = CassBoxDesc()
        d.length[0], d.length[1], d.length[2] = bx.length
        d.vdw_style, d.vdw_sum_style = bx.vdw_style, bx.vdw_sum_style
        d.rcut_vdw, d.rcut_coul, d.rcut_cbmc, d.rcut_low = bx.rcut_vdw, bx.rcut_coul, bx.rcut_cbmc, bx.rcut_low
        d.ron_switch, d.roff_switch = bx.ron_switch, bx.roff_switch
        d.charge_style, d.charge_sum_style = bx.charge_style, bx.charge_sum_style
        d.ewald_tol, d.alpha_dsf, d.temperature = bx.ewald_tol, bx.alpha_dsf, bx.temperature
        self._check("set_box", self._f["set_box"](self._h, ibox, C.byref(d)))

    def set_molecules(self, im, is_, ibox, xyz) -> None:
        im, is_, ib, x = _i32(im), _i32(is_), _i32(ibox), _f64(xyz)
        self._check("set_molecules", self._f["set_molecules"](self._h, len(im), _p(im), _p(is_), _p(ib), _p(x)))

    def remove_molecule(self, im: int, is_: int) -> None:
        self._check("remove_molecule", self._f["remove_molecule"](self._h, im, is_))

    def get_molecule(self, im: int, is_: int) -> np.ndarray:
        out = np.zeros(3 * self.natoms[is_])
        self._check("get_molecule", self._f["get_molecule"](self._h, im, is_, _p(out)))
        return out.reshape(-1, 3)

    def set_cbmc_options(self, energy_table_res: int = 0, sector_overlap: bool = False,
                         rmin_u_max: float = 0.0) -> None:
        """CBMC_Info energy_table N, Cell_List_Overlap and Rcutoff_Low adaptive U of the input file."""
        o = CassCBMCOptions(energy_table_res, int(sector_overlap), rmin_u_max)
        self._check("set_cbmc_options", self._f["set_cbmc_options"](self._h, C.byref(o)))

    def volume_scale(self, ibox: int, new_length: float):
        """Scale cubic box ibox to edge new_length (COMs kept fractional); returns (energy dict, overlap)."""
        e = CassEnergy()
        ov = C.c_int32()
        self._check("volume_scale", self._f["volume_scale"](self._h, ibox, new_length, C.byref(e), C.byref(ov)))
        return e.as_dict(), bool(ov.value)

    def volume_restore(self, ibox: int) -> None:
        self._check("volume_restore", self._f["volume_restore"](self._h, ibox))

    def load_next_frame(self, trajectories) -> bool:
        """Load_Next_Frame: the next frame of trajectories[k] into box k+1; True at the end of a trajectory."""
        hs = (C.c_void_p * len(trajectories))(*[t._h for t in trajectories])
        end = np.zeros(1, dtype=np.int32)
        self._check("load_next_frame", self._f["load_next_frame"](self._h, len(trajectories), hs, _p(end)))
        return bool(end[0])

    def molecule_boxes(self, is_: int) -> np.ndarray:
        """Box of every molecule slot im = 1..max_molecules of species is_ (0: not live)."""
        out = np.zeros(self.max_molecules[is_ - 1], dtype=np.int32)
        self._check("get_molecule_boxes", self._f["get_molecule_boxes"](self._h, is_, len(out), _p(out)))
        return out

    # -- energies ------------------------------------------------------
    def mol_inter_energy(self, im: int, is_: int, cbmc: bool = False):
        ev, eq, ov = C.c_double(), C.c_double(), C.c_int32()
        self._check("mol_inter_energy", self._f["mol_inter_energy"](
            self._h, im, is_, int(cbmc), C.byref(ev), C.byref(eq), C.byref(ov)))
        return ev.value, eq.value, bool(ov.value)

    def mol_intra_energy(self, im: int, is_: int, cbmc: bool = False):
        a, b, c, ov = C.c_double(), C.c_double(), C.c_double(), C.c_int32()
        self._check("mol_intra_energy", self._f["mol_intra_energy"](
            self._h, im, is_, int(cbmc), C.byref(a), C.byref(b), C.byref(c), C.byref(ov)))
        return a.value, b.value, c.value, bool(ov.value)

    def system_total_energy(self, ibox: int, intra: bool = True):
        e, ov = CassEnergy(), C.c_int32()
        self._check("system_total_energy", self._f["system_total_energy"](
            self._h, ibox, int(intra), C.byref(e), C.byref(ov)))
        return e.as_dict(), bool(ov.value)

    def ewald_update(self, im: int, is_: int, ibox: int, move_flag: int) -> float:
        e = C.c_double()
        self._check("ewald_update", self._f["ewald_update"](self._h, im, is_, ibox, move_flag, C.byref(e)))
        return e.value

    def ewald_restore(self, im: int, is_: int, ibox: int) -> None:
        self._check("ewald_restore", self._f["ewald_restore"](self._h, im, is_, ibox))

    def ewald_widom(self, is_: int, ibox: int, xyz) -> np.ndarray:
        x = _f64(xyz)
        n = x.size // (3 * self.natoms[is_])
        out = np.zeros(n)
        self._check("ewald_widom", self._f["ewald_widom"](self._h, is_, ibox, n, _p(x), _p(out)))
        return out

    def stats(self) -> dict:
        st = CassStats()
        self._check("get_stats", self._f["get_stats"](self._h, C.byref(st)))
        return st.as_dict()

    def set_widom_autotune(self, on: bool) -> None:
        """Launch-shape autotuning of cass_widom_insert (on by default)."""
        self._check("set_widom_autotune", self._f["set_widom_autotune"](self._h, int(on)))

    def set_widom_cells(self, cells_per_cutoff: float) -> None:
        """Widom cell edge = rcut_cbmc / cells_per_cutoff (0: the precision's default)."""
        self._check("set_widom_cells", self._f["set_widom_cells"](self._h, float(cells_per_cutoff)))

    def set_widom_band(self, scale: float) -> None:
        """Scale (>= 1) of the FP32 cutoff bands whose pairs the mixed Widom pass decides in FP64."""
        self._check("set_widom_band", self._f["set_widom_band"](self._h, float(scale)))

    def set_mc_cluster(self, ctas: int) -> None:
        """CTAs per chain of mc_sweeps (0: chosen per call)."""
        self._check("set_mc_cluster", self._f["set_mc_cluster"](self._h, int(ctas)))

    def set_count_pairs(self, on: bool) -> None:
        self._check("set_count_pairs", self._f["set_count_pairs"](self._h, int(on)))

    def set_stream(self, stream_ptr: int | None) -> None:
        self._check("set_stream", self._f["set_stream"](self._h, C.c_void_p(stream_ptr) if stream_ptr else None))

    def gcmc(self, boxes: Sequence[int], nsteps: int, is_exchange: int, mu_kjmol, max_disp, max_rot, seed: int,
             kappa_ins: int = 12, kappa_dih: int = 12, cuts=(0.2, 0.4, 0.6, 0.8, 1.0)):
        """Grand-canonical chains, one per box; cuts are the cumulative probabilities of
        translate, rotate, insert, delete and regrow."""
        b = _i32(boxes)
        mu = np.ascontiguousarray(np.array(mu_kjmol, dtype=np.float64).reshape(len(b)))
        md = np.ascontiguousarray(np.array(max_disp, dtype=np.float64).reshape(len(b), -1))
        mr = np.ascontiguousarray(np.array(max_rot, dtype=np.float64).reshape(len(b), -1))
        prm = CassGCMCParams(nsteps, is_exchange, kappa_ins, kappa_dih, 0, *cuts)
        res = (CassGCMCResult * len(b))()
        self._check("gcmc", self._f["gcmc"](
            self._h, len(b), _p(b), C.byref(prm), mu.ctypes.data_as(_f64p), md.ctypes.data_as(_f64p),
            mr.ctypes.data_as(_f64p), C.c_uint64(seed & (2**64 - 1)), res))
        return [r.as_dict() for r in res]

    def mc_sweeps(self, boxes: Sequence[int], nsweeps: int, max_disp, max_rot, seed: int,
                  prob_translate: float = 1.0, steps_per_sweep: int = 0, nupdate: int = 0,
                  target_accept: float = 0.5):
        """NVT translate/rotate sweeps, one chain per box.  max_disp / max_rot:
        [nboxes][nspecies] arrays (adapted copies are returned)."""
        b = _i32(boxes)
        md = np.ascontiguousarray(np.array(max_disp, dtype=np.float64).reshape(len(b), -1))
        mr = np.ascontiguousarray(np.array(max_rot, dtype=np.float64).reshape(len(b), -1))
        prm = CassMCParams(nsweeps, steps_per_sweep, nupdate, prob_translate, target_accept)
        res = (CassMCResult * len(b))()
        self._check("mc_sweeps", self._f["mc_sweeps"](
            self._h, len(b), _p(b), C.byref(prm), md.ctypes.data_as(_f64p), mr.ctypes.data_as(_f64p),
            C.c_uint64(seed & (2**64 - 1)), res))
        return [r.as_dict() for r in res], md, mr

    def atom_intra_energies(self, ibox: int, is_: int, ia: int, xyz, exist=None, cbmc: bool = True):
        """Compute_Atom_Nonbond_Intra_Energy of atom ia (1-based) for trial configurations
        xyz [ntrial][natoms][3]; returns (e [ntrial][3] = intra vdW, intra qq, inter qq, overlap [ntrial])."""
        x = _f64(xyz)
        ntrial = x.size // (3 * self.natoms[is_])
        ex = _i32(exist) if exist is not None else None
        e = np.zeros(3 * ntrial)
        ov = np.zeros(ntrial, dtype=np.int32)
        self._check("atom_intra_energies", self._f["atom_intra_energies"](
            self._h, ibox, is_, ia, ntrial, _p(x), _p(ex), int(cbmc), _p(e), _p(ov)))
        return e.reshape(ntrial, 3), ov.astype(bool)

    def cbmc_trial_energies(self, ibox: int, is_: int, atoms, xyz, cbmc: bool = True, skip_im: int = 0):
        """Energies of trial positions [ntrial, nat, 3] of atoms (1-based) of species is_."""
        at = _i32(atoms)
        x = np.ascontiguousarray(np.asarray(xyz, dtype=np.float64).reshape(-1, len(at), 3))
        e = np.zeros(x.shape[0])
        ov = np.zeros(x.shape[0], dtype=np.int32)
        self._check("cbmc_trial_energies", self._f["cbmc_trial_energies"](
            self._h, ibox, is_, skip_im, len(at), _p(at), x.shape[0], x.ctypes.data_as(_f64p), int(cbmc),
            e.ctypes.data_as(_f64p), ov.ctypes.data_as(_i32p)))
        return e, ov.astype(bool)

    def build_molecule(self, im: int, is_: int, ibox: int, del_flag: bool, kappa_ins: int, kappa_dih: int,
                       rng_state):
        """Build_Molecule for molecule im of species is_ in box ibox from the lfsr258
        state rng_state (5 words).  Returns a dict with frag_order (1-based), ln_pseq,
        ln_pbias, xyz [natoms, 3], cbmc_overlap and the advanced rng_state."""
        st = np.array(rng_state, dtype=np.uint64).reshape(-1)
        if st.shape != (5,):
            raise ValueError("rng_state must hold 5 words")
        order = np.zeros(8, dtype=np.int32)
        lp, lb = C.c_double(0.0), C.c_double(0.0)
        xyz = np.zeros(3 * self.natoms[is_])
        ov = C.c_int32(0)
        self._check("build_molecule", self._f["build_molecule"](
            self._h, im, is_, ibox, int(bool(del_flag)), kappa_ins, kappa_dih,
            st.ctypes.data_as(C.POINTER(C.c_uint64)), order.ctypes.data_as(_i32p), C.byref(lp), C.byref(lb),
            xyz.ctypes.data_as(_f64p), C.byref(ov)))
        return {"frag_order": order[:self.nfrag.get(is_, 8)], "ln_pseq": lp.value, "ln_pbias": lb.value,
                "xyz": xyz.reshape(-1, 3), "cbmc_overlap": bool(ov.value), "rng_state": st}

    def system_gradient(self, ibox: int, n_atoms_box: int):
        """(energy dict, dU/dr [n_atoms_box, 3], dU/deps [nt, nt], dU/dsig [nt, nt], dU/dq [sum natoms])."""
        e = CassEnergy()
        g = np.zeros((n_atoms_box, 3))
        de = np.zeros((self.ntypes, self.ntypes))
        ds = np.zeros((self.ntypes, self.ntypes))
        dq = np.zeros(int(sum(self.natoms[k] for k in sorted(self.natoms))))
        self._check("system_gradient", self._f["system_gradient"](
            self._h, ibox, C.byref(e), g.ctypes.data_as(_f64p), de.ctypes.data_as(_f64p), ds.ctypes.data_as(_f64p),
            dq.ctypes.data_as(_f64p)))
        return e.as_dict(), g, de, ds, dq

    def widom_insert(self, is_: int, boxes: Sequence[int], n_insertions: int, kappa_ins: int,
                     kappa_dih: int, seed: int, trace: bool = False):
        b = _i32(boxes)
        res = (CassWidomResult * len(b))()
        tr = np.zeros(len(b) * n_insertions, dtype=TRACE_DTYPE) if trace else None
        self._check("widom_insert", self._f["widom_insert"](
            self._h, is_, len(b), _p(b), n_insertions, kappa_ins, kappa_dih, C.c_uint64(seed & (2**64 - 1)),
            res, tr.ctypes.data_as(C.c_void_p) if tr is not None else None))
        out = [{"widom_sum": r.widom_sum, "prefactor": r.prefactor, "n_insertions": r.n_insertions,
                "n_overlaps": r.n_overlaps, "n_trials": r.n_trials} for r in res]
        if trace:
            return out, tr.reshape(len(b), n_insertions)
        return out


class Trajectory:
    """A pregenerated trajectory of one box (.xyz + optional .H), read one frame
    ahead by the library's reader thread into pinned host memory."""

    def __init__(self, fns: dict, xyz_path: str, h_path: str | None, natoms: Sequence[int],
                 nmols: Sequence[int] | None = None, box=None):
        self._f = fns
        self.natoms = _i32(natoms)
        self._nm = _i32(nmols) if nmols is not None else None
        self._box = None
        if box is not None:
            b = np.asarray(box, dtype=np.float64)
            self._box = _f64(np.diag(b) if b.shape == (3,) else b.reshape(3, 3))
        h = C.c_void_p()
        rc = fns["traj_open"](xyz_path.encode(), h_path.encode() if h_path else None, len(self.natoms),
                              _p(self.natoms), _p(self._nm), _p(self._box), C.byref(h))
        if rc != CASS_OK:
            raise CassError("traj_open", rc, fns["last_error"]().decode(errors="replace"))
        self._h = h
        self.nspecies = len(self.natoms)

    def next(self) -> dict | None:
        """The next frame as arrays (copied), or None at the end of the trajectory."""
        fr = CassFrame()
        rc = self._f["traj_next"](self._h, C.byref(fr))
        if rc != CASS_OK:
            raise CassError("traj_next", rc, self._f["last_error"]().decode(errors="replace"))
        if fr.status != 0:
            return None
        xyz = np.ctypeslib.as_array(fr.xyz, shape=(fr.natoms * 3,)).reshape(-1, 3).copy() if fr.natoms else \
            np.zeros((0, 3))
        return {"index": fr.index, "box": np.array(fr.box[:]).reshape(3, 3),
                "nmols": np.ctypeslib.as_array(fr.nmols, shape=(self.nspecies,)).copy(), "xyz": xyz,
                "pinned": bool(fr.pinned)}

    def stats(self) -> dict:
        n, t = C.c_int64(), C.c_double()
        self._f["traj_stats"](self._h, C.byref(n), C.byref(t))
        return {"frames": n.value, "parse_s": t.value}

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._f["traj_close"](self._h)
            self._h = None

    def __del__(self):  # pragma: no cover - best effort
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
