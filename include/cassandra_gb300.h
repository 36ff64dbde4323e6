/*
 * cassandra_gb300.h -- C-ABI of the GB300 molecular-energy hot path.
 *
 * The entry points below replace Cassandra's Fortran energy / CBMC / Widom
 * routines (module procedures that read module-global state) with calls on an
 * opaque context that owns the device state.  Each declaration names the
 * reference routine it stands in for (path:line inside the Cassandra source
 * tree).  Conventions kept from the reference so that an ISO_C_BINDING shim can
 * forward its arguments unchanged:
 *   - molecule "locate" (im), species (is), box (ibox) and atom indices are
 *     1-based;
 *   - lengths in Angstrom, energies in Cassandra atomic units
 *     (amu A^2 / ps^2 = 10 J/mol), epsilon already multiplied by kboltz,
 *     charges in e;
 *   - "overlap" is a data flag (core overlap found), not an error.
 * Every function returns an int status: CASS_OK (0) or a negative CASS_E*
 * code.  No exception or process exit crosses this boundary.  Caller-owned
 * pointers are read or written only during the call.
 */
#ifndef CASSANDRA_GB300_H
#define CASSANDRA_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CASS_ABI_VERSION 2

/* status codes */
#define CASS_OK 0
#define CASS_EINVAL (-1)     /* bad argument (index out of range, NULL, ...) */
#define CASS_ECAPACITY (-2)  /* a size exceeds what the context was created for */
#define CASS_ECUDA (-3)      /* CUDA runtime error */
#define CASS_ETIMEDOUT (-4)  /* a bounded device-side wait gave up */
#define CASS_ESTATE (-5)     /* call order violated (e.g. Widom before totals) */
#define CASS_ENOMEM (-6)     /* device allocation failed */
#define CASS_EUNSUPPORTED (-7) /* option not implemented on this path */

/* arithmetic of the pair / trial energies */
#define CASS_PREC_FP64 0   /* every operation in FP64 (reference arithmetic) */
#define CASS_PREC_MIXED 1  /* FP32 pair math, FP64 accumulation and structure factors */

/* VDW_Style / vdw sum styles (global_variables.f90: vdw_* parameters) */
#define CASS_VDW_NONE 0
#define CASS_VDW_LJ 1
#define CASS_VDW_MIE 2
#define CASS_VDW_SUM_CUT 0
#define CASS_VDW_SUM_CUT_TAIL 1
#define CASS_VDW_SUM_CUT_SHIFT 2
#define CASS_VDW_SUM_MINIMUM 3
#define CASS_VDW_SUM_CUT_SWITCH 4
#define CASS_VDW_SUM_CHARMM 5
#define CASS_VDW_SUM_CUT_SHIFT_FORCE 6

/* Charge_Style */
#define CASS_CHARGE_NONE 0
#define CASS_CHARGE_COUL 1
#define CASS_QQ_EWALD 0
#define CASS_QQ_CUT 1
#define CASS_QQ_MINIMUM 2
#define CASS_QQ_DSF 3

/* move_flag of Update_System_Ewald_Reciprocal_Energy (global_variables.f90:240-244) */
#define CASS_MOVE_INSERTION 0
#define CASS_MOVE_DELETION 1
#define CASS_MOVE_TRANSLATION 2
#define CASS_MOVE_ROTATION 3
#define CASS_MOVE_INTRA 4

/* bond / angle kinds */
#define CASS_BONDED_FIXED 0
#define CASS_BONDED_HARMONIC 1

typedef struct cass_ctx cass_ctx;

/* Sizes the context is created for.  max_molecules[is-1] is the number of
 * molecule slots ("locates") of species is, as max_molecules in
 * global_variables.f90. */
typedef struct CassConfig {
  int32_t nspecies;
  int32_t ntypes;      /* number of nonbond atom types */
  int32_t nboxes;
  int32_t precision;   /* CASS_PREC_FP64 or CASS_PREC_MIXED */
  int32_t device;      /* CUDA device ordinal (ignored by the CPU oracle) */
  int32_t max_kvectors; /* capacity per box for Ewald k-vectors (maxk) */
  const int32_t* max_molecules; /* [nspecies] */
} CassConfig;

/* One species: the parts of Species_Class / Nonbond_Class / bonded lists /
 * Frag_Class (type_definitions.f90) that the hot path reads.  Atom and
 * fragment indices inside are 1-based as in the .mcf file. */
typedef struct CassSpeciesDesc {
  int32_t natoms;
  const int32_t* atom_type;          /* [natoms] 1-based nonbond type, 0 = no vdW */
  const double* charge;              /* [natoms] */
  const double* mass;                /* [natoms] */
  const double* vdw_intra_scale;     /* [natoms*natoms], (ia-1)*natoms+(ja-1) */
  const double* charge_intra_scale;  /* [natoms*natoms] */
  const int32_t* bonded;             /* [natoms*natoms] l_bonded: 1-2 bonded pair */
  int32_t nbonds;
  const int32_t* bond_atoms;         /* [2*nbonds] */
  const int32_t* bond_kind;          /* [nbonds] CASS_BONDED_* */
  const double* bond_param;          /* [2*nbonds] fixed:(l0,tol) harmonic:(k,l0) */
  int32_t nangles;
  const int32_t* angle_atoms;        /* [3*nangles] */
  const int32_t* angle_kind;         /* [nangles] */
  const double* angle_param;         /* [2*nangles] fixed:(theta0 deg,tol deg) harmonic:(k, theta0 rad) */
  int32_t ndihedrals;                /* Ryckaert-Bellemans form (OPLS converted on input) */
  const int32_t* dihedral_atoms;     /* [4*ndihedrals] */
  const double* dihedral_rb;         /* [6*ndihedrals] c0..c5 */
  int32_t nimpropers;                /* harmonic impropers */
  const int32_t* improper_atoms;     /* [4*nimpropers] */
  const double* improper_param;      /* [2*nimpropers] (k, phi0 rad) */
  /* CBMC fragments (Fragment_Info / Fragment_Connectivity / fragment libraries) */
  int32_t nfragments;
  const int32_t* frag_natoms;        /* [nfragments] */
  const int32_t* frag_atoms;         /* concatenated; the first atom of each fragment is its anchor */
  const int32_t* frag_nconnect;      /* [nfragments] */
  const int32_t* frag_connect;       /* concatenated connected fragment ids */
  const int32_t* frag_nconfig;       /* [nfragments] library size */
  const double* frag_library;        /* concatenated [nconfig][frag_natoms][3] */
  int32_t l_coul_cbmc;               /* species_list%L_Coul_CBMC */
} CassSpeciesDesc;

/* One simulation box (Box_Class + the per-box cutoffs and styles). */
typedef struct CassBoxDesc {
  double length[3];       /* orthorhombic edges (cubic when all equal), A */
  int32_t vdw_style;      /* CASS_VDW_* */
  int32_t vdw_sum_style;  /* CASS_VDW_SUM_* */
  double rcut_vdw, rcut_coul, rcut_cbmc, rcut_low;
  double ron_switch, roff_switch;  /* cut_switch only */
  int32_t charge_style;      /* CASS_CHARGE_* */
  int32_t charge_sum_style;  /* CASS_QQ_* */
  double ewald_tol;          /* alpha, h_cut derived as input_routines.f90:711-716 */
  double alpha_dsf;          /* <= 0: default of input_routines.f90:742-747 */
  double temperature;        /* K */
} CassBoxDesc;

/* energy(ibox) components (Energy_Class, type_definitions.f90) */
typedef struct CassEnergy {
  double total, intra, bond, angle, dihedral, improper;
  double intra_vdw, intra_q, inter, inter_vdw, inter_q;
  double lrc, reciprocal, self;
} CassEnergy;

/* Result of one Widom_Insert call (widom_insert.f90:22) for one box. */
typedef struct CassWidomResult {
  double widom_sum;      /* sum of widom_var times the prefactor (widom_insert.f90:538) */
  double prefactor;      /* V / ((N+1) Lambda^3), Lambda = 1 here (de Broglie applied by the host) */
  int64_t n_insertions;
  int64_t n_overlaps;
  int64_t n_trials;      /* CBMC trial energies evaluated (kappa_ins + (nfrag-1)*kappa_dih per insertion) */
} CassWidomResult;

/* Per-insertion record, optional output for parity checks. */
typedef struct CassWidomTrace {
  double widom_var;      /* exp(-beta(dE - dE_frag) - ln_pbias), 0 on overlap */
  double ln_pbias;
  double e_inter;        /* full-cutoff inter energy incl. periodic qq and reciprocal */
  double e_first_trial_sum; /* sum of the kappa_ins first-fragment trial energies (non-overlap) */
  double e_inter_abs;    /* sum of |pair energy| behind e_inter (real space): its conditioning scale */
  int32_t selected_trial;   /* first fragment trial chosen, 1-based, 0 if none */
  int32_t overlap;          /* 1 cbmc, 2 inter, 3 intra overlap */
} CassWidomTrace;

/* ---- context ---------------------------------------------------------- */
int cass_abi_version(void);
const char* cass_last_error(void);      /* thread-local text of the last failure */
int cass_ctx_create(const CassConfig* cfg, cass_ctx** out);
int cass_ctx_destroy(cass_ctx* ctx);

/* vdw_param1..4_table(ntypes,ntypes) after mixing (create_nonbond_table.f90:207-210);
 * row-major [(itype-1)*ntypes+(jtype-1)] */
int cass_set_nonbond_table(cass_ctx* ctx, int32_t ntypes, const double* eps,
                           const double* sig, const double* mie_n, const double* mie_m);
int cass_set_species(cass_ctx* ctx, int32_t is, const CassSpeciesDesc* desc);
/* Box set-up; for Ewald boxes also Ewald_Reciprocal_Lattice_Vector_Setup
 * (energy_routines.f90:2170-2323). */
int cass_set_box(cass_ctx* ctx, int32_t ibox, const CassBoxDesc* desc);
/* Writes atom_list coordinates of n molecules and marks them live in ibox[k]
 * (all atoms exist).  xyz holds natoms(is[k])*3 doubles per molecule. */
int cass_set_molecules(cass_ctx* ctx, int32_t n, const int32_t* im, const int32_t* is,
                       const int32_t* ibox, const double* xyz);
/* Marks molecule (im,is) not live (molecule_list%live = .FALSE.). */
int cass_remove_molecule(cass_ctx* ctx, int32_t im, int32_t is);
/* Reads back the coordinates of molecule (im,is). */
int cass_get_molecule(cass_ctx* ctx, int32_t im, int32_t is, double* xyz);
/* Box of molecules im = 1..n of species is (molecule_list(im,is)%which_box,
 * type_definitions.f90:151-153), 0 where the molecule is not live
 * (molecule_list%live = .FALSE.).  n <= max_molecules[is-1].  Lets the host
 * rebuild its locate / nmols arrays after cass_gcmc has inserted and deleted
 * molecules on the device. */
int cass_get_molecule_boxes(cass_ctx* ctx, int32_t is, int32_t n, int32_t* which_box);

/* ---- energy routines -------------------------------------------------- */
/* Compute_Molecule_Nonbond_Inter_Energy (energy_routines.f90:1088-1206);
 * cbmc_flag selects the rcut_cbmc cutoffs of Check_AtomPair_Cutoff. */
int cass_mol_inter_energy(cass_ctx* ctx, int32_t im, int32_t is, int32_t cbmc_flag,
                          double* e_inter_vdw, double* e_inter_qq, int32_t* overlap);
/* Compute_Molecule_Nonbond_Intra_Energy (energy_routines.f90:980-1085);
 * cbmc_flag selects rcut_cbmc and drops the charge pairs of a species whose
 * L_Coul_CBMC is set (:1062-1064), as the reference does. */
int cass_mol_intra_energy(cass_ctx* ctx, int32_t im, int32_t is, int32_t cbmc_flag,
                          double* e_intra_vdw, double* e_intra_qq, double* e_inter_qq,
                          int32_t* overlap);
/* Compute_System_Total_Energy (energy_routines.f90:2648-2953), including
 * Compute_System_Ewald_Reciprocal_Energy (:4111-4231), the self energy
 * (:2553-2601) and Compute_LR_Correction (:2956-3023).  Rebuilds the
 * structure factors cos_sum/sin_sum and cos_mol/sin_mol of the box. */
int cass_system_total_energy(cass_ctx* ctx, int32_t ibox, int32_t intra_flag,
                             CassEnergy* out, int32_t* overlap);
/* Update_System_Ewald_Reciprocal_Energy (energy_routines.f90:2326-2497).
 * Saves cos_sum/sin_sum (and the molecule's cos_mol/sin_mol) so that
 * cass_ewald_restore can revert a rejected move (move_translate.f90:296-305). */
int cass_ewald_update(cass_ctx* ctx, int32_t im, int32_t is, int32_t ibox,
                      int32_t move_flag, double* e_reciprocal);
int cass_ewald_restore(cass_ctx* ctx, int32_t im, int32_t is, int32_t ibox);
/* Update_System_Ewald_Reciprocal_Energy_Widom (energy_routines.f90:2500-2550),
 * batched: n test molecules of species is, coordinates [n][natoms][3];
 * writes n absolute reciprocal energies. */
int cass_ewald_widom(cass_ctx* ctx, int32_t is, int32_t ibox, int32_t n,
                     const double* xyz, double* e_reciprocal);

/* ---- volume moves ------------------------------------------------------ */
/* Volume_Change (move_volume.f90:24-679) for a cubic box, split at its
 * acceptance test so that the host keeps the random draw, the acceptance
 * rule (:440-446) and the counters.  cass_volume_scale gives every live
 * molecule of ibox the same fractional COM in the box of edge new_length and
 * moves it rigidly (:296-336), sets the new edge and its k-vectors
 * (Ewald_Reciprocal_Lattice_Vector_Setup, :374) and recomputes the system
 * energy on the device (Compute_System_Total_Energy, :426); energy(ibox) is
 * then the new energy.  The previous coordinates, box and energy are kept:
 * cass_volume_restore brings them back (Reset_Coords, :555-677) after a
 * rejection or an overlap.  The new half edge must not be shorter than the
 * cutoffs (CASS_EINVAL, as :283-292 abort). */
int cass_volume_scale(cass_ctx* ctx, int32_t ibox, double new_length, CassEnergy* energy, int32_t* overlap);
int cass_volume_restore(cass_ctx* ctx, int32_t ibox);

/* ---- CBMC options ----------------------------------------------------- */
/* Input-file options that change how CBMC trial energies and trial overlaps
 * are computed; they apply to the calls that follow.
 *   energy_table_res > 0 ("# CBMC_Info ... energy_table N",
 *     input_routines.f90:6041-6050): every CBMC trial energy
 *     (Compute_Molecule_Nonbond_Inter_Energy / _Widom with cbmc_flag,
 *     energy_routines.f90:1182-1191,1275-1278) becomes the atom-pair table
 *     lookup of Estimate_MoleculePair_Energy (energy_routines.f90:1528-1587)
 *     over the table of Create_Atompair_Nrg_table
 *     (atompair_nrg_table_routines.f90:149-261): N bins in r^2 from
 *     rcut_low^2 to the largest rcut_cbmc^2 of the context's boxes, each the
 *     vdW + real-space Coulomb pair energy at the bin's midpoint.  Used by
 *     cass_widom_insert, cass_cbmc_trial_energies, cass_mol_inter_energy with
 *     cbmc_flag and cass_gcmc.  0: off.
 *   sector_overlap != 0 ("# Cell_List_Overlap true"): in cass_widom_insert a
 *     trial atom closer than r_min(type pair) to a box atom makes its trial
 *     overlap (check_overlap, sector_routines.f90:160-233, called from
 *     fragment_growth.f90:475-488 and 1930-1949).
 *   rmin_u_max > 0 ("# Rcutoff_Low ... adaptive U", input_routines.f90:
 *     6941-7102): r_min^2 per type pair from U_max = U k T_max
 *     (create_nonbond_table.f90:285-303,396-418); 0: r_min = rcut_low.
 * The boxes must share one rcut_low (the reference has a single one) and
 * r_min may not exceed a box's rcut_cbmc (CASS_EUNSUPPORTED at use). */
typedef struct CassCBMCOptions {
  int32_t energy_table_res;
  int32_t sector_overlap;
  double rmin_u_max;
} CassCBMCOptions;
int cass_set_cbmc_options(cass_ctx* ctx, const CassCBMCOptions* opt);

/* ---- CBMC / Widom ----------------------------------------------------- */
/* Compute_Molecule_Nonbond_Inter_Energy_Widom (energy_routines.f90:1209-1364)
 * for a batch of CBMC trial positions, the energy call of every trial in
 * Build_Molecule (fragment_growth.f90:519-524) and Fragment_Placement
 * (:1967-2000): ntrial configurations of the nat atoms `atoms` (1-based atom
 * indices of species is) at xyz [ntrial][nat][3], each against the molecules of
 * box ibox except molecule (skip_im, is) when skip_im > 0 (the molecule being
 * deleted or regrown).  cbmc_flag selects rcut_cbmc and drops Coulomb unless
 * the species' L_Coul_CBMC is set.  e[k] = E_vdw + E_qq of trial k,
 * overlap[k] = 1 on a core overlap (e[k] = 0). */
/* Compute_Atom_Nonbond_Intra_Energy (energy_routines.f90:691-737) for a batch
 * of trial configurations of one molecule of species is, as Fragment_Placement
 * calls it for each new atom of a dihedral trial (fragment_growth.f90:
 * 1994-2000): atom ia (1-based) against the other existing atoms of the molecule
 * (exist[natoms] flags, NULL = every atom) with no periodic image, pairs whose
 * vdW and charge scale factors are both zero skipped, in the cutoffs of box
 * ibox (rcut_cbmc when cbmc_flag, as Check_AtomPair_Cutoff).  xyz holds
 * [ntrial][natoms][3]; e[3k..3k+2] = E_intra_vdw, E_intra_qq, E_inter_qq of trial
 * k (E_inter_qq: the -erf part of an Ewald sum); overlap[k] = 1 when a pair with
 * a nonzero vdW scale is closer than rcut_low (e = 0).  natoms <= 32. */
int cass_atom_intra_energies(cass_ctx* ctx, int32_t ibox, int32_t is, int32_t ia, int32_t ntrial,
                             const double* xyz, const int32_t* exist, int32_t cbmc_flag, double* e,
                             int32_t* overlap);
int cass_cbmc_trial_energies(cass_ctx* ctx, int32_t ibox, int32_t is, int32_t skip_im, int32_t nat,
                             const int32_t* atoms, int32_t ntrial, const double* xyz, int32_t cbmc_flag,
                             double* e, int32_t* overlap);

/* Widom_Insert (widom_insert.f90:22-594) with Build_Molecule /
 * Fragment_Placement (fragment_growth.f90:72-707,1449-2132) for every
 * insertion, batched over nboxes boxes in one launch.  Insertion k of box b
 * draws its random numbers from an lfsr258 stream seeded by (seed, b, k)
 * (the same stream in the CPU oracle).  Requires a prior
 * cass_system_total_energy or cass_load_next_frame of each listed box (the
 * long-range correction and the structure factors).  trace may be NULL; else it
 * receives nboxes*n_insertions records, box-major. */
int cass_widom_insert(cass_ctx* ctx, int32_t is, int32_t nboxes, const int32_t* ibox,
                      int64_t n_insertions, int32_t kappa_ins, int32_t kappa_dih,
                      uint64_t seed, CassWidomResult* out, CassWidomTrace* trace);

/* ---- Monte Carlo sweeps ------------------------------------------------ */
/* NVT Monte Carlo with translation (move_translate.f90:22-355) and rotation
 * (move_rotate.f90:22-536) moves, the kind chosen as nvtmc_driver.f90:107-134
 * does, one independent chain per listed box, all boxes in one launch.  Each
 * move evaluates Compute_Molecule_Nonbond_Inter_Energy before and after the
 * trial position, Update_System_Ewald_Reciprocal_Energy for charged species in
 * Ewald boxes, and accept_or_reject (accept_or_reject.f90:22-65); the
 * energy(ibox) bookkeeping and the structure factors stay FP64.  Box b draws
 * its random numbers from the lfsr258 stream seeded by (seed, b, 0); FP64
 * contexts use the reference's full uniforms and decisions, mixed contexts the
 * top 23 bits of the same numbers for the move choices and steps, FP32 pair
 * energies summed as compensated FP32 pairs, and (on one CTA, without k-space
 * work) an FP32 acceptance test, so their chains are their own.  Requires
 * a prior cass_system_total_energy of each listed box; afterwards the
 * molecules, the structure factors and the energy of each box are those after
 * its last move.  Replaces one translate/rotate host call sequence per move. */
typedef struct CassMCParams {
  int64_t nsweeps;
  int32_t steps_per_sweep;  /* moves per sweep; 0 = the number of molecules in the box */
  int32_t nupdate;          /* adapt the step sizes every nupdate trials of a move kind and
                               species, as in equilibration runs; 0 = never */
  double prob_translate;    /* cut_trans: a translation if rranf() <= prob_translate, else a rotation */
  double target_accept;     /* translation acceptance the adaptation aims at (max_disp scaled by
                               success_ratio / target_accept); 0.5 is the reference's rule */
} CassMCParams;

typedef struct CassMCResult {
  CassEnergy energy;        /* energy(ibox) after the last move */
  int64_t n_translate, n_translate_accepted;
  int64_t n_rotate, n_rotate_accepted;
  int64_t n_overlap;        /* trial positions rejected by the core-overlap test */
} CassMCResult;

/* max_disp, max_rot: [nboxes][nspecies] step sizes (A, rad) on input; the
 * adapted sizes on output. */
int cass_mc_sweeps(cass_ctx* ctx, int32_t nboxes, const int32_t* ibox, const CassMCParams* params,
                   double* max_disp, double* max_rot, uint64_t seed, CassMCResult* out);

/* ---- grand-canonical Monte Carlo ---------------------------------------- */
/* GCMC (gcmc_driver.f90:30-102) of one exchanged species in every listed box,
 * boxes advancing in lockstep in one launch: Translate, Rotate, CBMC Insertion
 * (move_insert.f90), CBMC Deletion (move_delete.f90) and CBMC regrowth
 * (Cut_N_Grow, move_regrow.f90 with Cut_Regrow, fragment_growth.f90:1118-1312),
 * chosen by the cumulative thresholds below.  Charged boxes need the Ewald
 * sum (CASS_EUNSUPPORTED otherwise): every move then carries the real-space
 * Coulomb terms, the reciprocal energy from the box's running structure
 * factors (left updated for the calls that follow) and, for insertions and
 * deletions, the molecule's self energy; they run in FP64 on one CTA per box
 * whatever the context's precision.  The molecule a move picks is the im-th live molecule of its
 * species in slot order; new molecules take the highest free slot of the
 * box's share of free slots (free slots of the exchanged species are dealt to
 * the listed boxes in turn, in ascending slot order).  Box b draws from the
 * lfsr258 stream seeded by (seed, b, 0).  Requires a prior
 * cass_system_total_energy of each listed box. */
typedef struct CassGCMCParams {
  int64_t nsteps;           /* moves per box */
  int32_t is_exchange;      /* the inserted / deleted species (1-based) */
  int32_t kappa_ins, kappa_dih;
  int32_t reserved;
  double cut_translate, cut_rotate, cut_insert, cut_delete, cut_regrow;  /* cumulative, <= 1 */
} CassGCMCParams;

typedef struct CassGCMCResult {
  CassEnergy energy;         /* energy(ibox) after the last move */
  int64_t n_translate, n_translate_accepted, n_rotate, n_rotate_accepted;
  int64_t n_insert, n_insert_accepted, n_delete, n_delete_accepted, n_regrow, n_regrow_accepted;
  int64_t n_molecules;       /* molecules of the exchanged species after the last move */
  double sum_n_molecules;    /* that count summed over all moves (for <N>) */
} CassGCMCResult;

/* mu [nboxes]: chemical potential of the exchanged species, kJ/mol (the .inp
 * Chemical_Potential_Info value); max_disp, max_rot [nboxes][nspecies] step
 * sizes (not adapted). */
int cass_gcmc(cass_ctx* ctx, int32_t nboxes, const int32_t* ibox, const CassGCMCParams* params,
              const double* mu, const double* max_disp, const double* max_rot, uint64_t seed,
              CassGCMCResult* out);

/* ---- CBMC growth of one molecule ---------------------------------------- */
/* Build_Molecule (fragment_growth.f90:72-707) for molecule im (1-based locate)
 * of species is in box ibox, for a host that keeps its own insertion,
 * deletion and regrowth moves (Build_Molecule's callers move_insert.f90:166,
 * move_delete.f90:175, widom_insert.f90:345): the first fragment, its library
 * conformation, Euler rotation and kappa_ins trial positions, then kappa_dih
 * dihedral trials per further fragment, every trial's energy against the
 * box's live molecules evaluated on the device.
 *   del_flag 0: the molecule is grown anew; it must not be live.  xyz [natoms][3]
 *     receives the grown coordinates, not folded into the box (the caller folds,
 *     as move_insert.f90 does); the molecule stays not live until the caller
 *     stores it with cass_set_molecules.
 *   del_flag 1: the molecule is live in ibox; trial 1 of every stage is its
 *     present configuration (the old-weight pass of a deletion or regrowth),
 *     and xyz receives that configuration.
 *   rng_state [5] in / out: the lfsr258 state the draws come from
 *     (random_generators.f90:95-122), advanced exactly as rranf would be.
 *   frag_order [nfrag] out: the fragments (1-based) in growth order.
 *   ln_pseq, ln_pbias out: as Build_Molecule returns them, before the kappa
 *     terms that the calling move adds.
 *   cbmc_overlap out: 1 when every trial of a stage overlapped (ln_pbias and xyz
 *     are then undefined).
 * Boxes as cass_gcmc takes them (LJ; charges only with the Ewald sum, where
 * the trial energies carry the intramolecular charges and, for species with
 * L_Coul_CBMC, the intermolecular real-space ones within rcut_cbmc).  FP64
 * contexts, and every context for charged boxes, grow in FP64 and reproduce
 * the reference's arithmetic; mixed contexts grow uncharged boxes in FP32. */
int cass_build_molecule(cass_ctx* ctx, int32_t im, int32_t is, int32_t ibox, int32_t del_flag, int32_t kappa_ins,
                        int32_t kappa_dih, uint64_t* rng_state, int32_t* frag_order, double* ln_pseq,
                        double* ln_pbias, double* xyz, int32_t* cbmc_overlap);

/* ---- configuration gradient (adjoint) ---------------------------------- */
/* The derivatives of the total energy of box ibox, as cass_system_total_energy
 * computes it (and returns it in *energy), for boxes with LJ (cut, cut_tail,
 * cut_shift, cut_switch, cut_shift_force or minimum image), Mie (cut or
 * cut_shift) or no vdW, and no charges or an Ewald sum: the bonded terms
 * (harmonic bonds and angles, Ryckaert-Bellemans dihedrals, harmonic
 * impropers; molecules with such terms up to 64 atoms), intramolecular nonbond
 * pairs with their scale factors, intermolecular vdW and real-space Ewald
 * pairs, the long-range correction, the reciprocal sum and the self energy.  The real-space term is
 * differentiated through the same A&S erfc.  No counterpart in the reference,
 * which has no derivatives; computed in FP64.
 *   dU_dr    [n][natoms(is)][3]: the live molecules of the box in species-major,
 *            locate order;
 *   dU_deps, dU_dsig [ntypes*ntypes]: derivatives with respect to the symmetric
 *            mixed pair parameters eps_tu = eps_ut and sigma_tu = sigma_ut
 *            (both entries hold the same value);
 *   dU_dq    [sum over species of natoms]: derivative with respect to the charge
 *            of each species atom, shared by all molecules of the species.
 * Any output may be NULL.  A configuration with a core overlap returns
 * CASS_ESTATE; other styles return CASS_EUNSUPPORTED. */
int cass_system_gradient(cass_ctx* ctx, int32_t ibox, CassEnergy* energy, double* dU_dr, double* dU_deps,
                         double* dU_dsig, double* dU_dq);

/* ---- allocation-free energy entry point -------------------------------- */
/* No counterpart in the reference.  For hosts that cannot call cudaMalloc in
 * their Monte Carlo move loop (device memory owned by another allocator, or an
 * allocation that would synchronize the device mid-loop): the energy of one
 * molecule against the atoms of a box, as cass_mol_inter_energy computes it,
 * with caller-provided DEVICE arrays and no allocation of any kind.  Its
 * scratch (16 KB: per-block partial sums, a block counter, an overlap flag) is
 * a static device array that every GPU loading this library keeps until exit.
 *   box_xyzq [n][4] x, y, z, charge; box_type [n] 1-based type (0: no vdW);
 *   box_mol [n] molecule ids, atoms with box_mol == skip_mol are skipped;
 *   query_xyzq [nq][4], query_type [nq]; eps/sig: host [ntypes*ntypes] tables.
 *   out: device [3] = E_vdw, E_qq, overlap (1.0/0.0; energies 0 on overlap).
 * Limits: n <= 262144, 1 <= nq <= 64, LJ or no vdW.  Larger sizes return
 * CASS_ECAPACITY; LJ CHARMM or minimum-image charges with a vdW sum other than
 * minimum image (where Check_MoleculePair_Cutoff decides) CASS_EUNSUPPORTED.  Runs on the current device, asynchronously on `stream`.
 * All calls on a device share the scratch: calls that overlap on the GPU race.
 * The first call on a device resolves the scratch address; make it before any
 * stream capture.  The address is kept for the life of the process: after a
 * cudaDeviceReset (or any teardown of the device's primary context) the module
 * is loaded anew and the kept address is stale, so do not call this function
 * again in a process that has reset its device. */
int cass_mol_box_energy_noalloc(const CassBoxDesc* box, int32_t ntypes, const double* eps, const double* sig,
                                const double* box_xyzq, const int32_t* box_type, const int32_t* box_mol,
                                int32_t n, const double* query_xyzq, const int32_t* query_type, int32_t nq,
                                int32_t skip_mol, int32_t cbmc_flag, int32_t l_coul_cbmc, int32_t precision,
                                double* out, void* stream);

/* ---- trajectory feed (the pregen driver's frames) ---------------------- */
/* A pregenerated trajectory of one box, as Load_Next_Frame reads it
 * (load_next_frame.f90:5-330; files opened by Get_Pregen_Info,
 * input_routines.f90:5717-5880).  The .xyz file holds, per frame, an atom-count
 * record, a comment record and one "element x y z" record per atom
 * (Read_xyz_frame, :307-328); the .H file holds, per frame, a volume record,
 * the three rows of the box matrix, one skipped record, the number of species
 * listed and one "species nmols" record each (Read_H_frame, :184-228).
 * Without an .H file the molecule counts `nmols` and the box `box` (3 x 3,
 * rows) are fixed for every frame (the "# Pregen_Info" entries).  A reader
 * thread parses the next frame into pinned host memory while the caller uses
 * the current one. */
typedef struct cass_traj cass_traj;
typedef struct CassFrame {
  int32_t status;         /* 0: a frame; 1: the end of the trajectory was reached */
  int32_t natoms;         /* atoms of the frame (natoms_to_read) */
  int64_t index;          /* 0-based frame number */
  double box[9];          /* box_list%length, row-major (Read_H_frame) */
  const int32_t* nmols;   /* [nspecies] molecules of each species (nmols_to_read) */
  const double* xyz;      /* [natoms][3] species-major, in pinned host memory;
                             valid until the next cass_traj_next or cass_load_next_frame */
  int32_t pinned;         /* 1 when xyz is page-locked */
  int32_t reserved;
} CassFrame;
/* natoms[is-1] = atoms per molecule of species is.  h_path may be NULL (then
 * nmols and box are required).  Fails with CASS_EINVAL when a file cannot be
 * opened. */
int cass_traj_open(const char* xyz_path, const char* h_path, int32_t nspecies, const int32_t* natoms,
                   const int32_t* nmols, const double* box, cass_traj** out);
/* The next frame (status 1 at the end).  A malformed record fails with
 * CASS_EINVAL and the record's line number in cass_last_error(). */
int cass_traj_next(cass_traj* t, CassFrame* frame);
/* Frames parsed and the reader thread's parse time, for measurement. */
int cass_traj_stats(cass_traj* t, int64_t* frames, double* parse_seconds);
int cass_traj_close(cass_traj* t);
/* Load_Next_Frame (load_next_frame.f90:5-330): takes the next frame of
 * traj[k] for box k+1 (nboxes = the context's box count); every molecule is
 * first made not live; the molecules of box ibox are locates
 * base+1..base+nmols_to_read of each species, base = those of the same species
 * in lower boxes (:239-246); each molecule's COM is folded into the box with
 * Apply_PBC_Anint and its atoms shifted rigidly (:257-283); a box whose
 * matrix changed gets the new edges and k-vectors (Set_Frame_Box, :57-102;
 * orthorhombic matrices only).  The packed coordinates are uploaded from
 * pinned memory.  As at the end of Set_Frame_Coords (:290-301), each box gets
 * its long-range correction and, with Ewald, its structure factors and
 * reciprocal energy: enough for cass_widom_insert.  The other energy
 * components come from cass_system_total_energy (pregen_driver.f90:187),
 * which the MC entry points require.  On the end of any trajectory,
 * *end_reached = 1 and the context is unchanged. */
int cass_load_next_frame(cass_ctx* ctx, int32_t nboxes, cass_traj* const* traj, int32_t* end_reached);

/* ---- run-time extensions (no counterpart in the reference) ------------- */
/* Counters of a context, for measurement.  Times are CUDA-event durations on
 * the context's stream of the most recent cass_widom_insert call. */
typedef struct CassStats {
  double widom_ms;          /* whole call: cell lists + CBMC kernel + reciprocal + reduction */
  double widom_kernel_ms;   /* the CBMC Widom kernel alone */
  int64_t kernel_launches;  /* kernels launched by this context since creation */
  int64_t h2d_bytes, d2h_bytes;  /* host<->device bytes copied since creation */
  int64_t widom_pairs_visited;   /* box atoms visited by the last Widom call (count_pairs mode) */
  int64_t widom_pairs_in_cutoff; /* of which inside a cutoff */
  int32_t widom_grid_x, widom_grid_y, widom_block;
  int32_t widom_smem_bytes;
  double mc_ms;             /* the most recent cass_mc_sweeps or cass_gcmc: its kernel */
  int64_t mc_moves;         /* moves it ran, all boxes */
  int32_t gcmc_cluster;     /* CTAs per box (a thread-block cluster) of the most recent cass_gcmc or cass_mc_sweeps */
  int32_t widom_fixups;     /* mixed precision: insertions of the last Widom call whose full-cutoff pass met a
                               pair within FP32 rounding of a cutoff and was redone from FP64 coordinates */
} CassStats;
int cass_get_stats(cass_ctx* ctx, CassStats* out);
/* count_pairs != 0 makes the Widom kernel count visited / in-cutoff pairs. */
int cass_set_count_pairs(cass_ctx* ctx, int32_t count_pairs);
/* Edge of the cells of the Widom cell lists, as a divisor of rcut_cbmc: the
 * edge is rcut_cbmc / cells_per_cutoff (0 restores the default of the
 * context's precision).  Results do not depend on it beyond summation order. */
int cass_set_widom_cells(cass_ctx* ctx, double cells_per_cutoff);
/* on != 0 (the default): the first cass_widom_insert of each batch signature
 * times a few launch shapes (cell edge, CTAs per resident slot) on a sample of
 * insertions and the context keeps the fastest; a cell edge set with
 * cass_set_widom_cells disables it.  Results do not depend on the shape beyond
 * summation order. */
int cass_set_widom_autotune(cass_ctx* ctx, int32_t on);
/* CTAs (a thread-block cluster) that run each chain of cass_mc_sweeps: 0 (the
 * default) chooses per call -- several when few chains leave SMs idle, so a
 * single chain's pair and k-vector loops spread over up to 8 multiprocessors;
 * 1..8 fixes it (boxes kept in global memory always run on one CTA).  Results
 * do not depend on it beyond summation order.  cass_get_stats reports the
 * choice in gcmc_cluster. */
int cass_set_mc_cluster(cass_ctx* ctx, int32_t ctas);
/* Mixed precision: the full-cutoff pass of each Widom insertion notes the pairs
 * whose FP32 r^2 lies within a band about rcut_low^2, the vdW or the Coulomb
 * cutoff^2 (the bound of the FP32 rounding of the test and box coordinates),
 * and those pairs are decided again in FP64 from the molecule regrown in FP64,
 * so that every cutoff and overlap decision is the FP64 one.  scale (>= 1,
 * default 1) widens the bands: more pairs are decided in FP64, the results do
 * not change beyond rounding.  cass_get_stats reports the insertions
 * corrected in widom_fixups. */
int cass_set_widom_band(cass_ctx* ctx, double scale);
/* Runs the context's work on a caller-owned cudaStream_t (NULL: its own). */
int cass_set_stream(cass_ctx* ctx, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* CASSANDRA_GB300_H */
