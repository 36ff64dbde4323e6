// cass_ctx.h -- host-side state of a cass_ctx (internal to libcassgpu.so).
//
// The context replaces the module-global state of Cassandra (atom_list,
// molecule_list, box_list, cos_sum/sin_sum, cos_mol/sin_mol, ...).  The FP64
// coordinates are mirrored on the host (the caller's MC loop writes them); the
// device holds per-box packed atom arrays, cell-sorted copies for the Widom
// kernel, k-vectors and the FP64 structure factors.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <utility>
#include <vector>

#include "cass_molecule.cuh"

namespace cassgpu {

int set_error(int code, const std::string& msg);
int cuda_error(cudaError_t e, const char* where);

#define CASS_CUDA(call)                                     \
  do {                                                      \
    cudaError_t _e = (call);                                \
    if (_e != cudaSuccess) return cuda_error(_e, #call);    \
  } while (0)

// Owning device buffer.
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  DevBuf(DevBuf&& o) noexcept : p(o.p), bytes(o.bytes) {
    o.p = nullptr;
    o.bytes = 0;
  }
  DevBuf& operator=(DevBuf&& o) noexcept {
    if (this != &o) {
      release();
      p = o.p;
      bytes = o.bytes;
      o.p = nullptr;
      o.bytes = 0;
    }
    return *this;
  }
  ~DevBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  // grows (never shrinks); returns a CASS status
  int reserve(size_t n) {
    if (n <= bytes) return CASS_OK;
    release();
    if (cudaMalloc(&p, n) != cudaSuccess) {
      p = nullptr;
      return set_error(CASS_ENOMEM, "device allocation failed");
    }
    bytes = n;
    return CASS_OK;
  }
  template <class T>
  T* as() const {
    return static_cast<T*>(p);
  }
};

// Owning page-locked host buffer (cudaHostAlloc): the source of
// asynchronous uploads.
struct PinnedBuf {
  void* p = nullptr;
  size_t bytes = 0;
  PinnedBuf() = default;
  PinnedBuf(const PinnedBuf&) = delete;
  PinnedBuf& operator=(const PinnedBuf&) = delete;
  ~PinnedBuf() { release(); }
  void release() {
    if (p) cudaFreeHost(p);
    p = nullptr;
    bytes = 0;
  }
  // grows (never shrinks, contents not kept); returns a CASS status
  int reserve(size_t n) {
    if (n <= bytes) return CASS_OK;
    release();
    if (cudaHostAlloc(&p, n, cudaHostAllocDefault) != cudaSuccess) {
      p = nullptr;
      return set_error(CASS_ENOMEM, "pinned host allocation failed");
    }
    bytes = n;
    return CASS_OK;
  }
  template <class T>
  T* as() const {
    return static_cast<T*>(p);
  }
};

struct SpeciesH {
  bool defined = false;
  int natoms = 0;
  std::vector<int> type;  // 0-based, -1 = none
  std::vector<double> q, mass, vscale, qscale;
  std::vector<int> bonded;
  std::vector<int> bond_atoms, bond_kind;
  std::vector<double> bond_param;
  std::vector<int> angle_atoms, angle_kind;
  std::vector<double> angle_param;
  std::vector<int> dih_atoms;
  std::vector<double> dih_rb;
  std::vector<int> imp_atoms;
  std::vector<double> imp_param;
  int nfrag = 0;
  std::vector<std::vector<int>> frag_atoms, frag_connect;
  std::vector<int> frag_nconfig;
  std::vector<double> prob_ins, cum_prob_ins;
  std::vector<double> library;  // all fragments concatenated
  std::vector<int> lib_off;     // start (in doubles) of each fragment's library
  bool l_coul_cbmc = false, has_charge = false;
  DevBuf d_library;
  DevBuf d_library_f;  // FP32 copy of `library`
  // host FP64 coordinates of every molecule slot [max_mol][natoms][3]
  std::vector<double> pos;
};

struct BoxH {
  bool defined = false;
  CassBoxDesc desc{};
  BoxDev dev{};
  double rcut_max = 0, rcut3 = 0, rcut9 = 0;
  std::vector<double> kvec;  // [nvecs][4] = hx, hy, hz, Cn
  int nvecs = 0;
  bool energy_valid = false;
  // energy.lrc / energy.reciprocal and the structure factors are current
  // (a frame load sets them up without the other components)
  bool frame_ready = false;
  CassEnergy energy{};
  // packed atoms of the live molecules of this box, molecule-contiguous
  bool pack_dirty = true;
  int npacked = 0, npacked_mols = 0;
  std::vector<int> pk_mol;      // packed molecule -> molecule slot
  std::vector<int> pk_mol_off;  // packed molecule -> first packed atom
  DevBuf d_p64, d_p32, d_meta, d_molinfo;
  DevBuf d_kvec, d_cos_sum, d_sin_sum, d_cos_old, d_sin_old;
  // rows of the k-vector list: (first k, count) of runs of equal (ny, nz) with
  // nx rising by one, for the phase recurrence of the FP64 rebuild
  std::vector<int2> krow;
  DevBuf d_krow;
  bool cell_dirty = true;
  // Check_MoleculePair_Cutoff decides which molecule pairs interact when a
  // style has no atom cutoff (LJ CHARMM, minimum-image charges) and the vdW sum
  // is not minimum image: then each packed atom carries its molecule's COM and
  // max_dcom (x, y, z, max_dcom), rebuilt with the packed arrays
  bool comcut = false;
  DevBuf d_com;
  // the state cass_volume_scale keeps for cass_volume_restore
  bool vol_saved = false;
  CassBoxDesc vol_desc{};
  CassEnergy vol_energy{};
  std::vector<int> vol_im, vol_is;
  std::vector<double> vol_xyz;
};

// in-place coordinate update of one packed atom (charge and type stay)
struct PatchRec {
  double x, y, z;
  int box, atom;
};

struct cass_ctx_impl {
  int device = 0, precision = CASS_PREC_FP64;
  cudaStream_t stream = nullptr, own_stream = nullptr;
  CassStats stats{};
  int count_pairs = 0;
  double widom_cells = 0.0;  // cells per rcut_cbmc in the Widom cell lists (0: default)
  int widom_waves = 0;       // CTAs per resident slot of the FP32 Widom launch (0: default)
  int widom_threads = 0;     // threads per CTA of the FP32 Widom launch, 512 or 256 (0: 512)
  double widom_band = 1.0;   // scale of the FP32 cutoff bands of the mixed Widom full-cutoff pass
  int mc_cluster = 0;        // CTAs per chain of cass_mc_sweeps (0: chosen per call)
  // launch shapes the Widom autotuner chose, per batch signature: (cells per cutoff, waves)
  bool widom_autotune = true;
  struct WidomShape {
    double cells;
    int waves, threads;
  };
  std::vector<std::pair<std::vector<long long>, WidomShape>> widom_tuned;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  int nspecies = 0, ntypes = 0, nboxes = 0, max_kvec = 100000;
  std::vector<int> max_mol, mol_base;
  int nmol_slots = 0;
  std::vector<SpeciesH> sp;
  std::vector<BoxH> box;
  PairTable pt{};
  std::vector<double> pt_sig;  // mixed sigma per type pair, as given
  bool pt_set = false;
  std::vector<int> mol_box;  // -1 = not live
  std::vector<int> slot_sp;  // species (0-based) of each molecule slot
  // live molecule slots of each box in slot order (species-major, locate
  // order), rebuilt from mol_box when membership changed
  std::vector<std::vector<int>> box_members;
  bool members_dirty = true;
  std::vector<int> pk_index;  // slot -> packed molecule index in its box (valid while the box is packed)
  // staged in-place coordinate updates of set_molecules
  std::vector<PatchRec> h_patch;
  DevBuf d_patch;
  DevBuf d_mc;    // Monte Carlo sweep descriptors, outputs and scratch
  DevBuf d_mc_box;  // box layouts of MC sweeps too large for shared memory
  DevBuf d_grad;  // adjoint outputs and per-atom parameter derivatives
  DevBuf d_trial; // CBMC trial positions and their energies
  DevBuf d_gc;    // grand-canonical descriptors, records and outputs
  // structure factors of molecules: [nmol_slots][max nvecs] x2, allocated on first use
  DevBuf d_cos_mol, d_sin_mol, d_cos_mol_old, d_sin_mol_old;
  int cos_mol_stride = 0;
  // device species tables (SpeciesPools)
  DevBuf d_sp_hdr, d_sp_ip, d_sp_dp;
  SpeciesPools pools{};
  bool pools_dirty = true;
  // reduction scratch
  DevBuf d_partial, d_counter, d_result, d_query;
  std::vector<double> h_result;
  // cell-sorted arrays of the boxes of the last Widom batch
  DevBuf d_c64, d_c32, d_cq32, d_cell_start, d_cell_count, d_cell_of, d_boxdev, d_widom_out, d_widom_xyz,
      d_trace, d_box_sums, d_widom_fix;
  std::vector<int> widom_boxes;
  // CBMC options and the tables they derive (energy table per box, r_min^2)
  CassCBMCOptions cbmc_opt{};
  bool cbmc_dirty = true;
  DevBuf d_cbmc_tab;
  // pinned staging of the packed-box uploads
  PinnedBuf h_pack;
  DevBuf d_stage;  // device copy of a frame load's staging area
};

// builds the CBMC-option tables if needed and points each box's BoxDev at them
int ensure_cbmc(cass_ctx_impl* c);

// copies that keep the byte counters of CassStats
cudaError_t h2d(cass_ctx_impl* c, void* dst, const void* src, size_t n);
cudaError_t d2h(cass_ctx_impl* c, void* dst, const void* src, size_t n);
inline void count_launch(cass_ctx_impl* c, int n = 1) { c->stats.kernel_launches += n; }

}  // namespace cassgpu

struct cass_ctx : public cassgpu::cass_ctx_impl {};
