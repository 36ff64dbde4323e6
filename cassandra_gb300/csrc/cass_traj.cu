// cass_traj.cu -- the pregen driver's trajectory feed.
//
// Load_Next_Frame (load_next_frame.f90:5-330) reads, for every box, one frame
// of an .H box file and of an .xyz coordinate file, makes the frame's
// molecules live in the box with their COMs folded into it, and sets up the
// box (edges, k-vectors) when its size changed.  Here the text parsing runs on
// a reader thread per trajectory, one frame ahead of the caller, into two
// page-locked frame buffers, so that the parse of frame k+1 overlaps the
// device work on frame k (the Widom insertions and the energy rebuild).  The
// frame's coordinates then go to the context's host copy and the packed
// atoms are uploaded from pinned staging.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "cass_ctx.h"

namespace cassgpu {
void invalidate_ext(cass_ctx* c, int ibox);
void set_mol_box_ext(cass_ctx* c, int slot, int ibox);
int frame_setup_ext(cass_ctx* c);
}  // namespace cassgpu

using namespace cassgpu;

namespace {

// One record-oriented text stream with Fortran list-directed reading rules:
// a READ with no items consumes one record; a READ of values starts at the
// next record, continues over records until it has all its values and drops
// what is left of its last record.
struct RecordFile {
  FILE* f = nullptr;
  long line = 0;
  std::string buf;
  bool next_record(std::string& out) {
    out.clear();
    int ch;
    bool any = false;
    while ((ch = fgetc(f)) != EOF) {
      any = true;
      if (ch == '\n') break;
      out.push_back((char)ch);
    }
    if (!any) return false;
    if (!out.empty() && out.back() == '\r') out.pop_back();
    ++line;
    return true;
  }
};

// splits on blanks and commas (list-directed separators)
void tokens(const std::string& s, std::vector<std::string>& out) {
  out.clear();
  size_t i = 0;
  while (i < s.size()) {
    while (i < s.size() && (s[i] == ' ' || s[i] == '\t' || s[i] == ',')) ++i;
    size_t j = i;
    while (j < s.size() && !(s[j] == ' ' || s[j] == '\t' || s[j] == ',')) ++j;
    if (j > i) out.emplace_back(s.substr(i, j - i));
    i = j;
  }
}

// a Fortran real constant: D or Q exponents are read as E
bool parse_real(const std::string& t, double* v) {
  std::string u = t;
  for (char& ch : u)
    if (ch == 'd' || ch == 'D' || ch == 'q' || ch == 'Q') ch = 'E';
  char* end = nullptr;
  *v = std::strtod(u.c_str(), &end);
  return end && *end == '\0' && end != u.c_str();
}

bool parse_int(const std::string& t, long* v) {
  char* end = nullptr;
  *v = std::strtol(t.c_str(), &end, 10);
  return end && *end == '\0' && end != t.c_str();
}

struct Frame {
  int status = 0;  // 0 frame, 1 end, -1 error
  std::string err;
  int64_t index = 0;
  double H[9] = {0};
  std::vector<int32_t> nmols;
  int natoms = 0;
  PinnedBuf pin;                // page-locked coordinates
  std::vector<double> pageable; // used only where page-locked memory cannot be had
  double* xyz = nullptr;
  size_t cap = 0;
  bool pinned = false;
  bool reserve(size_t ndouble) {
    if (ndouble <= cap) return true;
    size_t n = std::max(ndouble, cap + cap / 2);
    if (pin.reserve(n * sizeof(double)) == CASS_OK) {
      pageable.clear();
      xyz = pin.as<double>();
      pinned = true;
    } else {
      pageable.assign(n, 0.0);
      xyz = pageable.data();
      pinned = false;
    }
    cap = n;
    return true;
  }
};

}  // namespace

// Readers parse at most (hardware threads - 1) frames at a time, so that the
// thread loading a frame (folding and packing its molecules) keeps a core:
// with one reader per box and all of them busy it ran 2-4x slower.
struct ParseSlots {
  std::mutex mu;
  std::condition_variable cv;
  int free_slots = std::max(1, (int)std::thread::hardware_concurrency() - 1);
  void acquire() {
    std::unique_lock<std::mutex> lk(mu);
    cv.wait(lk, [&] { return free_slots > 0; });
    --free_slots;
  }
  void release() {
    {
      std::lock_guard<std::mutex> lk(mu);
      ++free_slots;
    }
    cv.notify_one();
  }
};
ParseSlots& parse_slots() {
  static ParseSlots p;
  return p;
}

struct cass_traj {
  RecordFile fx, fh;
  bool has_h = false;
  int nspecies = 0;
  std::vector<int32_t> natoms_sp, nmols_fixed;
  double H_fixed[9] = {0};
  Frame slot[2];
  int state[2] = {0, 0};  // 0 free, 1 ready (filled by the reader), 2 held by the caller
  int fill = 0, take = 0;
  bool stop = false, finished = false;
  std::mutex mu;
  std::condition_variable cv;
  std::thread th;
  int64_t frames = 0;
  double parse_s = 0.0;

  // Read_H_frame (load_next_frame.f90:184-228) and Read_xyz_frame (:307-328)
  void read_frame(Frame& F) {
    F.status = 0;
    F.err.clear();
    F.nmols.assign(nspecies, 0);
    std::string rec;
    std::vector<std::string> tk;
    auto fail = [&](RecordFile& r, const char* what) {
      F.status = -1;
      F.err = std::string(what) + " at line " + std::to_string(r.line);
    };
    // values over as many records as needed (blank records are skipped)
    auto values = [&](RecordFile& r, int n, std::vector<std::string>& out) -> bool {
      out.clear();
      std::vector<std::string> t;
      while ((int)out.size() < n) {
        if (!r.next_record(rec)) return false;
        tokens(rec, t);
        for (auto& x : t)
          if ((int)out.size() < n) out.push_back(x);
      }
      return true;
    };
    if (has_h) {
      if (!fh.next_record(rec)) {  // the volume record; end of file ends the run
        F.status = 1;
        return;
      }
      for (int i = 0; i < 3; ++i) {
        if (!values(fh, 3, tk)) return fail(fh, "H file: incomplete box matrix");
        for (int j = 0; j < 3; ++j)
          if (!parse_real(tk[j], &F.H[3 * i + j])) return fail(fh, "H file: bad box matrix entry");
      }
      if (!fh.next_record(rec)) return fail(fh, "H file: record after the box matrix missing");
      long nsp = 0;
      if (!values(fh, 1, tk) || !parse_int(tk[0], &nsp) || nsp < 0 || nsp > nspecies)
        return fail(fh, "H file: bad number of species");
      for (long i = 0; i < nsp; ++i) {
        long is = 0, nm = 0;
        if (!values(fh, 2, tk) || !parse_int(tk[0], &is) || !parse_int(tk[1], &nm) || is < 1 || is > nspecies ||
            nm < 0)
          return fail(fh, "H file: bad species / molecule-count record");
        F.nmols[is - 1] = (int32_t)nm;
      }
    } else {
      memcpy(F.H, H_fixed, sizeof(F.H));
      F.nmols = nmols_fixed;
    }
    size_t na = 0;
    for (int is = 0; is < nspecies; ++is) na += (size_t)natoms_sp[is] * (size_t)F.nmols[is];
    if (na > (size_t)1 << 30) return fail(fh, "frame too large");
    F.natoms = (int)na;
    F.reserve(std::max<size_t>(3 * na, 3));
    if (!fx.next_record(rec)) {  // the atom-count record; end of file ends the run
      F.status = 1;
      return;
    }
    if (!fx.next_record(rec)) return fail(fx, "xyz file: comment record missing");
    for (size_t i = 0; i < na; ++i) {
      if (!values(fx, 4, tk)) return fail(fx, "xyz file: frame ends early");
      for (int k = 0; k < 3; ++k)
        if (!parse_real(tk[1 + k], &F.xyz[3 * i + k])) return fail(fx, "xyz file: bad coordinate");
    }
  }

  void run() {
    for (;;) {
      int k;
      {
        std::unique_lock<std::mutex> lk(mu);
        cv.wait(lk, [&] { return stop || state[fill] == 0; });
        if (stop) return;
        k = fill;
      }
      parse_slots().acquire();
      auto t0 = std::chrono::steady_clock::now();
      Frame& F = slot[k];
      read_frame(F);
      F.index = frames;
      auto t1 = std::chrono::steady_clock::now();
      parse_slots().release();
      {
        std::lock_guard<std::mutex> lk(mu);
        parse_s += std::chrono::duration<double>(t1 - t0).count();
        if (F.status == 0) ++frames;
        state[k] = 1;
        fill ^= 1;
        if (F.status != 0) finished = true;
      }
      cv.notify_all();
      if (F.status != 0) return;  // the end or an error: nothing more to read
    }
  }

  // the frame taken last goes back to the reader (its data is no longer read)
  void release_taken() {
    std::lock_guard<std::mutex> lk(mu);
    const int prev = take ^ 1;
    if (state[prev] == 2) {
      state[prev] = 0;
      cv.notify_all();
    }
  }

  // the next frame; the previously taken one is released to the reader
  Frame* next() {
    std::unique_lock<std::mutex> lk(mu);
    const int prev = take ^ 1;
    if (state[prev] == 2) {
      state[prev] = 0;
      cv.notify_all();
    }
    cv.wait(lk, [&] { return state[take] == 1; });
    Frame* F = &slot[take];
    if (F->status != 0) return F;  // stays ready: every later call sees the end too
    state[take] = 2;
    take ^= 1;
    return F;
  }

  ~cass_traj() {
    {
      std::lock_guard<std::mutex> lk(mu);
      stop = true;
    }
    cv.notify_all();
    if (th.joinable()) th.join();
    if (fx.f) fclose(fx.f);
    if (fh.f) fclose(fh.f);
  }
};

extern "C" {

int cass_traj_open(const char* xyz_path, const char* h_path, int32_t nspecies, const int32_t* natoms,
                   const int32_t* nmols, const double* box, cass_traj** out) {
  if (!out) return set_error(CASS_EINVAL, "NULL output");
  *out = nullptr;
  if (!xyz_path || nspecies < 1 || !natoms) return set_error(CASS_EINVAL, "bad trajectory arguments");
  if (!h_path && (!nmols || !box)) return set_error(CASS_EINVAL, "without an H file, nmols and box are required");
  for (int is = 0; is < nspecies; ++is)
    if (natoms[is] < 1 || (!h_path && nmols[is] < 0)) return set_error(CASS_EINVAL, "bad atom or molecule count");
  cass_traj* t = new cass_traj();
  t->nspecies = nspecies;
  t->natoms_sp.assign(natoms, natoms + nspecies);
  t->fx.f = fopen(xyz_path, "r");
  if (!t->fx.f) {
    delete t;
    return set_error(CASS_EINVAL, std::string("cannot open xyz file ") + xyz_path);
  }
  if (h_path) {
    t->has_h = true;
    t->fh.f = fopen(h_path, "r");
    if (!t->fh.f) {
      delete t;
      return set_error(CASS_EINVAL, std::string("cannot open H file ") + h_path);
    }
  } else {
    t->nmols_fixed.assign(nmols, nmols + nspecies);
    memcpy(t->H_fixed, box, sizeof(t->H_fixed));
  }
  t->th = std::thread([t] { t->run(); });
  *out = t;
  return CASS_OK;
}

int cass_traj_next(cass_traj* t, CassFrame* fr) {
  if (!t || !fr) return set_error(CASS_EINVAL, "NULL argument");
  Frame* F = t->next();
  memset(fr, 0, sizeof(*fr));
  if (F->status < 0) return set_error(CASS_EINVAL, F->err);
  fr->status = F->status;
  if (F->status != 0) return CASS_OK;
  fr->natoms = F->natoms;
  fr->index = F->index;
  memcpy(fr->box, F->H, sizeof(fr->box));
  fr->nmols = F->nmols.data();
  fr->xyz = F->xyz;
  fr->pinned = F->pinned ? 1 : 0;
  return CASS_OK;
}

int cass_traj_stats(cass_traj* t, int64_t* frames, double* parse_seconds) {
  if (!t) return set_error(CASS_EINVAL, "NULL trajectory");
  std::lock_guard<std::mutex> lk(t->mu);
  if (frames) *frames = t->frames;
  if (parse_seconds) *parse_seconds = t->parse_s;
  return CASS_OK;
}

int cass_traj_close(cass_traj* t) {
  delete t;
  return CASS_OK;
}

int cass_load_next_frame(cass_ctx* c, int32_t nboxes, cass_traj* const* traj, int32_t* end_reached) {
  if (!c || !traj || !end_reached) return set_error(CASS_EINVAL, "NULL argument");
  if (nboxes != c->nboxes) return set_error(CASS_EINVAL, "one trajectory per box is required");
  *end_reached = 0;
  std::vector<CassFrame> fr(nboxes);
  for (int b = 0; b < nboxes; ++b) {
    if (!traj[b]) return set_error(CASS_EINVAL, "NULL trajectory");
    if (traj[b]->nspecies != c->nspecies) return set_error(CASS_EINVAL, "trajectory species count differs");
    for (int is = 0; is < c->nspecies; ++is)
      if (traj[b]->natoms_sp[is] != c->sp[is].natoms) return set_error(CASS_EINVAL, "trajectory atom count differs");
    int rc = cass_traj_next(traj[b], &fr[b]);
    if (rc) return rc;
    if (fr[b].status != 0) {
      *end_reached = 1;
      return CASS_OK;
    }
  }
  // capacity: the frame's locates must exist (max_molecules)
  std::vector<int> tot(c->nspecies, 0);
  for (int b = 0; b < nboxes; ++b)
    for (int is = 0; is < c->nspecies; ++is) tot[is] += fr[b].nmols[is];
  for (int is = 0; is < c->nspecies; ++is)
    if (tot[is] > c->max_mol[is]) return set_error(CASS_ECAPACITY, "frame holds more molecules than max_molecules");
  for (int b = 0; b < nboxes; ++b) {
    const double* H = fr[b].box;
    if (H[1] != 0.0 || H[2] != 0.0 || H[3] != 0.0 || H[5] != 0.0 || H[6] != 0.0 || H[7] != 0.0)
      return set_error(CASS_EUNSUPPORTED, "frame box matrix is not orthorhombic");
    if (!(H[0] > 0.0 && H[4] > 0.0 && H[8] > 0.0)) return set_error(CASS_EINVAL, "frame box edge not positive");
    if (!c->box[b].defined) return set_error(CASS_ESTATE, "box not defined");
  }
  // Set_Frame_Box (:57-102): a box whose edges changed gets them and its k-vectors
  for (int b = 0; b < nboxes; ++b) {
    const double* H = fr[b].box;
    CassBoxDesc d = c->box[b].desc;
    if (d.length[0] != H[0] || d.length[1] != H[4] || d.length[2] != H[8]) {
      d.length[0] = H[0];
      d.length[1] = H[4];
      d.length[2] = H[8];
      int rc = cass_set_box(c, b + 1, &d);
      if (rc) return rc;
    }
  }
  // every molecule not live (:23-28), then the frame's molecules, box by box
  for (int slot = 0; slot < c->nmol_slots; ++slot) set_mol_box_ext(c, slot, -1);
  std::vector<int> base(c->nspecies, 0);
  for (int b = 0; b < nboxes; ++b) {
    const BoxH& B = c->box[b];
    const double L[3] = {B.desc.length[0], B.desc.length[1], B.desc.length[2]};
    const double* xyz = fr[b].xyz;
    size_t atom = 0;  // atom_ibounds(1,is,ibox) - 1
    for (int is = 0; is < c->nspecies; ++is) {
      SpeciesH& s = c->sp[is];
      for (int k = 0; k < fr[b].nmols[is]; ++k) {
        const int im = base[is] + k;  // 0-based locate
        double* r = &s.pos[(size_t)im * 3 * s.natoms];
        const double* src = xyz + 3 * atom;
        // Get_COM (get_com.f90:45-105) of the molecule as read
        double tm = 0.0, com[3] = {0.0, 0.0, 0.0};
        for (int a = 0; a < s.natoms; ++a) {
          tm = tm + s.mass[a];
          for (int q = 0; q < 3; ++q) com[q] = com[q] + s.mass[a] * src[3 * a + q];
        }
        double cn[3];
        for (int q = 0; q < 3; ++q) {
          com[q] = com[q] / tm;
          // Apply_PBC_Anint, orthorhombic: x - L * ANINT(x / L)
          cn[q] = com[q] - L[q] * std::round(com[q] / L[q]);
        }
        for (int a = 0; a < s.natoms; ++a)
          for (int q = 0; q < 3; ++q) r[3 * a + q] = src[3 * a + q] + cn[q] - com[q];
        set_mol_box_ext(c, c->mol_base[is] + im, b);
        atom += (size_t)s.natoms;
      }
      base[is] += fr[b].nmols[is];
    }
  }
  // the frames are copied: the readers parse the next ones while the boxes
  // are packed and the device works on this frame
  for (int b = 0; b < nboxes; ++b) traj[b]->release_taken();
  CASS_CUDA(cudaSetDevice(c->device));
  int rc;
  for (int b = 0; b < nboxes; ++b) {
    invalidate_ext(c, b);
    c->box[b].vol_saved = false;
  }
  if ((rc = frame_setup_ext(c))) return rc;
  return CASS_OK;
}

}  // extern "C"
