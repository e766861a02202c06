// vca_api.cu -- C-ABI entry points and host orchestration of the GB300
// cluster-ED -> Lanczos Green's function -> Potthoff Omega path.
//
// The host side only sequences kernels, moves the caller's arrays across the
// boundary and keeps scalar bookkeeping (sector order, the T=0 ground-state
// list); every vector, matrix and reduction of the solve runs on the GPU.
#include <cuda_runtime.h>

#include <algorithm>
#include <cerrno>
#include <cfloat>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/vca_gpu.h"
#include "vca_fx.cuh"
#include "vca_multi.cuh"
#include "vca_batch.cuh"
#include "vca_kernels.cuh"
#include "vca_gfmatrix.h"
#include "vca_host.h"

using namespace vca;
typedef std::complex<double> cd;

namespace {

std::string g_err;

#define VFAIL(code, msg)   \
  do {                     \
    g_err = (msg);         \
    return (code);         \
  } while (0)
#define CUCHK(x)                                                                            \
  do {                                                                                      \
    cudaError_t e_ = (x);                                                                   \
    if (e_ != cudaSuccess) {                                                                \
      g_err = std::string("CUDA error ") + cudaGetErrorString(e_) + " at " + #x;            \
      return e_ == cudaErrorMemoryAllocation ? VCA_ERR_ALLOC : VCA_ERR_CUDA;                \
    }                                                                                       \
  } while (0)
#define RCHK(x)            \
  do {                     \
    int r_ = (x);          \
    if (r_ != VCA_OK) return r_; \
  } while (0)

// Device allocations owned by one stage of the context.
struct Arena {
  std::vector<void*> ptrs;
  template <class T>
  int alloc(T** p, size_t n) {
    *p = nullptr;
    if (n == 0) n = 1;
    cudaError_t e = cudaMalloc((void**)p, n * sizeof(T));
    if (e != cudaSuccess) {
      *p = nullptr;
      g_err = std::string("cudaMalloc of ") + std::to_string(n * sizeof(T)) + " bytes failed: " +
              cudaGetErrorString(e);
      cudaGetLastError();
      return VCA_ERR_ALLOC;
    }
    ptrs.push_back(*p);
    return VCA_OK;
  }
  void release() {
    for (void* p : ptrs) cudaFree(p);
    ptrs.clear();
  }
};

struct GState {
  int sector;
  double e;
  void* vec;  // device, double (real model) or double2
};

struct ChainRec {
  int elem;   // spin-diagonal element index (il,jl,is,io,jo)
  int state;  // 0-based GS index
  int chan;   // 1..4 as the reference's channel numbers
  int nlanc;  // steps asked for: min(target dimension, LANC_NGFITER)
};

struct Ctx {
  vca_config cfg{};
  bool has_bath = false;
  int Ns = 0, Nsectors = 0, N = 0, L = 0, Nb = 0;
  cudaStream_t st = nullptr;
  Arena basis, ham, states, gf, omega, work;
  // frequency rule of the Omega integral (depends on omega_nodes and
  // omega_scale only): computed on the first solve, reused after
  Arena nodes;
  double2* node_z = nullptr;
  double* node_w = nullptr;
  int node_n = 0;
  double node_scale = 0.0;
  std::vector<int> dimn;
  std::vector<int*> words;
  int* d_iscratch = nullptr;
  // Hamiltonian of the current point
  bool ham_set = false, real_model = true;
  std::vector<cd> Hloc, bath_h, bath_v;
  std::vector<SpinSpace> sp[2];
  int dwset = 0;  // spin table used by the down word (0 when Nspin == 1)
  MixedDiag md{};
  HopPair* d_pairs[2] = {nullptr, nullptr};
  // fixed-point path (real Hamiltonians with <= 4 hopping magnitudes)
  bool fx = false;
  FxScales fxs{};
  FxView fxbase{};
  std::vector<signed char*> fx_code[2];
  std::vector<unsigned*> fx_hop[2];
  std::vector<i64*> fx_e1[2];
  std::vector<int*> fx_npos[2];   // sign-sorted hop lists: positive count per row
  std::vector<int*> fx_perm[2];   // rows by decreasing hop count
  struct PermTabs {
    unsigned* hop = nullptr;
    unsigned* rhop = nullptr;
    int* pinv = nullptr;
    int *cnt = nullptr, *npos = nullptr, *word = nullptr;
    i64* e1 = nullptr;
  };
  std::vector<PermTabs> fx_ptab[2];  // tables in perm order
  // bank schedules of the paired-column single-vector kernel (spin spaces
  // that can be the up role of a sector >= FX1_MIN_DIM), else nullptr
  std::vector<unsigned*> fx_sched[2];
  std::vector<int*> fx_wround[2];
  std::vector<int*> fx_wgrp[2];
  std::vector<HopPair> host_pairs;
  size_t host_pairs_set0 = 0;  // pairs of the up set (the rest are the down set's)
  std::vector<double> host_eps_abs;  // per spin set: bound of |one-body energy|
  // finite temperature (LANC_NSTATES_TOTAL != 1, VCA_SETUP.f90:157-175); the
  // list cap is adjusted by every finite-T diagonalisation and carries over
  bool finiteT = false;
  int nstates_total = 1;
  // "arpack" at finite T: eigenpairs asked of each sector, adapted by every
  // solve's sweeps (neigen_sector, VCA_DIAG.f90:98-102, vca_post_diag :411-437)
  std::vector<int> neigen;
  // results
  bool solved = false;
  std::vector<double> sector_e;
  std::vector<GState> gs;
  double egs = 0, zeta = 0, omega_int = 0, sft = 0;
  double omega_prime = 0, max_exc = 0, int_R = 0, sum_part = 0, contour_part = 0;
  int nmax = 0, contour_points = 0;
  std::vector<ChainRec> chains;
  int ld = 0;
  double* d_poles = nullptr;     // filled on demand from the chain store
  double2* d_weights = nullptr;
  int* d_nexc = nullptr;
  bool poles_ready = false;
  int ql_max_iter = 60;  // QL sweeps per eigenvalue before a chain is reported unconverged
  bool omega_inverse_form = true;  // T=0 k-sum through G'^-1 + M at nodes with w <= 10
  ChainStore cstore{};
  int nelem = 0;
  int* d_elem_ptr = nullptr;
  int* d_elem_chain = nullptr;
  // Hk and Omega
  int64_t Nk = 0;
  double2* d_Hk = nullptr;  // lso per k
  // k-points paired by H_k' = conj(H_k) (= H_k^T): representatives (lso)
  // and their multiplicities, for models whose Omega integrand is equal at
  // the two points of a pair
  int64_t Nk_rep = 0;
  double2* d_Hk_rep = nullptr;
  double* d_kw = nullptr;
  bool hk_spin_diag = true;
  std::vector<cd> hk_const;       // lso: value of Hk when equal at every k
  std::vector<char> hk_varying;   // lso: 1 when Hk differs between k-points
  double t_ms[4] = {0, 0, 0, 0};  // set_hamiltonian, diagonalise, chains, Omega
  double chain_ms[3] = {0, 0, 0};  // chain stage: start vectors, Lanczos steps (ms), batches
  // the last vca_gpu_solve_batch in the batched form: tables, search,
  // eigenvectors, chains, Omega, the closing plain solve (wall ms, all waves)
  double bt_ms[6] = {0, 0, 0, 0, 0, 0};
  int64_t bt_skipped = 0;  // (point, sector) searches the last batched solve skipped by their bound
  int bt_shape[2] = {MC_ROWS, 8};  // the chains' tile shape it ran: rows per tile, row lanes per block
  bool autotune = true;      // tune that shape on first use per problem class
  bool rhop_order = true;    // pair the position-ordered kernel's hop parities (fx_rhop_parity_order)
  int chain_streams = 1;     // chain column groups in flight at a time (their own streams)
  cudaStream_t st2 = nullptr;  // the second group's stream
  // GFmatrix read from a restart file (read_gfprime): replaces the solve's
  // tables for G'(z) and the channel getter until the next solve
  // Sigma read back by vca_read_impSigma: the Sigma getters return it until
  // the next solve, (Nlat,Nlat,Nspin,Nspin,Norb,Norb,L) complex per grid
  bool sigma_loaded = false;
  std::vector<double> sigma_mats, sigma_real;
  bool gfm_loaded = false;
  GfmTable gfm;                     // host copy, file order
  std::vector<int64_t> gfm_state0;  // per file element: its first entry in gfm.nchan
  std::vector<int64_t> gfm_chan0;   // per (element, state): its first entry in gfm.nexc
  std::vector<int64_t> gfm_exc0;    // per channel: its first excitation
  Arena gfm_dev;
  int64_t* d_gfm_ptr = nullptr;  // [nelem+1] excitation ranges, elem_index order
  double2* d_gfm_p = nullptr;
  double2* d_gfm_w = nullptr;
};
Ctx* g = nullptr;
static void gfm_drop();

inline int64_t binom_h(int n, int k) {
  if (k < 0 || k > n) return 0;
  int64_t v = 1;
  for (int t = 1; t <= k; t++) v = v * (n + 1 - t) / t;
  return v;
}
inline int sec_nup(int isector) { return ((isector - 1) / (g->Ns + 1)) % (g->Ns + 1); }
inline int sec_ndw(int isector) { return (isector - 1) % (g->Ns + 1); }
inline int sec_of(int nup, int ndw) { return 1 + ndw + nup * (g->Ns + 1); }

// column-major offsets of the caller's arrays
inline int64_t idx_nnn(const vca_config& c, int il, int jl, int is, int js, int io, int jo) {
  return il + (int64_t)c.Nlat * (jl + (int64_t)c.Nlat * (is + (int64_t)c.Nspin *
         (js + (int64_t)c.Nspin * (io + (int64_t)c.Norb * jo))));
}
inline int64_t idx_bh(const vca_config& c, int il, int jl, int is, int js, int io, int jo) {
  return il + (int64_t)c.Nlat_bath * (jl + (int64_t)c.Nlat_bath * (is + (int64_t)c.Nspin *
         (js + (int64_t)c.Nspin * (io + (int64_t)c.Norb_bath * jo))));
}
inline int64_t idx_bv(const vca_config& c, int il, int jl, int is, int js, int io, int jo) {
  return il + (int64_t)c.Nlat * (jl + (int64_t)c.Nlat_bath * (is + (int64_t)c.Nspin *
         (js + (int64_t)c.Nspin * (io + (int64_t)c.Norb * jo))));
}
inline int elem_index(const vca_config& c, int il, int jl, int is, int io, int jo) {
  return il + c.Nlat * (jl + c.Nlat * (is + c.Nspin * (io + c.Norb * jo)));
}

int check_finite(const double* p, size_t n, const char* what) {
  for (size_t i = 0; i < n; i++)
    if (!std::isfinite(p[i])) VFAIL(VCA_ERR_NUMERIC, std::string(what) + " holds NaN or Inf");
  return VCA_OK;
}

size_t hloc_len(const vca_config& c) {
  return (size_t)c.Nlat * c.Nlat * c.Nspin * c.Nspin * c.Norb * c.Norb;
}
size_t bh_len(const vca_config& c) {
  return (size_t)c.Nlat_bath * c.Nlat_bath * c.Nspin * c.Nspin * c.Norb_bath * c.Norb_bath;
}
size_t bv_len(const vca_config& c) {
  return (size_t)c.Nlat * c.Nlat_bath * c.Nspin * c.Nspin * c.Norb * c.Norb_bath;
}

// View of a sector whose first (fastest) spin index runs over spin space
// (sa, na) and second over (sb, nb).  view_of is the natural order; the
// chain batches of sectors with DimUp > DimDw run with the roles swapped
// (element idw + iup*DimDw): the stored Hamiltonian has no cross-spin sign
// and a mixed diagonal symmetric in the two words, so H is the same operator
// in either order, and the staged H x v then holds the smaller block.
SectorView view_pair(int sa, int na, int sb, int nb) {
  const SpinSpace& u = g->sp[sa][na];
  const SpinSpace& d = g->sp[sb][nb];
  SectorView v;
  v.dimup = u.dim;
  v.dimdw = d.dim;
  v.wup = u.width;
  v.wdw = d.width;
  v.up_words = u.words;
  v.dw_words = d.words;
  v.up_cnt = u.cnt;
  v.dw_cnt = d.cnt;
  v.up_src = u.src;
  v.dw_src = d.src;
  v.up_amp = u.amp;
  v.dw_amp = d.amp;
  v.up_e1 = u.e1;
  v.dw_e1 = d.e1;
  return v;
}
SectorView view_of(int nup, int ndw) { return view_pair(0, nup, g->dwset, ndw); }

FxView fx_view_pair(int sa, int na, int sb, int nb) {
  FxView f = g->fxbase;
  f.up_code = g->fx_code[sa][na];
  f.dw_code = g->fx_code[sb][nb];
  f.up_hop = g->fx_hop[sa][na];
  f.dw_hop = g->fx_hop[sb][nb];
  f.up_e1 = g->fx_e1[sa][na];
  f.dw_e1 = g->fx_e1[sb][nb];
  f.up_npos = g->fx_npos[sa][na];
  f.dw_npos = g->fx_npos[sb][nb];
  f.up_perm = g->fx_perm[sa][na];
  const Ctx::PermTabs& pt = g->fx_ptab[sa][na];
  f.up_phop = pt.hop;
  f.up_rhop = pt.rhop;
  f.up_pinv = pt.pinv;
  f.rows_permuted = 0;
  f.up_pcnt = pt.cnt;
  f.up_pnpos = pt.npos;
  f.up_pword = pt.word;
  f.up_pe1 = pt.e1;
  // hxv_variant 1 keeps the one-column single-vector form (the comparison arm)
  f.up_sched = g->cfg.hxv_variant == 1 ? nullptr : g->fx_sched[sa][na];
  f.up_wround = g->cfg.hxv_variant == 1 ? nullptr : g->fx_wround[sa][na];
  f.up_wgrp = g->cfg.hxv_variant == 1 ? nullptr : g->fx_wgrp[sa][na];
  return f;
}
FxView fx_view_of(int nup, int ndw) { return fx_view_pair(0, nup, g->dwset, ndw); }

inline int ceil_log2(double x) {  // smallest e with 2^e >= x (x > 0)
  int e = 0;
  double p = 1.0;
  while (p < x) { p *= 2.0; e++; }
  return e;
}

// ---------------------------------------------------------------------------
// One-body data of a solve point -> hop tables and diagonal energies.
// ---------------------------------------------------------------------------
int set_hamiltonian(const double* Hloc, const double* bath_h, const double* bath_v) {
  const vca_config& c = g->cfg;
  if (!Hloc) VFAIL(VCA_ERR_ARG, "Hloc is NULL");
  if ((bath_h == nullptr) != (bath_v == nullptr)) VFAIL(VCA_ERR_ARG, "bath_h and bath_v must be given together");
  if (g->has_bath && !bath_h) VFAIL(VCA_ERR_SHAPE, "the solver was initialised with a bath: bath_h/bath_v required");
  if (!g->has_bath && bath_h) VFAIL(VCA_ERR_SHAPE, "the solver was initialised without a bath (Nlat_bath=Norb_bath=0)");
  RCHK(check_finite(Hloc, 2 * hloc_len(c), "Hloc"));
  g->Hloc.resize(hloc_len(c));
  for (size_t i = 0; i < g->Hloc.size(); i++) g->Hloc[i] = cd(Hloc[2 * i], Hloc[2 * i + 1]);
  if (g->has_bath) {
    RCHK(check_finite(bath_h, 2 * bh_len(c), "bath_h"));
    RCHK(check_finite(bath_v, 2 * bv_len(c), "bath_v"));
    g->bath_h.resize(bh_len(c));
    g->bath_v.resize(bv_len(c));
    for (size_t i = 0; i < g->bath_h.size(); i++) g->bath_h[i] = cd(bath_h[2 * i], bath_h[2 * i + 1]);
    for (size_t i = 0; i < g->bath_v.size(); i++) g->bath_v[i] = cd(bath_v[2 * i], bath_v[2 * i + 1]);
    // vca_set_bath Hartree shift (VCA_BATH_SETUP.f90:127-136)
    if (c.hfmode && !c.hfshift)
      for (int il = 0; il < c.Nlat_bath; il++)
        for (int io = 0; io < c.Norb_bath && io < 5; io++)
          for (int is = 0; is < c.Nspin; is++)
            g->bath_h[idx_bh(c, il, il, is, is, io, io)] -=
                0.5 * c.Uloc[io] + 0.5 * c.Ust * (c.Norb - 1) + 0.5 * (c.Ust - c.Jh) * (c.Norb - 1);
  }
  g->ham.release();
  const int nsets = (c.Nspin == 2) ? 2 : 1;
  g->dwset = nsets - 1;
  // real model?  (only spin-diagonal blocks enter H, VCA_HAMILTONIAN/stored/*)
  bool real = true;
  for (int s = 0; s < c.Nspin; s++) {
    for (int il = 0; il < c.Nlat; il++)
      for (int jl = 0; jl < c.Nlat; jl++)
        for (int io = 0; io < c.Norb; io++)
          for (int jo = 0; jo < c.Norb; jo++)
            if (g->Hloc[idx_nnn(c, il, jl, s, s, io, jo)].imag() != 0.0) real = false;
    if (g->has_bath) {
      for (int a = 0; a < c.Nlat_bath; a++)
        for (int b = 0; b < c.Nlat_bath; b++)
          for (int oa = 0; oa < c.Norb_bath; oa++)
            for (int ob = 0; ob < c.Norb_bath; ob++)
              if (g->bath_h[idx_bh(c, a, b, s, s, oa, ob)].imag() != 0.0) real = false;
      for (int il = 0; il < c.Nlat; il++)
        for (int b = 0; b < c.Nlat_bath; b++)
          for (int io = 0; io < c.Norb; io++)
            for (int ob = 0; ob < c.Norb_bath; ob++)
              if (g->bath_v[idx_bv(c, il, b, s, s, io, ob)].imag() != 0.0) real = false;
    }
  }
  g->real_model = real;
  const int LC = c.Nlat * c.Norb;
  for (int set = 0; set < nsets; set++) {
    const int sidx = (set == 0) ? 0 : c.Nspin - 1;
    std::vector<HopPair> pairs;
    for (int il = 0; il < c.Nlat; il++)  // H_cluster_up.f90:1-28
      for (int jl = 0; jl < c.Nlat; jl++)
        for (int io = 0; io < c.Norb; io++)
          for (int jo = 0; jo < c.Norb; jo++) {
            int is = io + il * c.Norb, js = jo + jl * c.Norb;
            cd h = g->Hloc[idx_nnn(c, il, jl, sidx, sidx, io, jo)];
            if (is != js && h != 0.0) pairs.push_back({is, js, h.real(), h.imag()});
          }
    if (g->has_bath) {
      for (int la = 0; la < c.Nlat_bath; la++)  // H_cluster_up.f90:30-55
        for (int lb = 0; lb < c.Nlat_bath; lb++)
          for (int oa = 0; oa < c.Norb_bath; oa++)
            for (int ob = 0; ob < c.Norb_bath; ob++) {
              int ia = LC + la * c.Norb_bath + oa, ib = LC + lb * c.Norb_bath + ob;
              cd h = g->bath_h[idx_bh(c, la, lb, sidx, sidx, oa, ob)];
              if (ia != ib && h != 0.0) pairs.push_back({ia, ib, h.real(), h.imag()});
            }
      for (int il = 0; il < c.Nlat; il++)  // H_cluster_up.f90:57-86
        for (int io = 0; io < c.Norb; io++)
          for (int lb = 0; lb < c.Nlat_bath; lb++)
            for (int ob = 0; ob < c.Norb_bath; ob++) {
              int ia = LC + lb * c.Norb_bath + ob, is = io + il * c.Norb;
              cd v = g->bath_v[idx_bv(c, il, lb, sidx, sidx, io, ob)];
              if (v == 0.0) continue;
              pairs.push_back({is, ia, v.real(), v.imag()});
              pairs.push_back({ia, is, v.real(), -v.imag()});
            }
    }
    if ((int)pairs.size() > VCA_MAX_PAIRS) VFAIL(VCA_ERR_UNSUPPORTED, "too many one-body pairs");
    if (set == 0) { g->host_pairs.clear(); g->host_eps_abs.clear(); }
    g->host_pairs.insert(g->host_pairs.end(), pairs.begin(), pairs.end());
    if (set == 0) g->host_pairs_set0 = g->host_pairs.size();
    RCHK(g->ham.alloc(&g->d_pairs[set], pairs.size()));
    if (!pairs.empty())
      CUCHK(cudaMemcpyAsync(g->d_pairs[set], pairs.data(), pairs.size() * sizeof(HopPair),
                            cudaMemcpyHostToDevice, g->st));
    // diagonal one-body energies (H_cluster_local.f90)
    E1Params ep{};
    ep.norb = c.Norb;
    ep.upar = (c.Norb > 1) ? (c.Ust - c.Jh) : 0.0;
    for (int o = 0; o < c.Norb; o++) {
      unsigned m = 0;
      for (int il = 0; il < c.Nlat; il++) m |= 1u << (o + il * c.Norb);
      ep.omask[o] = m;
    }
    for (int il = 0; il < c.Nlat; il++)
      for (int io = 0; io < c.Norb; io++) {
        cd e = g->Hloc[idx_nnn(c, il, il, sidx, sidx, io, io)] - c.xmu;
        if (c.hfmode) {
          e += -0.5 * c.Uloc[io];
          if (c.Norb > 1) e += -0.5 * (2.0 * c.Ust - c.Jh) * (c.Norb - 1);
        }
        ep.eps[io + il * c.Norb] = make_double2(e.real(), e.imag());
      }
    if (g->has_bath)
      for (int lb = 0; lb < c.Nlat_bath; lb++)
        for (int ob = 0; ob < c.Norb_bath; ob++) {
          cd e = g->bath_h[idx_bh(c, lb, lb, sidx, sidx, ob, ob)] - c.xmu;
          ep.eps[LC + lb * c.Norb_bath + ob] = make_double2(e.real(), e.imag());
        }
    {
      double em = 0.0;
      for (int l = 0; l < g->Ns; l++) em = std::max(em, std::abs(cd(ep.eps[l].x, ep.eps[l].y)));
      g->host_eps_abs.push_back(em * g->Ns + std::fabs(ep.upar) * c.Nlat * c.Norb * c.Norb);
    }
    g->sp[set].assign(g->Ns + 1, SpinSpace());
    for (int n = 0; n <= g->Ns; n++) {
      SpinSpace& S = g->sp[set][n];
      S.n = n;
      S.dim = g->dimn[n];
      S.words = g->words[n];
      RCHK(g->ham.alloc(&S.cnt, S.dim));
      S.width = launch_hop_count(g->Ns, n, S.dim, S.words, g->d_pairs[set], (int)pairs.size(), S.cnt,
                                 g->d_iscratch, g->st);
      CUCHK(cudaGetLastError());
      RCHK(g->ham.alloc(&S.src, (size_t)S.width * S.dim));
      RCHK(g->ham.alloc(&S.amp, (size_t)S.width * S.dim));
      RCHK(g->ham.alloc(&S.e1, S.dim));
      launch_hop_fill(g->Ns, n, S.dim, S.width, S.words, g->d_pairs[set], (int)pairs.size(), S.src, S.amp,
                      g->st);
      launch_e1(S.dim, S.words, ep, false, S.e1, g->st);
      CUCHK(cudaGetLastError());
    }
  }
  if (nsets == 1) g->sp[1] = g->sp[0];
  // opposite-spin terms and constants (H_cluster_local.f90:26-76)
  MixedDiag md{};
  md.norb = c.Norb;
  for (int o = 0; o < c.Norb; o++) {
    unsigned m = 0;
    for (int il = 0; il < c.Nlat; il++) m |= 1u << (o + il * c.Norb);
    md.omask[o] = m;
    md.U[o] = c.Uloc[o];
  }
  md.Ust = (c.Norb > 1) ? c.Ust : 0.0;
  md.c0 = 0.0;
  if (c.hfmode) {
    for (int io = 0; io < c.Norb; io++) md.c0 += 0.25 * c.Uloc[io] * c.Nlat;
    if (c.Norb > 1) md.c0 += c.Nlat * (c.Norb * (c.Norb - 1) / 2) * 0.25 * (2.0 * c.Ust - c.Jh);
  }
  g->md = md;
  // ---- fixed-point tables -------------------------------------------------
  g->fx = false;
  if (c.arith != VCA_ARITH_FP64 && real) {
    std::vector<double> classes;
    double amax = 0.0, epsmax = 0.0;
    // distinct hopping magnitudes over both spin tables
    for (const HopPair& hp : g->host_pairs) {
      double m = std::fabs(hp.re);
      amax = std::max(amax, m);
      bool seen = false;
      for (double x : classes) if (x == m) seen = true;
      if (!seen) classes.push_back(m);
    }
    if ((int)classes.size() <= VCA_FX_KMAX) {
      // bound on max_i sum_j |H_ij| and on |d|
      for (double e : g->host_eps_abs) epsmax = std::max(epsmax, e);
      double dmax = 2.0 * epsmax;
      for (int o = 0; o < c.Norb; o++) dmax += std::fabs(c.Uloc[o]) * c.Nlat;
      if (c.Norb > 1) dmax += std::fabs(c.Ust) * c.Nlat * c.Norb * (c.Norb - 1);
      dmax += std::fabs(md.c0);
      int wmax = 0;
      for (int set = 0; set < nsets; set++)
        for (int n = 0; n <= g->Ns; n++) wmax = std::max(wmax, g->sp[set][n].width);
      const double hbound = dmax + 2.0 * wmax * amax + 1.0;
      FxScales fs;
      fs.F = 59;
      fs.G = 61 - ceil_log2(4.0 * hbound);
      fs.A = 62 - ceil_log2(std::max(dmax, amax) + 1.0);
      fs.C = 62 - ceil_log2(hbound + 1.0);
      FxView fb{};
      fb.K = (int)classes.size();
      for (int k = 0; k < fb.K; k++) fb.afx[k] = (i64)std::llrint(std::ldexp(classes[k], fs.A));
      fb.norb = c.Norb;
      for (int o = 0; o < c.Norb; o++) {
        fb.omask[o] = md.omask[o];
        fb.Ufx[o] = (i64)std::llrint(std::ldexp(md.U[o], fs.A));
      }
      fb.Ustfx = (i64)std::llrint(std::ldexp(md.Ust, fs.A));
      fb.c0fx = (i64)std::llrint(std::ldexp(md.c0, fs.A));
      fb.shift = fs.A + fs.F - fs.G;
      double* d_cls;
      RCHK(g->ham.alloc(&d_cls, classes.size()));
      CUCHK(cudaMemcpyAsync(d_cls, classes.data(), sizeof(double) * classes.size(), cudaMemcpyHostToDevice, g->st));
      for (int set = 0; set < nsets; set++) {
        g->fx_code[set].assign(g->Ns + 1, nullptr);
        g->fx_hop[set].assign(g->Ns + 1, nullptr);
        g->fx_e1[set].assign(g->Ns + 1, nullptr);
        g->fx_npos[set].assign(g->Ns + 1, nullptr);
        g->fx_perm[set].assign(g->Ns + 1, nullptr);
        g->fx_ptab[set].assign(g->Ns + 1, Ctx::PermTabs{});
        g->fx_sched[set].assign(g->Ns + 1, nullptr);
        g->fx_wround[set].assign(g->Ns + 1, nullptr);
        g->fx_wgrp[set].assign(g->Ns + 1, nullptr);
        int64_t partner = 0;  // largest spin space the other role can take
        for (int n = 0; n <= g->Ns; n++) partner = std::max<int64_t>(partner, g->sp[nsets - 1 - set][n].dim);
        for (int n = 0; n <= g->Ns; n++) {
          SpinSpace& S = g->sp[set][n];
          RCHK(g->ham.alloc(&g->fx_hop[set][n], (size_t)S.width * S.dim));
          launch_fx_pack(S.dim, S.width, S.src, S.amp, d_cls, fb.K, g->fx_hop[set][n], g->st);
          RCHK(g->ham.alloc(&g->fx_npos[set][n], S.dim));
          launch_fx_sign_sort(S.dim, S.width, S.cnt, g->fx_hop[set][n], g->fx_npos[set][n], g->st);
          {  // rows by decreasing hop count (stable), for warps of equal loop length
            std::vector<int> cnt(S.dim), perm(S.dim);
            if (S.dim) CUCHK(cudaMemcpy(cnt.data(), S.cnt, sizeof(int) * S.dim, cudaMemcpyDeviceToHost));
            for (int r = 0; r < S.dim; r++) perm[r] = r;
            std::stable_sort(perm.begin(), perm.end(), [&](int x, int y) { return cnt[x] > cnt[y]; });
            std::vector<int> pinv(S.dim);
            for (int r = 0; r < S.dim; r++) pinv[perm[r]] = r;
            RCHK(g->ham.alloc(&g->fx_perm[set][n], S.dim));
            RCHK(g->ham.alloc(&g->fx_ptab[set][n].pinv, S.dim));
            if (S.dim) {
              CUCHK(cudaMemcpy(g->fx_perm[set][n], perm.data(), sizeof(int) * S.dim, cudaMemcpyHostToDevice));
              CUCHK(cudaMemcpy(g->fx_ptab[set][n].pinv, pinv.data(), sizeof(int) * S.dim, cudaMemcpyHostToDevice));
            }
          }
          RCHK(g->ham.alloc(&g->fx_code[set][n], (size_t)S.width * S.dim));
          RCHK(g->ham.alloc(&g->fx_e1[set][n], S.dim));
          launch_fx_codes(S.dim, S.width, S.amp, d_cls, fb.K, g->fx_code[set][n], g->st);
          launch_fx_e1(S.dim, S.e1, fs.A, g->fx_e1[set][n], g->st);
          Ctx::PermTabs& pt = g->fx_ptab[set][n];
          RCHK(g->ham.alloc(&pt.hop, (size_t)S.width * S.dim));
          RCHK(g->ham.alloc(&pt.rhop, (size_t)S.width * S.dim));
          RCHK(g->ham.alloc(&pt.cnt, S.dim));
          RCHK(g->ham.alloc(&pt.npos, S.dim));
          RCHK(g->ham.alloc(&pt.word, S.dim));
          RCHK(g->ham.alloc(&pt.e1, S.dim));
          launch_fx_perm_tables(S.dim, S.width, g->fx_perm[set][n], pt.pinv, g->fx_hop[set][n], S.cnt,
                                g->fx_npos[set][n], S.words, g->fx_e1[set][n], pt.hop, pt.rhop, pt.cnt, pt.npos,
                                pt.word, pt.e1, g->st);
          if (S.dim > 1 && (size_t)S.dim * FX_SLAB * sizeof(i64) <= 200 * 1024 && g->rhop_order) {
            // the position-ordered kernel's up block fits: pair its rows' hop parities
            std::vector<int> pc(S.dim), pn(S.dim);
            std::vector<unsigned> rh((size_t)S.width * S.dim);
            CUCHK(cudaMemcpyAsync(pc.data(), pt.cnt, sizeof(int) * S.dim, cudaMemcpyDeviceToHost, g->st));
            CUCHK(cudaMemcpyAsync(pn.data(), pt.npos, sizeof(int) * S.dim, cudaMemcpyDeviceToHost, g->st));
            CUCHK(cudaMemcpyAsync(rh.data(), pt.rhop, sizeof(unsigned) * rh.size(), cudaMemcpyDeviceToHost, g->st));
            CUCHK(cudaStreamSynchronize(g->st));
            fx_rhop_parity_order(S.dim, S.width, pc.data(), pn.data(), rh.data());
            CUCHK(cudaMemcpyAsync(pt.rhop, rh.data(), sizeof(unsigned) * rh.size(), cudaMemcpyHostToDevice, g->st));
            CUCHK(cudaStreamSynchronize(g->st));
          }
          if (S.dim > 0 && fx_pair_fits(S.dim) && (int64_t)S.dim * partner >= FX1_MIN_DIM) {
            std::vector<int> cnt(S.dim);
            std::vector<unsigned> hop((size_t)S.width * S.dim), sched;
            std::vector<int> wround, wgrp;
            CUCHK(cudaMemcpyAsync(cnt.data(), S.cnt, sizeof(int) * S.dim, cudaMemcpyDeviceToHost, g->st));
            CUCHK(cudaMemcpyAsync(hop.data(), g->fx_hop[set][n], sizeof(unsigned) * hop.size(),
                                  cudaMemcpyDeviceToHost, g->st));
            CUCHK(cudaStreamSynchronize(g->st));
            if (fx_pair_schedule(S.dim, S.width, fb.K, cnt.data(), hop.data(), sched, wround, wgrp) < 0)
              VFAIL(VCA_ERR_NUMERIC, "hop schedule of the paired-column form left hops unplaced");
            RCHK(g->ham.alloc(&g->fx_sched[set][n], std::max<size_t>(1, sched.size())));
            RCHK(g->ham.alloc(&g->fx_wround[set][n], wround.size()));
            CUCHK(cudaMemcpyAsync(g->fx_sched[set][n], sched.data(), sizeof(unsigned) * sched.size(),
                                  cudaMemcpyHostToDevice, g->st));
            CUCHK(cudaMemcpyAsync(g->fx_wround[set][n], wround.data(), sizeof(int) * wround.size(),
                                  cudaMemcpyHostToDevice, g->st));
            RCHK(g->ham.alloc(&g->fx_wgrp[set][n], std::max<size_t>(1, wgrp.size())));
            CUCHK(cudaMemcpyAsync(g->fx_wgrp[set][n], wgrp.data(), sizeof(int) * wgrp.size(),
                                  cudaMemcpyHostToDevice, g->st));
            CUCHK(cudaStreamSynchronize(g->st));  // host vectors go out of scope
          }
        }
      }
      if (nsets == 1) {
        g->fx_code[1] = g->fx_code[0];
        g->fx_hop[1] = g->fx_hop[0];
        g->fx_e1[1] = g->fx_e1[0];
        g->fx_npos[1] = g->fx_npos[0];
        g->fx_perm[1] = g->fx_perm[0];
        g->fx_ptab[1] = g->fx_ptab[0];
        g->fx_sched[1] = g->fx_sched[0];
        g->fx_wround[1] = g->fx_wround[0];
        g->fx_wgrp[1] = g->fx_wgrp[0];
      }
      CUCHK(cudaGetLastError());
      g->fxs = fs;
      g->fxbase = fb;
      g->fx = true;
    }
  }
  if (c.arith == VCA_ARITH_FX && !g->fx)
    VFAIL(VCA_ERR_UNSUPPORTED, "fixed-point arithmetic needs a real Hamiltonian with at most 4 hopping magnitudes");
  g->ham_set = true;
  CUCHK(cudaStreamSynchronize(g->st));
  return VCA_OK;
}

// ---------------------------------------------------------------------------
// Batched Lanczos driver on a column batch (GS: one chain; GF: many).
// ---------------------------------------------------------------------------
struct BatchBufs {
  void* b[3];
  double* partial;
  int nblk;
  double *col_a, *ch_a, *ch_b2, *invb, *bnow;
  double *A, *Bt;
  ChainMeta* meta;
  int* col2ch;
  i64 *afx, *bfx, *scr;  // fixed-point coefficients and per-chain scratch (2*nch)
  i64* wpart;            // alpha partials of the column H x v [2*rows*m]
  int64_t wpart_rows;
};

int lanczos_step(const SectorView& sv, const ColBatch& cb, BatchBufs& bb, int k, double tol, int ldab,
                 cudaStream_t stream = nullptr) {
  cudaStream_t st = stream ? stream : g->st;
  void* X = bb.b[0];
  void* Xp = bb.b[1];
  void* Y = bb.b[2];
  if (cb.cplx)
    launch_hxv_cplx(sv, g->md, cb.m, (const double2*)X, (double2*)Y, st);
  else
    launch_hxv_real(sv, g->md, cb.m, (const double*)X, (double*)Y, st);
  if (k > 1) launch_col_axpy(cb, bb.bnow, Xp, Y, true, st);
  launch_col_dot(cb, X, Y, bb.partial, bb.nblk, bb.col_a, st);
  launch_chain_sum(cb, bb.col_a, bb.ch_a, st);
  launch_col_axpy(cb, bb.ch_a, X, Y, true, st);
  launch_col_dot(cb, Y, Y, bb.partial, bb.nblk, bb.col_a, st);
  launch_chain_sum(cb, bb.col_a, bb.ch_b2, st);
  launch_lanczos_record(cb.nch, bb.meta, k, bb.ch_a, bb.ch_b2, bb.A, bb.Bt, ldab, tol, bb.invb, bb.bnow, st);
  launch_col_scale(cb, bb.invb, Y, Y, st);
  // rotate (X, Xp, Y) <- (Y, X, Xp)
  bb.b[0] = Y;
  bb.b[1] = X;
  bb.b[2] = Xp;
  CUCHK(cudaGetLastError());
  return VCA_OK;
}

// One Lanczos step in fixed point: X (2^-F) -> W = H X - a X - b Xp (2^-G)
// -> X_next = W / beta (2^-F).  Buffers rotate as (X, Xp, YW) <- (new, X, YW).
int lanczos_step_fx(const SectorView& sv, const FxView& fv, const ColBatch& cb, BatchBufs& bb, int k,
                    double tol, int ldab, cudaStream_t stream = nullptr) {
  cudaStream_t st = stream ? stream : g->st;
  const FxScales& fs = g->fxs;
  i64* X = (i64*)bb.b[0];
  i64* Xp = (i64*)bb.b[1];
  i64* YW = (i64*)bb.b[2];
  const bool warp_only = g->cfg.hxv_variant == 1;
  if (cb.m >= 16 && bb.wpart && bb.wpart_rows >= hxv_fx_cols_rows(sv, fv, cb.m, warp_only)) {
    // alpha partials come out of the product kernel
    const int rb = hxv_fx_cols_rows(sv, fv, cb.m, warp_only);
    launch_hxv_fx_cols(sv, fv, cb.m, X, YW, bb.wpart, warp_only, st);
    launch_fx_partial_reduce(cb.m, rb, bb.wpart, fs.F + fs.G, bb.col_a, st);
  } else {
    launch_hxv_fx(sv, fv, cb.m, X, YW, st);
    launch_fx_dot(cb, X, YW, fs.F, fs.G, (i64*)bb.partial, bb.nblk, bb.col_a, st);
  }
  launch_chain_sum(cb, bb.col_a, bb.ch_a, st);
  launch_fx_coef(cb.nch, bb.ch_a, 1.0, fs.C, bb.afx, st);
  if (k > 1) launch_fx_coef(cb.nch, bb.bnow, 1.0, fs.C, bb.bfx, st);
  launch_fx_update_dot(cb, fs, bb.afx, bb.bfx, k > 1, X, Xp, YW, (i64*)bb.partial, bb.nblk, bb.col_a, st);
  launch_chain_sum(cb, bb.col_a, bb.ch_b2, st);
  launch_lanczos_record(cb.nch, bb.meta, k, bb.ch_a, bb.ch_b2, bb.A, bb.Bt, ldab, tol, bb.invb, bb.bnow, st);
  launch_fx_normalize(cb, fs, bb.invb, YW, Xp, bb.scr, st);  // X_next into the old Xp buffer
  bb.b[0] = Xp;
  bb.b[1] = X;
  bb.b[2] = YW;
  CUCHK(cudaGetLastError());
  return VCA_OK;
}

int alloc_batch(Arena& ar, int64_t rows, int m, bool cplx, int nch, int ldab, BatchBufs& bb) {
  const size_t es = cplx ? sizeof(double2) : sizeof(double);
  // fixed-point batches are slab-major with zero pad columns
  const int mc = g->fx ? fx_cols_alloc(m) : m;
  for (int q = 0; q < 3; q++) {
    char* p;
    RCHK(ar.alloc(&p, (size_t)rows * mc * es));
    if (mc > m) CUCHK(cudaMemsetAsync(p, 0, (size_t)rows * mc * es, g->st));
    bb.b[q] = p;
  }
  bb.nblk = (int)std::min<int64_t>(std::max<int64_t>(1, rows / 256), 608);
  RCHK(ar.alloc(&bb.partial, (size_t)bb.nblk * m * 2));  // int128 partials in the FX path
  RCHK(ar.alloc(&bb.afx, nch));
  RCHK(ar.alloc(&bb.bfx, nch));
  RCHK(ar.alloc(&bb.scr, 2 * (size_t)nch));
  bb.wpart = nullptr;
  bb.wpart_rows = 0;
  RCHK(ar.alloc(&bb.col_a, m));
  RCHK(ar.alloc(&bb.ch_a, nch));
  RCHK(ar.alloc(&bb.ch_b2, nch));
  RCHK(ar.alloc(&bb.invb, nch));
  RCHK(ar.alloc(&bb.bnow, nch));
  RCHK(ar.alloc(&bb.A, (size_t)nch * ldab));
  RCHK(ar.alloc(&bb.Bt, (size_t)nch * ldab));
  RCHK(ar.alloc(&bb.meta, nch));
  RCHK(ar.alloc(&bb.col2ch, m));
  CUCHK(cudaMemsetAsync(bb.A, 0, sizeof(double) * nch * ldab, g->st));
  CUCHK(cudaMemsetAsync(bb.Bt, 0, sizeof(double) * nch * ldab, g->st));
  CUCHK(cudaMemsetAsync(bb.bnow, 0, sizeof(double) * nch, g->st));
  return VCA_OK;
}

// Ground state of one sector by Lanczos (replaces SciFortran sp_lanc_eigh,
// VCA_DIAG.f90:172-184): deterministic start vector, residual test every
// gs_check_every steps, eigenvector by a second pass over stored coefficients.
int sector_gs(int isector, double* E, void** vec_out, Arena& keep) {
  const vca_config& c = g->cfg;
  const int nup = sec_nup(isector), ndw = sec_ndw(isector);
  SectorView sv = view_of(nup, ndw);
  const int64_t D = (int64_t)sv.dimup * sv.dimdw;
  const bool cplx = !g->real_model;
  const int nmax = (int)std::min<int64_t>(D, std::min(c.lanc_niter, 512));
  Arena ar;
  BatchBufs bb;
  int rc = alloc_batch(ar, D, 1, cplx, 1, nmax + 1, bb);
  if (rc) { ar.release(); return rc; }
  double *theta, *svec, *resid, *invB, *norm2, *invn;
  double2* dummy = nullptr;
  (void)dummy;
  if ((rc = ar.alloc(&theta, 1)) || (rc = ar.alloc(&svec, 5 * (size_t)(nmax + 1))) ||
      (rc = ar.alloc(&resid, 1)) || (rc = ar.alloc(&invB, nmax + 1)) || (rc = ar.alloc(&norm2, 1)) ||
      (rc = ar.alloc(&invn, 1))) {
    ar.release();
    return rc;
  }
  ChainMeta m0{1, 0, nmax, 1, 0};
  int zero = 0;
  cudaMemcpyAsync(bb.meta, &m0, sizeof(m0), cudaMemcpyHostToDevice, g->st);
  cudaMemcpyAsync(bb.col2ch, &zero, sizeof(int), cudaMemcpyHostToDevice, g->st);
  ColBatch cb{D, 1, cplx, 1, bb.col2ch, bb.meta};
  auto start = [&](void* X) {
    if (cplx) {
      launch_start_vector(D, c.start_seed, isector, (double*)bb.b[2], g->st);
      launch_real_to_cplx(D, (const double*)bb.b[2], (double2*)X, g->st);
    } else {
      launch_start_vector(D, c.start_seed, isector, (double*)X, g->st);
    }
    launch_col_dot(cb, X, X, bb.partial, bb.nblk, norm2, g->st);
    launch_chain_norm_init(1, bb.meta, norm2, invn, g->st);
    launch_col_scale(cb, invn, X, X, g->st);
  };
  start(bb.b[0]);
  int mconv = 0;
  double th = 0.0;
  for (int k = 1; k <= nmax; k++) {
    if ((rc = lanczos_step(sv, cb, bb, k, c.gs_beta_tol, nmax + 1))) { ar.release(); return rc; }
    if (k % std::max(1, c.gs_check_every) == 0 || k == nmax) {
      ChainMeta mh;
      double bn;
      cudaMemcpyAsync(&mh, bb.meta, sizeof(mh), cudaMemcpyDeviceToHost, g->st);
      cudaMemcpyAsync(&bn, bb.bnow, sizeof(double), cudaMemcpyDeviceToHost, g->st);
      CUCHK(cudaStreamSynchronize(g->st));
      const int kk = mh.len;
      if (kk < 1) { ar.release(); VFAIL(VCA_ERR_NUMERIC, "Lanczos start vector has zero norm"); }
      launch_tri_lowest(bb.A, bb.Bt, kk, bn, theta, svec, resid, g->st);
      double rs;
      cudaMemcpyAsync(&th, theta, sizeof(double), cudaMemcpyDeviceToHost, g->st);
      cudaMemcpyAsync(&rs, resid, sizeof(double), cudaMemcpyDeviceToHost, g->st);
      CUCHK(cudaStreamSynchronize(g->st));
      const bool exhausted = !mh.active && kk < nmax;
      if (exhausted || rs <= c.gs_residual_tol * std::max(1.0, std::fabs(th)) || k == nmax || !mh.active) {
        mconv = kk;
        break;
      }
    }
  }
  // second pass: psi = sum_k s_k v_k with the stored alpha/beta
  const size_t es = cplx ? sizeof(double2) : sizeof(double);
  char* psi;
  if ((rc = keep.alloc(&psi, (size_t)D * es))) { ar.release(); return rc; }
  CUCHK(cudaMemsetAsync(psi, 0, (size_t)D * es, g->st));
  m0 = ChainMeta{1, 0, nmax, 1, 0};
  cudaMemcpyAsync(bb.meta, &m0, sizeof(m0), cudaMemcpyHostToDevice, g->st);
  launch_recip(nmax + 1, bb.Bt, invB, g->st);
  bb.b[0] = bb.b[0];
  void* X = bb.b[0];
  void* Xp = bb.b[1];
  void* Y = bb.b[2];
  start(X);
  for (int k = 1; k <= mconv; k++) {
    launch_psi_accum(D, cplx, svec, k - 1, X, psi, g->st);
    if (k == mconv) break;
    if (cplx) launch_hxv_cplx(sv, g->md, 1, (const double2*)X, (double2*)Y, g->st);
    else launch_hxv_real(sv, g->md, 1, (const double*)X, (double*)Y, g->st);
    if (k > 1) launch_col_axpy(cb, bb.Bt + (k - 1), Xp, Y, true, g->st);
    launch_col_axpy(cb, bb.A + (k - 1), X, Y, true, g->st);
    launch_col_scale(cb, invB + k, Y, Y, g->st);
    void* t = Xp;
    Xp = X;
    X = Y;
    Y = t;
  }
  launch_col_dot(cb, psi, psi, bb.partial, bb.nblk, norm2, g->st);
  launch_chain_norm_init(1, bb.meta, norm2, invn, g->st);
  launch_col_scale(cb, invn, psi, psi, g->st);
  CUCHK(cudaGetLastError());
  CUCHK(cudaStreamSynchronize(g->st));
  ar.release();
  *E = th;
  *vec_out = psi;
  return VCA_OK;
}

// Fixed-point variant of sector_gs: same start vector (normalised in FP64,
// then converted), same stopping rule and second pass; psi stays fixed point
// (scale 2^-F) for the exact chain gathers.
int sector_gs_fx(int isector, double* E, void** vec_out, Arena& keep) {
  const vca_config& c = g->cfg;
  const FxScales& fs = g->fxs;
  const int nup = sec_nup(isector), ndw = sec_ndw(isector);
  SectorView sv = view_of(nup, ndw);
  FxView fv = fx_view_of(nup, ndw);
  const int64_t D = (int64_t)sv.dimup * sv.dimdw;
  const int nmax = (int)std::min<int64_t>(D, std::min(c.lanc_niter, 512));
  Arena ar;
  BatchBufs bb;
  int rc = alloc_batch(ar, D, 1, false, 1, nmax + 1, bb);
  if (rc) { ar.release(); return rc; }
  double *theta, *svec, *resid, *invB, *norm2, *invn, *dtmp;
  if ((rc = ar.alloc(&theta, 1)) || (rc = ar.alloc(&svec, 5 * (size_t)(nmax + 1))) ||
      (rc = ar.alloc(&resid, 1)) || (rc = ar.alloc(&invB, nmax + 1)) || (rc = ar.alloc(&norm2, 1)) ||
      (rc = ar.alloc(&invn, 1)) || (rc = ar.alloc(&dtmp, D))) {
    ar.release();
    return rc;
  }
  ChainMeta m0{1, 0, nmax, 1, 0};
  int zero = 0;
  cudaMemcpyAsync(bb.meta, &m0, sizeof(m0), cudaMemcpyHostToDevice, g->st);
  cudaMemcpyAsync(bb.col2ch, &zero, sizeof(int), cudaMemcpyHostToDevice, g->st);
  ColBatch cb{D, 1, false, 1, bb.col2ch, bb.meta};
  // start vector normalised exactly: R = round(v*2^40), ||R||^2 an exact
  // int128 sum, one multiplier (the batched multi-sector search does the same)
  i64* R = (i64*)dtmp;
  auto start = [&](i64* X) {
    launch_fx_start_raw(D, c.start_seed, isector, R, g->st);
    launch_fx_dot(cb, R, R, 40, 40, (i64*)bb.partial, bb.nblk, norm2, g->st);
    launch_chain_norm_init(1, bb.meta, norm2, invn, g->st);
    launch_fx_rescale(cb, invn, 40, fs.F, R, X, bb.scr, g->st);
  };
  start((i64*)bb.b[0]);
  int mconv = 0;
  double th = 0.0;
  for (int k = 1; k <= nmax; k++) {
    if ((rc = lanczos_step_fx(sv, fv, cb, bb, k, c.gs_beta_tol, nmax + 1))) { ar.release(); return rc; }
    if (k % std::max(1, c.gs_check_every) == 0 || k == nmax) {
      ChainMeta mh;
      double bn;
      cudaMemcpyAsync(&mh, bb.meta, sizeof(mh), cudaMemcpyDeviceToHost, g->st);
      cudaMemcpyAsync(&bn, bb.bnow, sizeof(double), cudaMemcpyDeviceToHost, g->st);
      CUCHK(cudaStreamSynchronize(g->st));
      const int kk = mh.len;
      if (kk < 1) { ar.release(); VFAIL(VCA_ERR_NUMERIC, "Lanczos start vector has zero norm"); }
      launch_tri_lowest(bb.A, bb.Bt, kk, bn, theta, svec, resid, g->st);
      double rs;
      cudaMemcpyAsync(&th, theta, sizeof(double), cudaMemcpyDeviceToHost, g->st);
      cudaMemcpyAsync(&rs, resid, sizeof(double), cudaMemcpyDeviceToHost, g->st);
      CUCHK(cudaStreamSynchronize(g->st));
      if (!mh.active || rs <= c.gs_residual_tol * std::max(1.0, std::fabs(th)) || k == nmax) {
        mconv = kk;
        break;
      }
    }
  }
  // second pass: psi = sum_k s_k v_k from the stored coefficients
  i64* psi;
  if ((rc = keep.alloc(&psi, (size_t)D))) { ar.release(); return rc; }
  CUCHK(cudaMemsetAsync(psi, 0, (size_t)D * sizeof(i64), g->st));
  m0 = ChainMeta{1, 0, nmax, 1, 0};
  cudaMemcpyAsync(bb.meta, &m0, sizeof(m0), cudaMemcpyHostToDevice, g->st);
  launch_recip(nmax + 1, bb.Bt, invB, g->st);
  i64* X = (i64*)bb.b[0];
  i64* Xp = (i64*)bb.b[1];
  i64* YW = (i64*)bb.b[2];
  start(X);
  for (int k = 1; k <= mconv; k++) {
    launch_fx_psi_accum(D, svec, k - 1, X, psi, g->st);
    if (k == mconv) break;
    launch_hxv_fx(sv, fv, 1, X, YW, g->st);
    launch_fx_coef(1, bb.A + (k - 1), 1.0, fs.C, bb.afx, g->st);
    if (k > 1) launch_fx_coef(1, bb.Bt + (k - 1), 1.0, fs.C, bb.bfx, g->st);
    launch_fx_update(cb, fs, bb.afx, bb.bfx, k > 1, X, Xp, YW, YW, g->st);
    launch_fx_normalize(cb, fs, invB + k, YW, Xp, bb.scr, g->st);
    i64* t = Xp;
    Xp = X;
    X = t;
  }
  launch_fx_dot(cb, psi, psi, fs.F, fs.F, (i64*)bb.partial, bb.nblk, norm2, g->st);
  launch_chain_norm_init(1, bb.meta, norm2, invn, g->st);
  launch_fx_rescale(cb, invn, fs.F, fs.F, psi, psi, bb.scr, g->st);
  CUCHK(cudaGetLastError());
  CUCHK(cudaStreamSynchronize(g->st));
  ar.release();
  *E = th;
  *vec_out = psi;
  return VCA_OK;
}

// All sector energies of the fixed-point path in batched multi-sector
// Lanczos runs (groups of sectors bounded to ~2^28 elements per vector).
int batched_sector_energies(std::vector<double>& energy) {
  const vca_config& c = g->cfg;
  const int64_t cap = (int64_t)1 << 28;
  energy.assign(g->Nsectors, INFINITY);
  int s0 = 1;
  while (s0 <= g->Nsectors) {
    std::vector<MsSector> secs;
    std::vector<int> tsec;
    std::vector<int64_t> tstart;
    int64_t tot = 0;
    int nmaxg = 1;
    int s1 = s0;
    while (s1 <= g->Nsectors) {
      const int nu = sec_nup(s1), nd = sec_ndw(s1);
      const int64_t D = (int64_t)g->dimn[nu] * g->dimn[nd];
      if (!secs.empty() && tot + D > cap) break;
      MsSector m{};
      m.sv = view_of(nu, nd);
      m.fv = fx_view_of(nu, nd);
      m.off = tot;
      m.D = D;
      m.tile0 = (int)tsec.size();
      m.isector = s1;
      for (int64_t st = 0; st < D; st += MS_TILE) {
        tsec.push_back((int)secs.size());
        tstart.push_back(st);
      }
      m.ntile = (int)tsec.size() - m.tile0;
      nmaxg = std::max(nmaxg, (int)std::min<int64_t>(D, std::min(c.lanc_niter, 512)));
      secs.push_back(m);
      tot += D;
      s1++;
    }
    const int nsec = (int)secs.size(), ntiles = (int)tsec.size();
    const int ld = nmaxg + 1;
    Arena ar;
    MsSector* d_secs;
    int* d_tsec;
    int64_t* d_tstart;
    MsBufs b{};
    b.ld = ld;
    int rc = VCA_OK;
    if ((rc = ar.alloc(&d_secs, nsec)) || (rc = ar.alloc(&d_tsec, ntiles)) || (rc = ar.alloc(&d_tstart, ntiles)) ||
        (rc = ar.alloc(&b.X, tot)) || (rc = ar.alloc(&b.Xp, tot)) || (rc = ar.alloc(&b.YW, tot)) ||
        (rc = ar.alloc(&b.tpart, 2 * (size_t)ntiles)) || (rc = ar.alloc(&b.meta, nsec)) ||
        (rc = ar.alloc(&b.alpha, nsec)) || (rc = ar.alloc(&b.bnow, nsec)) ||
        (rc = ar.alloc(&b.A, (size_t)nsec * ld)) || (rc = ar.alloc(&b.Bt, (size_t)nsec * ld)) ||
        (rc = ar.alloc(&b.svec, (size_t)nsec * 5 * ld)) || (rc = ar.alloc(&b.theta, nsec)) ||
        (rc = ar.alloc(&b.resid, nsec)) || (rc = ar.alloc(&b.afx, nsec)) || (rc = ar.alloc(&b.bfx, nsec)) ||
        (rc = ar.alloc(&b.mul, nsec)) || (rc = ar.alloc(&b.msh, nsec)) || (rc = ar.alloc(&b.state, nsec)) ||
        (rc = ar.alloc(&b.mconv, nsec)) || (rc = ar.alloc(&b.undone, 1))) {
      ar.release();
      return rc;
    }
    std::vector<ChainMeta> meta(nsec);
    for (int q = 0; q < nsec; q++)
      meta[q] = ChainMeta{1, q, (int)std::min<int64_t>(secs[q].D, std::min(c.lanc_niter, 512)), 1, 0};
    cudaMemcpyAsync(d_secs, secs.data(), sizeof(MsSector) * nsec, cudaMemcpyHostToDevice, g->st);
    cudaMemcpyAsync(d_tsec, tsec.data(), sizeof(int) * ntiles, cudaMemcpyHostToDevice, g->st);
    cudaMemcpyAsync(d_tstart, tstart.data(), sizeof(int64_t) * ntiles, cudaMemcpyHostToDevice, g->st);
    cudaMemcpyAsync(b.meta, meta.data(), sizeof(ChainMeta) * nsec, cudaMemcpyHostToDevice, g->st);
    cudaMemsetAsync(b.A, 0, sizeof(double) * nsec * ld, g->st);
    cudaMemsetAsync(b.Bt, 0, sizeof(double) * nsec * ld, g->st);
    cudaMemsetAsync(b.bnow, 0, sizeof(double) * nsec, g->st);
    cudaMemsetAsync(b.state, 0, sizeof(int) * nsec, g->st);
    MsGroup gp{d_secs, d_tsec, d_tstart, nsec, ntiles};
    ms_launch_start(gp, c.start_seed, g->fxs.F, b.YW, b.X, b.tpart, b.meta, b.mul, b.msh, g->st);
    for (int k = 1; k <= nmaxg; k++) {
      ms_launch_step(gp, g->fxs, g->fxbase.K, k, c.gs_beta_tol, b, g->st);
      if (k % std::max(1, c.gs_check_every) == 0 || k == nmaxg) {
        cudaMemsetAsync(b.undone, 0, sizeof(int), g->st);
        ms_launch_check(gp, b, c.gs_residual_tol, g->st);
        int undone = 0;
        cudaMemcpyAsync(&undone, b.undone, sizeof(int), cudaMemcpyDeviceToHost, g->st);
        CUCHK(cudaStreamSynchronize(g->st));
        if (undone == 0) break;
      }
    }
    CUCHK(cudaGetLastError());
    std::vector<double> th(nsec);
    cudaMemcpyAsync(th.data(), b.theta, sizeof(double) * nsec, cudaMemcpyDeviceToHost, g->st);
    CUCHK(cudaStreamSynchronize(g->st));
    for (int q = 0; q < nsec; q++) energy[secs[q].isector - 1] = th[q];
    ar.release();
    s0 = s1;
  }
  return VCA_OK;
}

// All sector energies of the FP64 path (real or complex H) in batched
// multi-sector Lanczos runs: one launch per phase over every sector of a
// group (groups bounded to ~2^28 elements per vector); the single-sector
// recurrence, start vectors and stopping rule.
int batched_sector_energies_f64(std::vector<double>& energy) {
  const vca_config& c = g->cfg;
  const bool cplx = !g->real_model;
  const size_t es = cplx ? sizeof(double2) : sizeof(double);
  const int64_t cap = (int64_t)1 << 28;
  energy.assign(g->Nsectors, INFINITY);
  int s0 = 1;
  while (s0 <= g->Nsectors) {
    std::vector<MsSector> secs;
    std::vector<int> tsec;
    std::vector<int64_t> tstart;
    int64_t tot = 0;
    int nmaxg = 1;
    int s1 = s0;
    while (s1 <= g->Nsectors) {
      const int nu = sec_nup(s1), nd = sec_ndw(s1);
      const int64_t D = (int64_t)g->dimn[nu] * g->dimn[nd];
      if (!secs.empty() && tot + D > cap) break;
      MsSector m{};
      m.sv = view_of(nu, nd);
      m.off = tot;
      m.D = D;
      m.tile0 = (int)tsec.size();
      m.isector = s1;
      for (int64_t st = 0; st < D; st += MS_TILE) {
        tsec.push_back((int)secs.size());
        tstart.push_back(st);
      }
      m.ntile = (int)tsec.size() - m.tile0;
      nmaxg = std::max(nmaxg, (int)std::min<int64_t>(D, std::min(c.lanc_niter, 512)));
      secs.push_back(m);
      tot += D;
      s1++;
    }
    const int nsec = (int)secs.size(), ntiles = (int)tsec.size();
    const int ld = nmaxg + 1;
    Arena ar;
    MsSector* d_secs;
    int* d_tsec;
    int64_t* d_tstart;
    char *x0, *x1, *x2;
    Ms64Bufs b{};
    b.ld = ld;
    int rc = VCA_OK;
    if ((rc = ar.alloc(&d_secs, nsec)) || (rc = ar.alloc(&d_tsec, ntiles)) || (rc = ar.alloc(&d_tstart, ntiles)) ||
        (rc = ar.alloc(&x0, (size_t)tot * es)) || (rc = ar.alloc(&x1, (size_t)tot * es)) ||
        (rc = ar.alloc(&x2, (size_t)tot * es)) || (rc = ar.alloc(&b.tpart, ntiles)) ||
        (rc = ar.alloc(&b.meta, nsec)) || (rc = ar.alloc(&b.alpha, nsec)) || (rc = ar.alloc(&b.bnow, nsec)) ||
        (rc = ar.alloc(&b.invb, nsec)) || (rc = ar.alloc(&b.A, (size_t)nsec * ld)) ||
        (rc = ar.alloc(&b.Bt, (size_t)nsec * ld)) || (rc = ar.alloc(&b.svec, (size_t)nsec * 5 * ld)) ||
        (rc = ar.alloc(&b.theta, nsec)) || (rc = ar.alloc(&b.resid, nsec)) || (rc = ar.alloc(&b.state, nsec)) ||
        (rc = ar.alloc(&b.mconv, nsec)) || (rc = ar.alloc(&b.undone, 1))) {
      ar.release();
      return rc;
    }
    b.X = x0;
    b.Xp = x1;
    b.Y = x2;
    std::vector<ChainMeta> meta(nsec);
    for (int q = 0; q < nsec; q++)
      meta[q] = ChainMeta{1, q, (int)std::min<int64_t>(secs[q].D, std::min(c.lanc_niter, 512)), 1, 0};
    cudaMemcpyAsync(d_secs, secs.data(), sizeof(MsSector) * nsec, cudaMemcpyHostToDevice, g->st);
    cudaMemcpyAsync(d_tsec, tsec.data(), sizeof(int) * ntiles, cudaMemcpyHostToDevice, g->st);
    cudaMemcpyAsync(d_tstart, tstart.data(), sizeof(int64_t) * ntiles, cudaMemcpyHostToDevice, g->st);
    cudaMemcpyAsync(b.meta, meta.data(), sizeof(ChainMeta) * nsec, cudaMemcpyHostToDevice, g->st);
    cudaMemsetAsync(b.A, 0, sizeof(double) * nsec * ld, g->st);
    cudaMemsetAsync(b.Bt, 0, sizeof(double) * nsec * ld, g->st);
    cudaMemsetAsync(b.bnow, 0, sizeof(double) * nsec, g->st);
    cudaMemsetAsync(b.state, 0, sizeof(int) * nsec, g->st);
    MsGroup gp{d_secs, d_tsec, d_tstart, nsec, ntiles};
    m64_launch_start(gp, cplx, c.start_seed, b, g->st);
    for (int k = 1; k <= nmaxg; k++) {
      m64_launch_step(gp, cplx, g->md, k, c.gs_beta_tol, b, g->st);
      if (k % std::max(1, c.gs_check_every) == 0 || k == nmaxg) {
        cudaMemsetAsync(b.undone, 0, sizeof(int), g->st);
        m64_launch_check(gp, b, c.gs_residual_tol, g->st);
        int undone = 0;
        cudaMemcpyAsync(&undone, b.undone, sizeof(int), cudaMemcpyDeviceToHost, g->st);
        CUCHK(cudaStreamSynchronize(g->st));
        if (undone == 0) break;
      }
    }
    CUCHK(cudaGetLastError());
    std::vector<double> th(nsec);
    cudaMemcpyAsync(th.data(), b.theta, sizeof(double) * nsec, cudaMemcpyDeviceToHost, g->st);
    CUCHK(cudaStreamSynchronize(g->st));
    for (int q = 0; q < nsec; q++) energy[secs[q].isector - 1] = th[q];
    ar.release();
    s0 = s1;
  }
  return VCA_OK;
}

// vca_diag_c at T=0 with LANC_METHOD="lanczos" (VCA_DIAG.f90:49-267)
// Finite T, one state per sector (LANC_METHOD="lanczos", Neigen = 1): the
// annealing sweeps of VCA_DIAG.f90:78-256 insert every sector's lowest state
// into a list capped at LANC_NSTATES_TOTAL (es_add_state_c with size,
// VCA_EIGENSPACE.f90:136-159: below the cap insert in energy order, else
// replace the last entry when lower) and stop once exp(-beta(emax-emin)) <
// cutoff; after each sweep vca_post_diag (VCA_DIAG.f90:357-363,:395-451)
// sums zeta over the list, then grows the cap by LANC_NSTATES_STEP or trims
// the entries past the cut-off and resets the cap to max(size,step)+step.
// Every sweep finds the same sector energies, so one pass computes them and
// the host replays the sweeps; eigenvectors are computed for the states left.
int diagonalize_finite_t() {
  const vca_config& c = g->cfg;
  std::vector<double> E(g->Nsectors, INFINITY);
  RCHK(g->fx ? batched_sector_energies(E) : batched_sector_energies_f64(E));
  g->sector_e = E;
  std::vector<ListEntry> lst;
  double zeta = 0.0, lo = 0.0;
  replay_finite_t(E, c, g->nstates_total, lst, zeta, lo);
  for (const ListEntry& x : lst) {
    double e;
    void* vec = nullptr;
    RCHK(g->fx ? sector_gs_fx(x.sector, &e, &vec, g->states) : sector_gs(x.sector, &e, &vec, g->states));
    if (std::fabs(e - x.e) > 1e-12 * std::max(1.0, std::fabs(e)))
      VFAIL(VCA_ERR_NUMERIC, "two Lanczos runs on the same sector disagree");
    g->gs.push_back({x.sector, x.e, vec});
  }
  g->egs = lo;
  g->zeta = zeta;
  return VCA_OK;
}

// ---------------------------------------------------------------------------
// LANC_METHOD="arpack" (the reference default; VCA_DIAG.f90:98-111,153-170):
// the k = min(dim, LANC_NSTATES_SECTOR) lowest eigenpairs of a sector.  Above
// LANC_DIM_THRESHOLD (and k < dim): a Lanczos with full reorthogonalisation
// (classical Gram-Schmidt twice per step) from the ground-state search's
// start vector, stopped when the k lowest Ritz pairs have
// |beta_{m+1} z_{m,q}| <= LANC_TOLERANCE max(1, |theta_q|) (tested every 5
// steps) or the Krylov space is exhausted; the Ritz vectors are V z_q.  At
// or below the threshold the dense H (H x v on the unit vectors) is
// diagonalised on the host, which returns whole degenerate multiplets as
// the reference's dense path does.  Vectors come back unit-norm in the
// solve's state storage: int64 at 2^-F on the fixed-point path, else FP64
// real or complex.
// ---------------------------------------------------------------------------
int sector_pairs(int isector, int k, std::vector<double>& e, std::vector<void*>& vecs, Arena& keep,
                 bool fp64_out = false) {
  const vca_config& c = g->cfg;
  const int nup = sec_nup(isector), ndw = sec_ndw(isector);
  SectorView sv = view_of(nup, ndw);
  const int64_t D = (int64_t)sv.dimup * sv.dimdw;
  const bool cplx = !g->real_model;
  const size_t es = cplx ? sizeof(double2) : sizeof(double);
  e.clear();
  vecs.clear();
  k = (int)std::min<int64_t>(k, D);
  if (k <= 0) return VCA_OK;
  auto emit = [&](const void* x) -> int {  // x: unit-norm FP64 vector on the device
    if (g->fx && !fp64_out) {
      i64* X;
      RCHK(keep.alloc(&X, (size_t)D));
      launch_fx_from_double(D, (const double*)x, g->fxs.F, X, g->st);
      vecs.push_back(X);
    } else {
      char* X;
      RCHK(keep.alloc(&X, (size_t)D * es));
      CUCHK(cudaMemcpyAsync(X, x, (size_t)D * es, cudaMemcpyDeviceToDevice, g->st));
      vecs.push_back(X);
    }
    return VCA_OK;
  };
  auto hxv1 = [&](const void* x, void* y, int m) {
    if (cplx) launch_hxv_cplx(sv, g->md, m, (const double2*)x, (double2*)y, g->st);
    else launch_hxv_real(sv, g->md, m, (const double*)x, (double*)y, g->st);
  };
  Arena ar;
  int rc = VCA_OK;
  const bool lanc_solve = k != D && D > std::max(c.lanc_dim_threshold, 1);
  if (!lanc_solve) {  // dense: H column by column, Jacobi on the host
    char *X, *Y;
    if ((rc = ar.alloc(&X, (size_t)D * D * es)) || (rc = ar.alloc(&Y, (size_t)D * D * es))) {
      ar.release();
      return rc;
    }
    std::vector<double> h((size_t)D * D * (es / sizeof(double)), 0.0);
    for (int64_t i = 0; i < D; i++) h[(size_t)(i * D + i) * (es / sizeof(double))] = 1.0;
    CUCHK(cudaMemcpyAsync(X, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, g->st));
    hxv1(X, Y, (int)D);  // Y[i*D + col] = H[i][col]
    CUCHK(cudaMemcpyAsync(h.data(), Y, h.size() * sizeof(double), cudaMemcpyDeviceToHost, g->st));
    CUCHK(cudaStreamSynchronize(g->st));
    std::vector<double> A(2 * (size_t)D * D, 0.0), w, Z;
    for (size_t t = 0; t < (size_t)D * D; t++) {
      A[2 * t] = cplx ? h[2 * t] : h[t];
      A[2 * t + 1] = cplx ? h[2 * t + 1] : 0.0;
    }
    if (!herm_eig((int)D, A.data(), w, Z)) { ar.release(); VFAIL(VCA_ERR_NUMERIC, "dense sector eigensolver did not converge"); }
    std::vector<double> xh((size_t)D * (es / sizeof(double)));
    for (int j = 0; j < k; j++) {
      for (int64_t i = 0; i < D; i++) {
        const double re = Z[2 * (i + (size_t)j * D)], im = Z[2 * (i + (size_t)j * D) + 1];
        if (cplx) { xh[2 * i] = re; xh[2 * i + 1] = im; }
        else xh[i] = re;  // a real symmetric H: Jacobi's rotations are real up to signs
      }
      CUCHK(cudaMemcpyAsync(X, xh.data(), xh.size() * sizeof(double), cudaMemcpyHostToDevice, g->st));
      if ((rc = emit(X))) { ar.release(); return rc; }
      CUCHK(cudaStreamSynchronize(g->st));
      e.push_back(w[j]);
    }
    ar.release();
    return VCA_OK;
  }
  const int mmax = (int)std::min<int64_t>(D, std::max(c.lanc_niter, 2 * k));
  char *V, *w, *partial, *cq;
  double* dz;
  if ((rc = ar.alloc(&V, (size_t)mmax * D * es))) {
    ar.release();
    VFAIL(VCA_ERR_ALLOC, "the arpack path stores " + std::to_string(mmax) + " Lanczos vectors of sector " +
                             std::to_string(isector) + " (" + std::to_string((size_t)mmax * D * es) +
                             " bytes); use lanc_method=lanczos");
  }
  if ((rc = ar.alloc(&w, (size_t)D * es)) || (rc = ar.alloc(&partial, (size_t)ap_partial_len(mmax) * es)) ||
      (rc = ar.alloc(&cq, (size_t)mmax * es)) || (rc = ar.alloc(&dz, (size_t)mmax))) {
    ar.release();
    return rc;
  }
  auto vec = [&](int j) { return V + (size_t)j * D * es; };
  auto dotr = [&](const void* x, const void* y, double* out) -> int {  // Re <x, y>
    launch_ap_proj(D, 1, cplx, x, y, partial, cq, g->st);
    CUCHK(cudaMemcpyAsync(out, cq, sizeof(double), cudaMemcpyDeviceToHost, g->st));
    CUCHK(cudaStreamSynchronize(g->st));
    return VCA_OK;
  };
  launch_start_vector(D, c.start_seed, isector, (double*)w, g->st);
  if (cplx) launch_real_to_cplx(D, (const double*)w, (double2*)vec(0), g->st);
  else CUCHK(cudaMemcpyAsync(vec(0), w, (size_t)D * es, cudaMemcpyDeviceToDevice, g->st));
  double n2 = 0.0;
  if ((rc = dotr(vec(0), vec(0), &n2))) { ar.release(); return rc; }
  if (!(n2 > 0.0)) { ar.release(); VFAIL(VCA_ERR_NUMERIC, "Lanczos start vector has zero norm"); }
  launch_ap_axpby(D, cplx, 0.0, -1.0 / std::sqrt(n2), vec(0), vec(0), g->st);
  std::vector<double> a, b(1, 0.0), theta, Zt;
  int m = 0;
  for (int j = 0; j < mmax; j++) {
    hxv1(vec(j), w, 1);
    if (j > 0) launch_ap_axpby(D, cplx, 1.0, b[j], vec(j - 1), w, g->st);
    double aj = 0.0;
    if ((rc = dotr(vec(j), w, &aj))) { ar.release(); return rc; }
    launch_ap_axpby(D, cplx, 1.0, aj, vec(j), w, g->st);
    for (int pass = 0; pass < 2; pass++) {
      launch_ap_proj(D, j + 1, cplx, V, w, partial, cq, g->st);
      launch_ap_orth(D, j + 1, cplx, V, cq, w, g->st);
    }
    double bb2 = 0.0;
    if ((rc = dotr(w, w, &bb2))) { ar.release(); return rc; }
    const double bj1 = std::sqrt(std::max(bb2, 0.0));
    a.push_back(aj);
    b.push_back(bj1);
    m = j + 1;
    const bool exhausted = bj1 <= c.gs_beta_tol * std::max(1.0, std::fabs(aj));
    if (exhausted || m == mmax) break;
    if (m >= k && m % 5 == 0) {
      if (!tridiag_eig(m, a.data(), b.data() + 1, theta, Zt)) { ar.release(); VFAIL(VCA_ERR_NUMERIC, "Ritz QL did not converge"); }
      bool conv = true;
      for (int q = 0; q < k && conv; q++)
        conv = std::fabs(bj1 * Zt[(m - 1) + (size_t)q * m]) <= c.lanc_tolerance * std::max(1.0, std::fabs(theta[q]));
      if (conv) break;
    }
    launch_ap_axpby(D, cplx, 0.0, -1.0 / bj1, w, vec(j + 1), g->st);
  }
  if (!tridiag_eig(m, a.data(), b.data() + 1, theta, Zt)) { ar.release(); VFAIL(VCA_ERR_NUMERIC, "Ritz QL did not converge"); }
  const int nk = std::min(k, m);
  for (int q = 0; q < nk; q++) {
    CUCHK(cudaMemcpyAsync(dz, Zt.data() + (size_t)q * m, sizeof(double) * m, cudaMemcpyHostToDevice, g->st));
    launch_ap_combine(D, m, cplx, V, dz, w, g->st);
    double nx = 0.0;
    if ((rc = dotr(w, w, &nx))) { ar.release(); return rc; }
    launch_ap_axpby(D, cplx, 0.0, -1.0 / std::sqrt(nx), w, w, g->st);
    if ((rc = emit(w))) { ar.release(); return rc; }
    CUCHK(cudaStreamSynchronize(g->st));
    e.push_back(theta[q]);
  }
  ar.release();
  return VCA_OK;
}

// T=0, LANC_METHOD="arpack": every sector's eigenpairs through the
// ground-state bookkeeping of VCA_DIAG.f90:224-236 (a level below the running
// zero by more than 10 GS_THRESHOLD restarts the list, one within
// GS_THRESHOLD joins it, inserted before the first entry with e <= its
// energy), sector by sector and, inside a sector, in ascending order.  Only
// sectors whose lowest level (the batched search) lies within 11
// GS_THRESHOLD of the minimum need their pairs: the minimum restarts the list
// below every level above that window whenever it comes, and after it no
// such level joins, so the list is the one of a scan of all pairs of all
// sectors.
int diagonalize_arpack_t0() {
  const vca_config& c = g->cfg;
  const double thr = c.gs_threshold;
  std::vector<double> eb;
  RCHK(g->fx ? batched_sector_energies(eb) : batched_sector_energies_f64(eb));
  double emin = INFINITY;
  for (double x : eb) emin = std::min(emin, x);
  std::vector<std::vector<double>> E(g->Nsectors);
  std::vector<std::vector<void*>> X(g->Nsectors);
  Arena keep;
  for (int isector = 1; isector <= g->Nsectors; isector++) {
    const int64_t D = (int64_t)g->dimn[sec_nup(isector)] * g->dimn[sec_ndw(isector)];
    if (eb[isector - 1] <= emin + 11.0 * thr) {
      const int k = (int)std::min<int64_t>(D, std::max(1, c.lanc_nstates_sector));
      const int rc = sector_pairs(isector, k, E[isector - 1], X[isector - 1], keep);
      if (rc) { keep.release(); return rc; }
    }
    if (E[isector - 1].empty()) {  // outside the window: its lowest level stands for the sector
      E[isector - 1].assign(1, eb[isector - 1]);
      X[isector - 1].assign(1, nullptr);
    }
    g->sector_e[isector - 1] = E[isector - 1][0];
  }
  struct Entry {
    double e;
    int sector, idx;
  };
  std::vector<Entry> list;
  double oldzero = 1000.0;
  for (int isector = 1; isector <= g->Nsectors; isector++)
    for (int i = 0; i < (int)E[isector - 1].size(); i++) {
      const double en = E[isector - 1][i];
      if (en < oldzero - 10.0 * thr) {
        oldzero = en;
        list.assign(1, Entry{en, isector, i});
      } else if (std::fabs(en - oldzero) <= thr) {
        oldzero = std::min(oldzero, en);
        auto it = list.begin();
        while (it != list.end() && !(en <= it->e)) ++it;
        list.insert(it, Entry{en, isector, i});
      }
    }
  g->states.release();
  g->gs.clear();
  for (const Entry& x : list) {
    void* v = X[x.sector - 1][x.idx];
    if (!v) { keep.release(); VFAIL(VCA_ERR_NUMERIC, "a level outside the screened window entered the state list"); }
    g->gs.push_back(GState{x.sector, x.e, v});
  }
  g->states.ptrs = keep.ptrs;
  g->egs = INFINITY;
  for (auto& st : g->gs) g->egs = std::min(g->egs, st.e);
  g->zeta = (double)g->gs.size();  // VCA_DIAG.f90:363
  return VCA_OK;
}

// Finite T, LANC_METHOD="arpack": the annealing sweeps of VCA_DIAG.f90:
// 78-256 with Neigen = min(dim, neigen_sector) eigenpairs of every sector in
// the capped list (es_add_state_c with size, VCA_EIGENSPACE.f90:136-159),
// then vca_post_diag (:357-451): zeta over the whole list; neigen_sector + 1
// for sectors in the list and - 1 for the others, at most the sector's count
// in the list + 1 and at least 1 (:411-437); the cap grows by
// LANC_NSTATES_STEP, or the list is trimmed at the cut-off and the cap reset
// to max(size, step) + step.  A sector's pairs are computed again only when a
// sweep asks for more of them.
int diagonalize_arpack_finite_t() {
  const vca_config& c = g->cfg;
  const int ns = g->Nsectors;
  auto dim = [&](int isector) { return (int64_t)g->dimn[sec_nup(isector)] * g->dimn[sec_ndw(isector)]; };
  if ((int)g->neigen.size() != ns) {
    g->neigen.resize(ns);
    for (int i = 0; i < ns; i++) g->neigen[i] = (int)std::min<int64_t>(dim(i + 1), std::max(1, c.lanc_nstates_sector));
  }
  std::vector<std::vector<double>> E(ns);
  std::vector<std::vector<void*>> X(ns);
  std::vector<int> have(ns, -1);
  Arena keep;
  struct Entry {
    int sector, idx;
  };
  std::vector<Entry> list;
  auto en = [&](const Entry& x) { return E[x.sector - 1][x.idx]; };
  double emin = DBL_MAX, emax = -DBL_MAX, zeta = 0.0;
  auto insert = [&](Entry x) {  // es_insert_state_c (:167-216): before the first entry with e >= its energy
    const double ev = en(x);
    size_t pos = 0;
    while (pos < list.size() && !(ev <= en(list[pos]))) pos++;
    list.insert(list.begin() + pos, x);
    if (ev > emax) emax = ev;
    if (ev < emin) emin = ev;
  };
  auto pop = [&]() {  // es_pop_state (:230-312): the last entry
    list.pop_back();
    if (!list.empty()) {
      emax = en(list.back());
      emin = en(list.front());
    }
  };
  bool converged = false;
  for (int iter = 0; !converged && iter < c.lanc_niter_spectrum; iter++) {
    for (int isector = 1; isector <= ns; isector++)
      if (have[isector - 1] < g->neigen[isector - 1]) {
        std::vector<void*> v;
        const int rc = sector_pairs(isector, g->neigen[isector - 1], E[isector - 1], v, keep);
        if (rc) { keep.release(); return rc; }
        X[isector - 1] = v;
        have[isector - 1] = g->neigen[isector - 1];
      }
    list.clear();
    emin = DBL_MAX;
    emax = -DBL_MAX;
    for (int isector = 1; isector <= ns; isector++) {
      const int ne = std::min(g->neigen[isector - 1], (int)E[isector - 1].size());
      for (int i = 0; i < ne; i++) {
        const Entry x{isector, i};
        if ((int)list.size() < g->nstates_total) insert(x);
        else if (en(x) < en(list.back())) { pop(); insert(x); }
      }
    }
    converged = std::exp(-c.beta * (emax - emin)) < c.cutoff;  // VCA_DIAG.f90:251-256
    zeta = 0.0;
    for (const Entry& x : list) zeta += std::exp(-c.beta * (en(x) - emin));
    std::vector<int> count(ns, 0);
    for (const Entry& x : list) count[x.sector - 1]++;
    for (int i = 0; i < ns; i++) {
      int& ne = g->neigen[i];
      ne += count[i] > 0 ? 1 : -1;
      if (ne > count[i]) ne = count[i] + 1;
      if (ne <= 0) ne = 1;
    }
    if (std::exp(-c.beta * (emax - emin)) > c.cutoff) {
      g->nstates_total += c.lanc_nstates_step;
    } else {
      double Ei = en(list.back());
      while (std::exp(-c.beta * (Ei - emin)) <= c.cutoff) {
        pop();
        Ei = en(list.back());
      }
      g->nstates_total = std::max((int)list.size(), c.lanc_nstates_step) + c.lanc_nstates_step;
    }
  }
  for (int isector = 1; isector <= ns; isector++)
    if (!E[isector - 1].empty()) g->sector_e[isector - 1] = E[isector - 1][0];
  g->states.release();
  g->gs.clear();
  for (const Entry& x : list) g->gs.push_back(GState{x.sector, en(x), X[x.sector - 1][x.idx]});
  g->states.ptrs = keep.ptrs;
  g->egs = emin;
  g->zeta = zeta;
  return VCA_OK;
}

int diagonalize() {
  const vca_config& c = g->cfg;
  g->states.release();
  g->gs.clear();
  g->sector_e.assign(g->Nsectors, INFINITY);
  if (c.lanc_method != VCA_LANC_LANCZOS) return g->finiteT ? diagonalize_arpack_finite_t() : diagonalize_arpack_t0();
  if (g->finiteT) return diagonalize_finite_t();
  double oldzero = 1000.0;
  const double thr = c.gs_threshold;
  // every sector's energy from the batched search (fixed point or FP64), then
  // the T=0 list below needs vectors only for the sectors it keeps
  std::vector<double> eb;
  std::vector<char> keep_sec(g->Nsectors + 1, 1);
  {
    if (c.sector_at_a_time) {  // the reference's loop, one sector per Lanczos run
      eb.assign(g->Nsectors, INFINITY);
      for (int isector = 1; isector <= g->Nsectors; isector++) {
        double e;
        void* vec = nullptr;
        Arena tmp;
        const int rc = g->fx ? sector_gs_fx(isector, &e, &vec, tmp) : sector_gs(isector, &e, &vec, tmp);
        tmp.release();
        if (rc) return rc;
        eb[isector - 1] = e;
      }
    } else {
      RCHK(g->fx ? batched_sector_energies(eb) : batched_sector_energies_f64(eb));
    }
    std::vector<ListEntry> lst;
    replay_t0(eb, thr, lst);
    std::fill(keep_sec.begin(), keep_sec.end(), 0);
    for (const ListEntry& q : lst) keep_sec[q.sector] = 1;
  }
  for (int isector = 1; isector <= g->Nsectors; isector++) {
    double e;
    void* vec = nullptr;
    Arena tmp;
    if (!keep_sec[isector]) {
      g->sector_e[isector - 1] = eb[isector - 1];
      const double ee = eb[isector - 1];  // advance the running minimum exactly as below
      if (ee < oldzero - 10.0 * thr) { oldzero = ee; g->states.release(); g->gs.clear(); }
      else if (std::fabs(ee - oldzero) <= thr) oldzero = std::min(oldzero, ee);
      continue;
    }
    RCHK(g->fx ? sector_gs_fx(isector, &e, &vec, tmp) : sector_gs(isector, &e, &vec, tmp));
    // the same recurrence and stopping rule: the two runs agree
    if (std::fabs(e - eb[isector - 1]) > 1e-12 * std::max(1.0, std::fabs(e))) {
      tmp.release();
      VFAIL(VCA_ERR_NUMERIC, "batched and single-sector Lanczos disagree");
    }
    g->sector_e[isector - 1] = e;
    // T=0 bookkeeping (VCA_DIAG.f90:224-236), list ordered by energy
    // (es_insert_state_c, VCA_EIGENSPACE.f90:167-216)
    if (e < oldzero - 10.0 * thr) {
      oldzero = e;
      g->states.release();
      g->gs.clear();
      g->states.ptrs = tmp.ptrs;
      g->gs.push_back({isector, e, vec});
    } else if (std::fabs(e - oldzero) <= thr) {
      oldzero = std::min(oldzero, e);
      for (void* p : tmp.ptrs) g->states.ptrs.push_back(p);
      auto it = g->gs.begin();
      while (it != g->gs.end() && !(e <= it->e)) ++it;
      g->gs.insert(it, GState{isector, e, vec});
    } else {
      tmp.release();
    }
  }
  g->egs = INFINITY;
  for (auto& s : g->gs) g->egs = std::min(g->egs, s.e);
  g->zeta = (double)g->gs.size();  // VCA_DIAG.f90:363
  return VCA_OK;
}

// ---------------------------------------------------------------------------
// Green's function chains (build_gf_normal, VCA_GF_NORMAL.f90:37-104): every
// chain of one (state, spin, particle|hole) target sector runs as one column
// batch; batches are split to fit device memory.
// ---------------------------------------------------------------------------
struct ChainSpec {
  ChainInit ci;
  ChainRec rec;
  int isign;
  cd wfac;
  int ncol;
};

// Boltzmann factor of a state's chains (VCA_GF_NORMAL.f90:987-993): 1 at
// T=0; exp(-beta(Ei-Egs)) at finite T, 0 once beta(Ei-Egs) >= 200
double state_weight(const GState& S) {
  if (!g->finiteT) return 1.0;
  const double x = g->cfg.beta * (S.e - g->egs);
  return x < 200.0 ? std::exp(-x) : 0.0;
}

double now_ms();

// One column batch of Green's-function chains: the chains of one (state,
// spin, particle|hole) target sector whose columns fit, on its own stream.
struct ChainGroup {
  int state = 0, spin = 0;
  bool dag = false;
  std::vector<ChainSpec>* specs = nullptr;
  size_t q0 = 0, q1 = 0;
  int tup = 0, tdw = 0, m = 0, nch = 0, nlanc = 0;
  int64_t D = 0;
  bool swap = false;
  SectorView tv{}, hv{};
  FxView hf{};
  Arena ar;
  BatchBufs bb{};
  double *norm2c = nullptr, *norm2 = nullptr, *invn = nullptr;
  ChainInit* d_ci = nullptr;
  int* d_isign = nullptr;
  double2* d_wfac = nullptr;
  ColBatch cb{};
  cudaStream_t st = nullptr;
};

// Cut the chains of one (state, spin, particle|hole) list into column groups
// whose three column buffers fit 1/npar of half the free device memory (npar
// groups run at a time).
int chain_groups(int state, int spin, bool dag, std::vector<ChainSpec>& specs, int npar,
                 std::vector<ChainGroup>& out) {
  const vca_config& c = g->cfg;
  const GState& S = g->gs[state];
  const int nup = sec_nup(S.sector), ndw = sec_ndw(S.sector);
  const int tup = nup + (spin == 0 ? (dag ? 1 : -1) : 0);
  const int tdw = ndw + (spin == 1 ? (dag ? 1 : -1) : 0);
  if (tup < 0 || tup > g->Ns || tdw < 0 || tdw > g->Ns) return VCA_OK;  // no target sector
  const SectorView tv = view_of(tup, tdw);
  const int64_t D = (int64_t)tv.dimup * tv.dimdw;
  const bool cplx = !g->real_model;
  const size_t es = cplx ? sizeof(double2) : sizeof(double);
  size_t freeb = 0, totb = 0;
  CUCHK(cudaMemGetInfo(&freeb, &totb));
  const size_t budget = (size_t)(0.5 * (double)freeb / std::max(1, npar));
  int64_t maxcols = (int64_t)(budget / (3 * (size_t)D * es + 1));
  if (g->fx && maxcols > FX_SLAB) maxcols = maxcols / FX_SLAB * FX_SLAB;  // room for the pad columns
  if (maxcols < 2) VFAIL(VCA_ERR_ALLOC, "not enough device memory for one Green's function chain");
  size_t q0 = 0;
  while (q0 < specs.size()) {
    size_t q1 = q0;
    int m = 0;
    while (q1 < specs.size() && m + specs[q1].ncol <= maxcols) { m += specs[q1].ncol; q1++; }
    ChainGroup G;
    G.state = state;
    G.spin = spin;
    G.dag = dag;
    G.specs = &specs;
    G.q0 = q0;
    G.q1 = q1;
    G.tup = tup;
    G.tdw = tdw;
    G.m = m;
    G.nch = (int)(q1 - q0);
    G.D = D;
    G.nlanc = (int)std::min<int64_t>(D, c.lanc_ngfiter);
    G.tv = tv;
    out.push_back(G);
    q0 = q1;
  }
  return VCA_OK;
}

// allocations, tables and the normalised start vectors of a group, on G.st
int chain_group_prepare(ChainGroup& G) {
  const GState& S = g->gs[G.state];
  const int nup = sec_nup(S.sector);
  const bool cplx = !g->real_model;
  const int m = G.m, nch = G.nch;
  int rc = alloc_batch(G.ar, G.D, m, cplx, nch, g->ld, G.bb);
  BatchBufs& bb = G.bb;
  // fixed-point batches hold the smaller spin block first (see view_pair),
  // its rows in hop-count order where the position-ordered H x v applies
  G.swap = g->fx && G.tv.dimup > G.tv.dimdw;
  G.hv = G.swap ? view_pair(g->dwset, G.tdw, 0, G.tup) : G.tv;
  if (g->fx) {
    G.hf = G.swap ? fx_view_pair(g->dwset, G.tdw, 0, G.tup) : fx_view_of(G.tup, G.tdw);
    G.hf.rows_permuted = (g->cfg.hxv_variant != 1 && hxv_fx_r_ok(G.hv, G.hf, m)) ? 1 : 0;
  }
  if (!rc && g->fx) {
    const int rbw = hxv_fx_cols_rows(G.hv, G.hf, m, g->cfg.hxv_variant == 1);
    rc = G.ar.alloc(&bb.wpart, 2 * (size_t)rbw * m);
    bb.wpart_rows = rbw;
  }
  if (!rc) rc = G.ar.alloc(&G.norm2c, m);
  if (!rc) rc = G.ar.alloc(&G.norm2, nch);
  if (!rc) rc = G.ar.alloc(&G.invn, nch);
  if (!rc) rc = G.ar.alloc(&G.d_ci, nch);
  if (!rc) rc = G.ar.alloc(&G.d_isign, nch);
  if (!rc) rc = G.ar.alloc(&G.d_wfac, nch);
  if (rc) return rc;
  std::vector<ChainMeta> meta(nch);
  std::vector<int> col2ch(m);
  std::vector<ChainInit> ci(nch);
  std::vector<int> isg(nch);
  std::vector<double2> wf(nch);
  int col = 0;
  for (int q = 0; q < nch; q++) {
    ChainSpec& sp = (*G.specs)[G.q0 + q];
    sp.ci.col0 = col;
    ci[q] = sp.ci;
    meta[q] = ChainMeta{sp.ncol, col, G.nlanc, 1, 0};
    for (int t = 0; t < sp.ncol; t++) col2ch[col + t] = q;
    col += sp.ncol;
    isg[q] = sp.isign;
    wf[q] = make_double2(sp.wfac.real(), sp.wfac.imag());
  }
  cudaStream_t st = G.st;
  CUCHK(cudaMemcpyAsync(bb.meta, meta.data(), sizeof(ChainMeta) * nch, cudaMemcpyHostToDevice, st));
  CUCHK(cudaMemcpyAsync(bb.col2ch, col2ch.data(), sizeof(int) * m, cudaMemcpyHostToDevice, st));
  CUCHK(cudaMemcpyAsync(G.d_ci, ci.data(), sizeof(ChainInit) * nch, cudaMemcpyHostToDevice, st));
  CUCHK(cudaMemcpyAsync(G.d_isign, isg.data(), sizeof(int) * nch, cudaMemcpyHostToDevice, st));
  CUCHK(cudaMemcpyAsync(G.d_wfac, wf.data(), sizeof(double2) * nch, cudaMemcpyHostToDevice, st));
  G.cb = ColBatch{G.D, m, cplx, nch, bb.col2ch, bb.meta};
  const ColBatch& cb = G.cb;
  // start vectors: gather from the ground state, normalise per chain
  if (g->fx) {
    const FxScales& fs = g->fxs;
    launch_chain_init_fx(G.tv, g->sp[0][nup].dim, (const i64*)S.vec, nch, G.d_ci, m, G.swap,
                         G.hf.rows_permuted ? G.hf.up_pinv : nullptr, (i64*)bb.b[0], st);
    launch_fx_dot(cb, (i64*)bb.b[0], (i64*)bb.b[0], fs.F, fs.F, (i64*)bb.partial, bb.nblk, G.norm2c, st);
    launch_chain_sum(cb, G.norm2c, G.norm2, st);
    launch_chain_norm_init(nch, bb.meta, G.norm2, G.invn, st);
    launch_fx_rescale(cb, G.invn, fs.F, fs.F, (i64*)bb.b[0], (i64*)bb.b[0], bb.scr, st);
  } else {
    launch_chain_init(G.tv, g->sp[0][nup].dim, S.vec, cplx, nch, G.d_ci, m, cplx, bb.b[0], st);
    launch_col_dot(cb, bb.b[0], bb.b[0], bb.partial, bb.nblk, G.norm2c, st);
    launch_chain_sum(cb, G.norm2c, G.norm2, st);
    launch_chain_norm_init(nch, bb.meta, G.norm2, G.invn, st);
    launch_col_scale(cb, G.invn, bb.b[0], bb.b[0], st);
  }
  CUCHK(cudaGetLastError());
  return VCA_OK;
}

int chain_group_step(ChainGroup& G, int k) {
  const vca_config& c = g->cfg;
  if (g->fx) return lanczos_step_fx(G.hv, G.hf, G.cb, G.bb, k, c.gf_beta_tol, g->ld, G.st);
  return lanczos_step(G.tv, G.cb, G.bb, k, c.gf_beta_tol, g->ld, G.st);
}

// poles and weights into the global chain table, after every earlier group
int chain_group_finish(ChainGroup& G) {
  const GState& S = g->gs[G.state];
  const int base = (int)g->chains.size();
  launch_chain_store(G.nch, G.bb.meta, G.bb.A, G.bb.Bt, g->ld, G.norm2, G.d_wfac, G.d_isign, S.e, state_weight(S),
                     g->zeta, g->cstore, base, G.st);
  CUCHK(cudaGetLastError());
  CUCHK(cudaStreamSynchronize(G.st));
  for (int q = 0; q < G.nch; q++) {
    g->chains.push_back((*G.specs)[G.q0 + q].rec);
    g->chains.back().nlanc = G.nlanc;
  }
  G.ar.release();
  return VCA_OK;
}

// The groups npar at a time, each on its own stream, their steps
// interleaved so one group's H x v overlaps the other's element passes;
// every group computes exactly what it computes alone.
int run_chain_groups(std::vector<ChainGroup>& groups, int npar) {
  CUCHK(cudaStreamSynchronize(g->st));  // ground states and the chain store are in place
  cudaStream_t streams[2] = {g->st, g->st2};
  for (size_t i = 0; i < groups.size(); i += (size_t)npar) {
    const size_t j1 = std::min(groups.size(), i + (size_t)npar);
    auto release = [&]() { for (size_t j = i; j < j1; j++) groups[j].ar.release(); };
    const double tb0 = now_ms();
    int kmax = 0;
    for (size_t j = i; j < j1; j++) {
      groups[j].st = streams[(j - i) % 2];
      const int rc = chain_group_prepare(groups[j]);
      if (rc) { release(); return rc; }
      kmax = std::max(kmax, groups[j].nlanc);
    }
    for (size_t j = i; j < j1; j++) CUCHK(cudaStreamSynchronize(groups[j].st));
    const double tb1 = now_ms();
    for (int k = 1; k <= kmax; k++)
      for (size_t j = i; j < j1; j++)
        if (k <= groups[j].nlanc) {
          const int rc = chain_group_step(groups[j], k);
          if (rc) { release(); return rc; }
        }
    for (size_t j = i; j < j1; j++) {
      const int rc = chain_group_finish(groups[j]);
      if (rc) { release(); return rc; }
    }
    g->chain_ms[0] += tb1 - tb0;
    g->chain_ms[1] += now_ms() - tb1;
    g->chain_ms[2] += (double)(j1 - i);
  }
  return VCA_OK;
}

int count_chains() {
  const vca_config& c = g->cfg;
  const int L = c.Nlat * c.Norb;
  const int per = c.vca_gf_symmetric ? 2 : 4;
  return (int)g->gs.size() * c.Nspin * (2 * L + per * L * (L - 1));
}

int build_gf() {
  const vca_config& c = g->cfg;
  g->gf.release();
  g->chains.clear();
  for (double& t : g->chain_ms) t = 0.0;
  g->ld = std::max(1, c.lanc_ngfiter);
  const int nmax = count_chains();
  RCHK(g->gf.alloc(&g->d_poles, (size_t)nmax * g->ld));
  RCHK(g->gf.alloc(&g->d_weights, (size_t)nmax * g->ld));
  RCHK(g->gf.alloc(&g->d_nexc, nmax));
  CUCHK(cudaMemsetAsync(g->d_nexc, 0, sizeof(int) * nmax, g->st));
  g->poles_ready = false;
  ChainStore& cs = g->cstore;
  cs.ld = g->ld;
  RCHK(g->gf.alloc(&cs.A, (size_t)nmax * g->ld));
  RCHK(g->gf.alloc(&cs.B, (size_t)nmax * g->ld));
  RCHK(g->gf.alloc(&cs.n, nmax));
  RCHK(g->gf.alloc(&cs.pes, nmax));
  RCHK(g->gf.alloc(&cs.isign, nmax));
  RCHK(g->gf.alloc(&cs.wfac, nmax));
  RCHK(g->gf.alloc(&cs.Ei, nmax));
  CUCHK(cudaMemsetAsync(cs.n, 0, sizeof(int) * nmax, g->st));
  const bool cplx = !g->real_model;
  const cd XI(0.0, 1.0);
  const int npar = std::max(1, std::min(2, g->chain_streams));
  std::vector<std::vector<ChainSpec>> speclists;
  speclists.reserve(2 * g->gs.size() * (size_t)c.Nspin);  // the groups point into them
  std::vector<ChainGroup> groups;
  for (int k = 0; k < (int)g->gs.size(); k++)
    for (int is = 0; is < c.Nspin; is++) {
      speclists.emplace_back();
      std::vector<ChainSpec>& part = speclists.back();
      speclists.emplace_back();
      std::vector<ChainSpec>& hole = speclists.back();
      auto add = [&](std::vector<ChainSpec>& v, int dag, int e, int chan, int p, cd cp, int q, cd cq,
                     int nterm, cd wfac) {
        ChainSpec s{};
        s.ci.spin = is;
        s.ci.dag = dag;
        s.ci.nterm = nterm;
        s.ci.t[0] = OpTerm{p, cp.real(), cp.imag()};
        s.ci.t[1] = OpTerm{q, cq.real(), cq.imag()};
        const bool imagcoef = (cp.imag() != 0.0) || (nterm > 1 && cq.imag() != 0.0);
        s.ci.cplxcol = (!cplx && imagcoef) ? 1 : 0;
        s.ncol = cplx ? 1 : (imagcoef ? 2 : 1);
        s.rec = ChainRec{e, k, chan};
        s.isign = dag ? 1 : -1;
        s.wfac = wfac;
        v.push_back(s);
      };
      for (int io = 0; io < c.Norb; io++)
        for (int il = 0; il < c.Nlat; il++) {
          const int p = io + il * c.Norb;
          const int ed = elem_index(c, il, il, is, io, io);
          add(part, 1, ed, 1, p, 1.0, 0, 0.0, 1, 1.0);  // VCA_GF_NORMAL.f90:121-318
          add(hole, 0, ed, 2, p, 1.0, 0, 0.0, 1, 1.0);
          for (int jl = 0; jl < c.Nlat; jl++)
            for (int jo = 0; jo < c.Norb; jo++) {
              if (il == jl && io == jo) continue;
              const int q = jo + jl * c.Norb;
              const int e = elem_index(c, il, jl, is, io, jo);
              add(part, 1, e, 1, p, 1.0, q, 1.0, 2, 1.0);
              add(hole, 0, e, 2, p, 1.0, q, 1.0, 2, 1.0);
              if (!c.vca_gf_symmetric) {  // chan4 (VCA_GF_NORMAL.f90:561-958)
                add(part, 1, e, 3, p, 1.0, q, XI, 2, -XI);
                add(hole, 0, e, 4, p, 1.0, q, -XI, 2, -XI);
              }
            }
        }
      RCHK(chain_groups(k, is, true, part, npar, groups));
      RCHK(chain_groups(k, is, false, hole, npar, groups));
    }
  RCHK(run_chain_groups(groups, npar));
  // element -> chains CSR
  g->nelem = c.Nlat * c.Nlat * c.Nspin * c.Norb * c.Norb;
  std::vector<std::vector<int>> lists(g->nelem);
  for (int ch = 0; ch < (int)g->chains.size(); ch++) lists[g->chains[ch].elem].push_back(ch);
  std::vector<int> ptr(g->nelem + 1, 0), flat;
  for (int e = 0; e < g->nelem; e++) {
    ptr[e + 1] = ptr[e] + (int)lists[e].size();
    flat.insert(flat.end(), lists[e].begin(), lists[e].end());
  }
  RCHK(g->gf.alloc(&g->d_elem_ptr, ptr.size()));
  RCHK(g->gf.alloc(&g->d_elem_chain, std::max<size_t>(1, flat.size())));
  CUCHK(cudaMemcpyAsync(g->d_elem_ptr, ptr.data(), sizeof(int) * ptr.size(), cudaMemcpyHostToDevice, g->st));
  if (!flat.empty())
    CUCHK(cudaMemcpyAsync(g->d_elem_chain, flat.data(), sizeof(int) * flat.size(), cudaMemcpyHostToDevice, g->st));
  CUCHK(cudaStreamSynchronize(g->st));
  return VCA_OK;
}

// Poles and weights of every chain from the chain store, once per solve
int ensure_poles() {
  if (g->poles_ready || g->chains.empty()) return VCA_OK;
  Arena ar;
  double* work;
  int* d_fail;
  const int nch = (int)g->chains.size();
  RCHK(ar.alloc(&work, (size_t)nch * 3 * g->ld));
  RCHK(ar.alloc(&d_fail, 1));
  CUCHK(cudaMemsetAsync(d_fail, 0, sizeof(int), g->st));
  launch_chain_poles(nch, g->cstore, work, g->d_poles, g->d_weights, g->d_nexc, g->ql_max_iter, d_fail, g->st);
  int nfail = 0;
  cudaError_t err = cudaMemcpyAsync(&nfail, d_fail, sizeof(int), cudaMemcpyDeviceToHost, g->st);
  if (err == cudaSuccess) err = cudaStreamSynchronize(g->st);
  ar.release();
  CUCHK(err);
  if (nfail > 0)
    VFAIL(VCA_ERR_NUMERIC, "tridiagonal QL of " + std::to_string(nfail) + " Green's function chain(s) did not converge");
  g->poles_ready = true;
  return VCA_OK;
}

GfLayout gf_layout() {
  GfLayout gl;
  gl.nelem = g->nelem;
  gl.elem_ptr = g->d_elem_ptr;
  gl.elem_chain = g->d_elem_chain;
  gl.cs = g->cstore;
  return gl;
}

// G'(z) in lso layout for nz device points, from the tables vca_gf_cluster
// would use: a GFmatrix read by read_gfprime while one is loaded, else the
// solve's chains (solve_tables = true: always the solve's, as the grids that
// build_gf_normal accumulates)
int gf_lso(int nz, const double2* d_z, double2* d_Glso, Arena& ar, bool solve_tables = false) {
  const vca_config& c = g->cfg;
  const int nelem = c.Nlat * c.Nlat * c.Nspin * c.Norb * c.Norb;
  double2* raw;
  RCHK(ar.alloc(&raw, (size_t)nz * nelem));
  if (g->gfm_loaded && !solve_tables)
    launch_gf_eval_poles(nelem, g->d_gfm_ptr, g->d_gfm_p, g->d_gfm_w, nz, d_z, raw, g->st);
  else
    launch_gf_eval(gf_layout(), nz, d_z, raw, g->st);
  ClusterDims cdm{c.Nlat, c.Norb, c.Nspin, g->N, c.vca_gf_symmetric ? 0 : 1};
  launch_gf_assemble(cdm, nz, raw, d_Glso, g->st);
  CUCHK(cudaGetLastError());
  return VCA_OK;
}

// Bath matrices in lso layout (VCA_AUX_FUNX.f90:255-279, :445-468)
void bath_lso(std::vector<double2>& hb, std::vector<double2>& V) {
  const vca_config& c = g->cfg;
  const int N = g->N, Nb = g->Nb;
  hb.assign((size_t)Nb * Nb, make_double2(0, 0));
  V.assign((size_t)N * Nb, make_double2(0, 0));
  for (int a = 0; a < c.Nlat_bath; a++)
    for (int b = 0; b < c.Nlat_bath; b++)
      for (int is = 0; is < c.Nspin; is++)
        for (int js = 0; js < c.Nspin; js++)
          for (int oa = 0; oa < c.Norb_bath; oa++)
            for (int ob = 0; ob < c.Norb_bath; ob++) {
              int r = oa + a * c.Norb_bath + is * c.Norb_bath * c.Nlat_bath;
              int q = ob + b * c.Norb_bath + js * c.Norb_bath * c.Nlat_bath;
              cd h = g->bath_h[idx_bh(c, a, b, is, js, oa, ob)];
              hb[r + (size_t)q * Nb] = make_double2(h.real(), h.imag());
            }
  for (int il = 0; il < c.Nlat; il++)
    for (int b = 0; b < c.Nlat_bath; b++)
      for (int is = 0; is < c.Nspin; is++)
        for (int js = 0; js < c.Nspin; js++)
          for (int io = 0; io < c.Norb; io++)
            for (int ob = 0; ob < c.Norb_bath; ob++) {
              int r = io + il * c.Norb + is * c.Norb * c.Nlat;
              int q = ob + b * c.Norb_bath + js * c.Norb_bath * c.Nlat_bath;
              cd v = g->bath_v[idx_bv(c, il, b, is, js, io, ob)];
              V[r + (size_t)q * N] = make_double2(v.real(), v.imag());
            }
}

// spin-block structure of the Omega matrices (all spin-off-diagonal blocks 0)
bool hk_spin_diagonal(const double* Hk, int64_t Nk) {
  const vca_config& c = g->cfg;
  if (c.Nspin == 1) return true;
  const size_t nel = hloc_len(c);
  for (int il = 0; il < c.Nlat; il++)
    for (int jl = 0; jl < c.Nlat; jl++)
      for (int io = 0; io < c.Norb; io++)
        for (int jo = 0; jo < c.Norb; jo++)
          for (int s = 0; s < 2; s++) {
            int64_t x = idx_nnn(c, il, jl, s, 1 - s, io, jo);
            for (int64_t k = 0; k < Nk; k++)
              if (Hk[2 * (k * nel + x)] != 0.0 || Hk[2 * (k * nel + x) + 1] != 0.0) return false;
          }
  return true;
}
bool point_spin_diagonal() {
  const vca_config& c = g->cfg;
  if (c.Nspin == 1) return true;
  for (int il = 0; il < c.Nlat; il++)
    for (int jl = 0; jl < c.Nlat; jl++)
      for (int io = 0; io < c.Norb; io++)
        for (int jo = 0; jo < c.Norb; jo++)
          for (int s = 0; s < 2; s++)
            if (g->Hloc[idx_nnn(c, il, jl, s, 1 - s, io, jo)] != 0.0) return false;
  if (g->has_bath) {
    for (int a = 0; a < c.Nlat_bath; a++)
      for (int b = 0; b < c.Nlat_bath; b++)
        for (int oa = 0; oa < c.Norb_bath; oa++)
          for (int ob = 0; ob < c.Norb_bath; ob++)
            for (int s = 0; s < 2; s++)
              if (g->bath_h[idx_bh(c, a, b, s, 1 - s, oa, ob)] != 0.0) return false;
    for (int il = 0; il < c.Nlat; il++)
      for (int b = 0; b < c.Nlat_bath; b++)
        for (int io = 0; io < c.Norb; io++)
          for (int ob = 0; ob < c.Norb_bath; ob++)
            for (int s = 0; s < 2; s++)
              if (g->bath_v[idx_bv(c, il, b, s, 1 - s, io, ob)] != 0.0) return false;
  }
  return true;
}

// Omega integral (frequency_integration, VCA_OMEGA.f90:123-146) with the
// fixed Gauss-Legendre rule; also returns f(w) at the nodes when asked.
// The Omega integrand is equal at k and its conjugate partner when the model
// is real and Hloc, bath_h are symmetric with a real bath_v (P and G'
// symmetric; see pair_kpoints).
bool omega_pairs_valid() {
  const vca_config& c = g->cfg;
  if (!g->real_model) return false;
  for (int il = 0; il < c.Nlat; il++)
    for (int jl = 0; jl < c.Nlat; jl++)
      for (int is = 0; is < c.Nspin; is++)
        for (int js = 0; js < c.Nspin; js++)
          for (int io = 0; io < c.Norb; io++)
            for (int jo = 0; jo < c.Norb; jo++) {
              const cd a = g->Hloc[idx_nnn(c, il, jl, is, js, io, jo)];
              if (a.imag() != 0.0 || a != g->Hloc[idx_nnn(c, jl, il, js, is, jo, io)]) return false;
            }
  if (g->has_bath) {
    for (int a = 0; a < c.Nlat_bath; a++)
      for (int b = 0; b < c.Nlat_bath; b++)
        for (int is = 0; is < c.Nspin; is++)
          for (int js = 0; js < c.Nspin; js++)
            for (int oa = 0; oa < c.Norb_bath; oa++)
              for (int ob = 0; ob < c.Norb_bath; ob++) {
                const cd h = g->bath_h[idx_bh(c, a, b, is, js, oa, ob)];
                if (h.imag() != 0.0 || h != g->bath_h[idx_bh(c, b, a, js, is, ob, oa)]) return false;
              }
    for (size_t i = 0; i < g->bath_v.size(); i++)
      if (g->bath_v[i].imag() != 0.0) return false;
  }
  return true;
}

// P(z) = Hloc + Delta(z) in lso at n device points (VCA_OMEGA.f90:62-66)
int hloc_delta(int n, const double2* d_z, Arena& ar, double2** P_out) {
  const vca_config& c = g->cfg;
  const int N = g->N, NN = N * N;
  int rc = VCA_OK;
  double2 *P, *D = nullptr, *Hl, *hraw;
  if ((rc = ar.alloc(&P, (size_t)n * NN)) || (rc = ar.alloc(&Hl, NN)) || (rc = ar.alloc(&hraw, NN))) return rc;
  cudaMemcpyAsync(hraw, g->Hloc.data(), sizeof(double2) * NN, cudaMemcpyHostToDevice, g->st);
  launch_nnn2lso(c.Nlat, c.Nspin, c.Norb, 1, hraw, Hl, g->st);
  if (g->has_bath) {  // Delta(z)
    std::vector<double2> hb, V;
    bath_lso(hb, V);
    double2 *dhb, *dV, *work;
    const int Nb = g->Nb;
    if ((rc = ar.alloc(&dhb, (size_t)Nb * Nb)) || (rc = ar.alloc(&dV, (size_t)N * Nb)) ||
        (rc = ar.alloc(&work, (size_t)n * 2 * Nb * Nb)) || (rc = ar.alloc(&D, (size_t)n * NN)))
      return rc;
    cudaMemcpyAsync(dhb, hb.data(), sizeof(double2) * hb.size(), cudaMemcpyHostToDevice, g->st);
    cudaMemcpyAsync(dV, V.data(), sizeof(double2) * V.size(), cudaMemcpyHostToDevice, g->st);
    launch_delta_bath(n, d_z, N, Nb, dhb, dV, c.xmu, work, D, g->st);
  }
  launch_add_hloc(n, NN, D, Hl, P, g->st);
  *P_out = P;
  return VCA_OK;
}

// Omega integrand at n device points d_z (sum_kmesh / sum_kmesh_complex,
// VCA_OMEGA.f90:37-114): on return *f_re[i] = (1/Nk) sum_k ln|det(1 + (Delta
// + Hloc - Hk) G'(z_i))| and, when want_im, *f_im[i] = (1/Nk) sum_k arg det
// (principal), both device arrays owned by ar.
int ksum_device(int n, const double2* d_z, bool want_im, Arena& ar, double** f_re, double** f_im) {
  const vca_config& c = g->cfg;
  const int64_t Nk = g->Nk;
  const int N = g->N, NN = N * N;
  int rc = VCA_OK;
  double2 *Glso, *P;
  if ((rc = ar.alloc(&Glso, (size_t)n * NN))) return rc;
  RCHK(gf_lso(n, d_z, Glso, ar));
  RCHK(hloc_delta(n, d_z, ar, &P));
  const bool blk = g->hk_spin_diag && point_spin_diagonal();
  const int nblk = blk ? c.Nspin : 1;
  const int nb = N / nblk;
  if (nb > 32) VFAIL(VCA_ERR_UNSUPPORTED, "Omega k-sum supports spin blocks up to 32 orbitals");
  const int kchunks = (int)std::max<int64_t>(1, std::min<int64_t>(Nk, (152 * 8 + n - 1) / n));
  double *fpart, *fpart_im = nullptr;
  if ((rc = ar.alloc(&fpart, (size_t)n * kchunks)) || (rc = ar.alloc(f_re, n))) return rc;
  if (want_im && ((rc = ar.alloc(&fpart_im, (size_t)n * kchunks)) || (rc = ar.alloc(f_im, n)))) return rc;
  // union sparsity pattern of M = Delta + Hloc - Hk within each spin block
  std::vector<int> rowptr(N + 1, 0), cols;
  for (int a = 0; a < N; a++) {
    const int b0 = (a / nb) * nb;
    for (int b = b0; b < b0 + nb; b++) {
      const int il = (a / c.Norb) % c.Nlat, io = a % c.Norb, is = a / (c.Norb * c.Nlat);
      const int jl = (b / c.Norb) % c.Nlat, jo = b % c.Norb, js = b / (c.Norb * c.Nlat);
      const cd hl = g->Hloc[idx_nnn(c, il, jl, is, js, io, jo)];
      const size_t ab = a + (size_t)b * N;
      if (g->has_bath || g->hk_varying[ab] || hl != g->hk_const[ab]) cols.push_back(b);
    }
    rowptr[a + 1] = (int)cols.size();
  }
  int *d_rowptr, *d_cols;
  if ((rc = ar.alloc(&d_rowptr, N + 1)) || (rc = ar.alloc(&d_cols, std::max<size_t>(1, cols.size())))) return rc;
  cudaMemcpyAsync(d_rowptr, rowptr.data(), sizeof(int) * (N + 1), cudaMemcpyHostToDevice, g->st);
  if (!cols.empty()) cudaMemcpyAsync(d_cols, cols.data(), sizeof(int) * cols.size(), cudaMemcpyHostToDevice, g->st);
  const bool pairs = g->d_Hk_rep && g->Nk_rep < Nk && omega_pairs_valid();
  const int64_t nks = pairs ? g->Nk_rep : Nk;
  const double2* hks = pairs ? g->d_Hk_rep : g->d_Hk;
  // without a bath P = Hloc at every node: M_k = Hloc - H_k once per k
  const bool pre_m = !g->has_bath;
  if (pre_m) {
    double2* M;
    if ((rc = ar.alloc(&M, (size_t)nks * NN))) return rc;
    launch_m_from_hk(nks, NN, P, hks, M, g->st);
    hks = M;
  }
  KsumInverse ki;
  if (!want_im && g->omega_inverse_form) {  // T=0 integrand: the inverse form below omega_c
    double2* Ginv;
    double* ldG;
    if ((rc = ar.alloc(&Ginv, (size_t)n * NN)) || (rc = ar.alloc(&ldG, (size_t)n * nblk))) return rc;
    launch_ginv_blocks(n, N, nblk, nb, Glso, Ginv, ldG, g->st);
    ki.z = d_z;
    ki.Ginv = Ginv;
    ki.ldG = ldG;
    ki.omega_c = 10.0;
  }
  launch_omega_ksum2(n, N, nblk, nb, P, Glso, nks, hks, pairs ? g->d_kw : nullptr, d_rowptr, d_cols, fpart,
                     fpart_im, kchunks, pre_m, ki, g->st);
  launch_reduce_rows(n, kchunks, fpart, 1.0 / (double)Nk, *f_re, g->st);
  if (want_im) launch_reduce_rows(n, kchunks, fpart_im, 1.0 / (double)Nk, *f_im, g->st);
  CUCHK(cudaGetLastError());
  return VCA_OK;
}

// The integrand at n host points (f_im may be NULL: real part only)
int ksum_host(int n, const double2* zh, double* f_re, double* f_im) {
  Arena ar;
  double2* d_z;
  double *dre = nullptr, *dim = nullptr;
  int rc = ar.alloc(&d_z, n);
  if (!rc) rc = (cudaMemcpyAsync(d_z, zh, sizeof(double2) * n, cudaMemcpyHostToDevice, g->st) == cudaSuccess)
                    ? VCA_OK : VCA_ERR_CUDA;
  if (!rc) rc = ksum_device(n, d_z, f_im != nullptr, ar, &dre, &dim);
  if (!rc) {
    cudaMemcpyAsync(f_re, dre, sizeof(double) * n, cudaMemcpyDeviceToHost, g->st);
    if (f_im) cudaMemcpyAsync(f_im, dim, sizeof(double) * n, cudaMemcpyDeviceToHost, g->st);
    if (cudaStreamSynchronize(g->st) != cudaSuccess) rc = VCA_ERR_CUDA;
  }
  ar.release();
  if (rc == VCA_ERR_CUDA) VFAIL(VCA_ERR_CUDA, cudaGetErrorString(cudaGetLastError()));
  return rc;
}

// frequency_integration (VCA_OMEGA.f90:123-136) with the fixed rule w =
// scale*s/(1-s) (Gauss-Legendre in s, nodes cached per context) replacing
// the adaptive quad(imaginary_axis, 0, inf)
// Nodes i*w_j and weights of the fixed rule on [0, inf), computed once per
// context (they depend on omega_nodes and omega_scale only)
int ensure_omega_nodes() {
  const vca_config& c = g->cfg;
  const int n = c.omega_nodes;
  if (g->node_n == n && g->node_scale == c.omega_scale && g->node_z) return VCA_OK;
  Arena ar;
  int rc = VCA_OK;
  g->nodes.release();
  g->node_n = 0;
  double *s, *w, *inv;
  if ((rc = ar.alloc(&s, n)) || (rc = ar.alloc(&w, n)) || (rc = ar.alloc(&inv, n + 1)) ||
      (rc = g->nodes.alloc(&g->node_z, n)) || (rc = g->nodes.alloc(&g->node_w, n))) {
    ar.release();
    return rc;
  }
  launch_gauss_legendre(n, inv, s, w, g->st);
  launch_omega_nodes(n, c.omega_scale, s, w, g->node_z, g->node_w, g->st);
  const cudaError_t e = cudaStreamSynchronize(g->st);
  ar.release();
  CUCHK(e);
  g->node_n = n;
  g->node_scale = c.omega_scale;
  return VCA_OK;
}

int omega_integral(double* out) {
  const vca_config& c = g->cfg;
  RCHK(ensure_omega_nodes());
  Arena ar;
  int rc = VCA_OK;
  const int n = c.omega_nodes;
  double *f = nullptr, *acc = nullptr;
  if ((rc = ksum_device(n, g->node_z, false, ar, &f, nullptr)) || (rc = ar.alloc(&acc, 1))) {
    ar.release();
    return rc;
  }
  launch_wsum(n, g->node_w, f, acc, g->st);
  double integral = 0.0;
  CUCHK(cudaMemcpyAsync(&integral, acc, sizeof(double), cudaMemcpyDeviceToHost, g->st));
  CUCHK(cudaStreamSynchronize(g->st));
  ar.release();
  *out = (3.0 - c.Nspin) * integral / M_PI;
  return VCA_OK;
}

// Largest excitation de = diag(j) - Ei over the poles of every chain
// (max_exc, VCA_GF_NORMAL.f90:57,1018).  The reference diagonalises the
// whole nlanc x nlanc tridiagonal: a chain that stopped after n < nlanc steps
// keeps the zeros its coefficient arrays were cleared to (VCA_GF_NORMAL.f90:
// 211-213), which add eigenvalues 0, i.e. de = -Ei.  Chains whose start
// vector vanished (n = 0; NaN in the reference, which the comparison skips)
// add nothing.
int chains_max_exc(double* out) {
  RCHK(ensure_poles());
  const size_t nch = g->chains.size();
  double m = -DBL_MAX;
  if (nch) {
    std::vector<double> p(nch * (size_t)g->ld);
    std::vector<int> n(nch), sg(nch);
    CUCHK(cudaMemcpy(p.data(), g->d_poles, sizeof(double) * p.size(), cudaMemcpyDeviceToHost));
    CUCHK(cudaMemcpy(n.data(), g->d_nexc, sizeof(int) * nch, cudaMemcpyDeviceToHost));
    CUCHK(cudaMemcpy(sg.data(), g->cstore.isign, sizeof(int) * nch, cudaMemcpyDeviceToHost));
    for (size_t ch = 0; ch < nch; ch++) {
      for (int j = 0; j < n[ch]; j++) m = std::max(m, sg[ch] * p[ch * g->ld + j]);  // poles = isign*de
      if (n[ch] > 0 && n[ch] < g->chains[ch].nlanc) m = std::max(m, -g->gs[g->chains[ch].state].e);
    }
  }
  *out = m;
  return VCA_OK;
}

// frequency_integration_finite_t (VCA_OMEGA.f90:153-182): Matsubara sum up
// to nmax plus the contour integral over |w| = R, times (3 - Nspin)
int omega_integral_finite_t(double* out) {
  const vca_config& c = g->cfg;
  const double beta = c.beta, mu = c.xmu;
  RCHK(chains_max_exc(&g->max_exc));
  if (!std::isfinite(g->max_exc)) VFAIL(VCA_ERR_NUMERIC, "no Green's function pole: max_exc undefined");
  const double xn = 2.0 * (std::fabs(g->max_exc) + c.bandwidth) * beta / M_PI;
  if (!(xn < 1e8)) VFAIL(VCA_ERR_UNSUPPORTED, "finite-T Matsubara sum beyond 5e7 frequencies");
  int nmax = (int)xn;
  nmax = (nmax % 2 == 0) ? nmax / 2 : (nmax + 1) / 2;
  const double R = 2.0 * (nmax + 1) * M_PI / beta;
  // 2) Matsubara sum 2/beta sum_{n=0..nmax} Re F(i w_n)
  std::vector<double2> zm(nmax + 1);
  for (int n = 0; n <= nmax; n++) zm[n] = make_double2(0.0, (2.0 * n + 1.0) * M_PI / beta);
  std::vector<double> fm(nmax + 1);
  RCHK(ksum_host(nmax + 1, zm.data(), fm.data(), nullptr));
  double sum = 0.0;
  for (int n = 0; n <= nmax; n++) sum += fm[n];
  sum = 2.0 * (1.0 / beta) * sum;
  // 3) contour part: integral_contour (:186-199) on the fixed rule
  std::vector<double> th, wt;
  contour_nodes_host(R, beta, mu, c.contour_nodes, th, wt);
  const int nc = (int)th.size();
  std::vector<double2> zc(nc);
  for (int i = 0; i < nc; i++) zc[i] = make_double2(R * std::cos(th[i]), R * std::sin(th[i]));
  std::vector<double> fre(nc), fim(nc);
  RCHK(ksum_host(nc, zc.data(), fre.data(), fim.data()));
  double integral = 0.0;
  for (int i = 0; i < nc; i++) {
    const cd w(zc[i].x, zc[i].y);
    cd fermi = 0.0;
    if (((w - mu) * beta).real() < 100.0) fermi = 1.0 / (std::exp(beta * (w - mu)) + 1.0);
    integral += wt[i] * ((1.0 / M_PI) * w * fermi * cd(fre[i], fim[i])).real();
  }
  g->nmax = nmax;
  g->int_R = R;
  g->sum_part = sum;
  g->contour_part = integral;
  g->contour_points = nc;
  *out = (3.0 - c.Nspin) * (sum + integral);
  return VCA_OK;
}

// Custom-observable integrand at n device points (sum_observable_kmesh and
// _complex, VCA_OBSERVABLES.f90:408-500): *f[i] = (1/Lk) sum_k Re{Tr[s_k
// G_k(z_i)] - tail*Tr[s_k]/(z_i - 1.1)}, G_k = (G'^-1 - (H_k - Hloc -
// Delta))^-1; d_s holds s_k in lso, sk_stride = N*N per k or 0.
int obs_device(int n, const double2* d_z, bool tail, const double2* d_s, int64_t sk_stride, Arena& ar,
               double** f) {
  const vca_config& c = g->cfg;
  const int N = g->N, NN = N * N;
  const int64_t Nk = g->Nk;
  int rc = VCA_OK;
  double2 *Glso, *Ginv, *P;
  if ((rc = ar.alloc(&Glso, (size_t)n * NN)) || (rc = ar.alloc(&Ginv, (size_t)n * NN))) return rc;
  RCHK(gf_lso(n, d_z, Glso, ar));
  launch_inverse_batch(n, N, Glso, Ginv, g->st);
  RCHK(hloc_delta(n, d_z, ar, &P));
  const bool blk = g->hk_spin_diag && point_spin_diagonal();
  const int nblk = blk ? c.Nspin : 1;
  const int nb = N / nblk;
  if (nb > 32) VFAIL(VCA_ERR_UNSUPPORTED, "custom observables support spin blocks up to 32 orbitals");
  const int kchunks = (int)std::max<int64_t>(1, std::min<int64_t>(Nk, (152 * 8 + n - 1) / n));
  double* fpart;
  if ((rc = ar.alloc(&fpart, (size_t)n * kchunks)) || (rc = ar.alloc(f, n))) return rc;
  launch_obs_ksum(n, N, nblk, nb, d_z, Ginv, P, Nk, g->d_Hk, d_s, sk_stride, tail, fpart, kchunks, g->st);
  launch_reduce_rows(n, kchunks, fpart, 1.0 / (double)Nk, *f, g->st);
  CUCHK(cudaGetLastError());
  return VCA_OK;
}

// The same at n host points, result on the host
int obs_host(int n, const double2* zh, bool tail, const double2* d_s, int64_t sk_stride, double* f_host) {
  Arena ar;
  double2* d_z;
  double* f = nullptr;
  int rc = ar.alloc(&d_z, n);
  if (!rc) rc = cudaMemcpyAsync(d_z, zh, sizeof(double2) * n, cudaMemcpyHostToDevice, g->st) == cudaSuccess
                    ? VCA_OK : VCA_ERR_CUDA;
  if (!rc) rc = obs_device(n, d_z, tail, d_s, sk_stride, ar, &f);
  if (!rc) {
    cudaMemcpyAsync(f_host, f, sizeof(double) * n, cudaMemcpyDeviceToHost, g->st);
    if (cudaStreamSynchronize(g->st) != cudaSuccess) rc = VCA_ERR_CUDA;
  }
  ar.release();
  if (rc == VCA_ERR_CUDA) VFAIL(VCA_ERR_CUDA, cudaGetErrorString(cudaGetLastError()));
  return rc;
}

// One custom observable of the last solve (get_custom_observables with one
// item, VCA_OBSERVABLES.f90:140-170).  T=0 (:337-347): (3-Nspin)/pi times
// the integral over [0, inf) of the tail-subtracted integrand, on the fixed
// rule of the Omega integral.  Finite T (:351-388): 2/beta sum_{n<=nmax} of
// the integrand at i w_n plus the integral of Re[(1/pi) w fermi(w - xmu)
// F(w)] over the whole circle |w| = R (quad from -pi to pi), F taken real as
// the reference's DREAL does, times (3-Nspin); nmax and R as for Omega.
int custom_observable(const double* s_host, bool kdep, double* value) {
  const vca_config& c = g->cfg;
  const int N = g->N, NN = N * N;
  const int64_t L = kdep ? g->Nk : 1;
  Arena ar;
  double2 *sraw, *slso;
  int rc = VCA_OK;
  if ((rc = ar.alloc(&sraw, (size_t)L * NN)) || (rc = ar.alloc(&slso, (size_t)L * NN))) { ar.release(); return rc; }
  CUCHK(cudaMemcpyAsync(sraw, s_host, sizeof(double2) * (size_t)L * NN, cudaMemcpyHostToDevice, g->st));
  launch_nnn2lso(c.Nlat, c.Nspin, c.Norb, L, sraw, slso, g->st);
  const int64_t stride = kdep ? NN : 0;
  if (!g->finiteT) {
    if ((rc = ensure_omega_nodes())) { ar.release(); return rc; }
    const int n = c.omega_nodes;
    double *f = nullptr, *acc = nullptr;
    if ((rc = obs_device(n, g->node_z, true, slso, stride, ar, &f)) || (rc = ar.alloc(&acc, 1))) {
      ar.release();
      return rc;
    }
    launch_wsum(n, g->node_w, f, acc, g->st);
    double integral = 0.0;
    cudaMemcpyAsync(&integral, acc, sizeof(double), cudaMemcpyDeviceToHost, g->st);
    const cudaError_t e = cudaStreamSynchronize(g->st);
    ar.release();
    CUCHK(e);
    *value = (3.0 - c.Nspin) * integral / M_PI;
    return VCA_OK;
  }
  const double beta = c.beta, mu = c.xmu, R = g->int_R;
  const int nmax = g->nmax;
  std::vector<double2> zm(nmax + 1);
  for (int n = 0; n <= nmax; n++) zm[n] = make_double2(0.0, (2.0 * n + 1.0) * M_PI / beta);
  std::vector<double> fm(nmax + 1);
  if ((rc = obs_host(nmax + 1, zm.data(), false, slso, stride, fm.data()))) { ar.release(); return rc; }
  double out = 0.0;
  for (int n = 0; n <= nmax; n++) out += fm[n];
  out = 2.0 * (1.0 / beta) * out;
  std::vector<double> th, wt;
  contour_nodes_host(R, beta, mu, c.contour_nodes, th, wt);
  const int nh = (int)th.size();
  std::vector<double2> zc(2 * nh);  // the upper half, then its mirror image
  for (int i = 0; i < nh; i++) {
    zc[i] = make_double2(R * std::cos(th[i]), R * std::sin(th[i]));
    zc[nh + i] = make_double2(zc[i].x, -zc[i].y);
  }
  std::vector<double> fc(2 * nh);
  rc = obs_host(2 * nh, zc.data(), false, slso, stride, fc.data());
  ar.release();
  if (rc) return rc;
  double integral = 0.0;
  for (int i = 0; i < 2 * nh; i++) {
    const cd w(zc[i].x, zc[i].y);
    cd fermi = 0.0;
    if (((w - mu) * beta).real() < 100.0) fermi = 1.0 / (std::exp(beta * (w - mu)) + 1.0);
    integral += wt[i % nh] * ((1.0 / M_PI) * w * fermi * fc[i]).real();
  }
  *value = (3.0 - c.Nspin) * (out + integral);
  return VCA_OK;
}

// Omega' (VCA_MAIN.f90:186-193): E_gs at T=0, E_min - T ln sum_i
// exp(-beta(E_i - E_min)) over the final state list at finite T
double omega_prime() {
  if (!g->finiteT) return g->egs;
  double z = 0.0;
  for (const GState& s : g->gs) z += std::exp(-g->cfg.beta * (s.e - g->egs));
  return g->egs - (1.0 / g->cfg.beta) * std::log(z);
}

// Pairs k, k' with H_k' = conj(H_k) to 1e-13 of the largest |H_k| entry
// (time reversal: k' = -k on a symmetric grid).  For a real model whose
// Omega matrices P = Delta + Hloc and G' are symmetric, M_k' = P - H_k^T =
// M_k^T and det(1 + M_k^T G) = det(1 + G M_k) = det(1 + M_k G), so the
// integrand is equal at the two points: the k-sum then runs over one point
// per pair with weight 2.  Candidates are found through a random linear
// signature of the matrix (sorted), then checked entry by entry; a point
// without a partner keeps weight 1.
int pair_kpoints(const double* Hk, int64_t Nk, size_t nel) {
  std::vector<int64_t> reps;
  std::vector<double> wts;
  pair_kpoints_host(Hk, Nk, nel, reps, wts);
  g->Nk_rep = (int64_t)reps.size();
  int64_t* d_rep;
  Arena tmp;
  RCHK(g->omega.alloc(&g->d_Hk_rep, nel * g->Nk_rep));
  RCHK(g->omega.alloc(&g->d_kw, g->Nk_rep));
  RCHK(tmp.alloc(&d_rep, g->Nk_rep));
  CUCHK(cudaMemcpyAsync(d_rep, reps.data(), sizeof(int64_t) * g->Nk_rep, cudaMemcpyHostToDevice, g->st));
  CUCHK(cudaMemcpyAsync(g->d_kw, wts.data(), sizeof(double) * g->Nk_rep, cudaMemcpyHostToDevice, g->st));
  launch_gather_blocks(g->Nk_rep, (int64_t)nel, d_rep, g->d_Hk, g->d_Hk_rep, g->st);
  cudaError_t e = cudaStreamSynchronize(g->st);
  tmp.release();
  CUCHK(e);
  return VCA_OK;
}

int upload_hk(const double* Hk, int64_t Nk) {
  const vca_config& c = g->cfg;
  if (!Hk || Nk <= 0) VFAIL(VCA_ERR_SHAPE, "Hk must hold at least one k-point");
  const size_t nel = hloc_len(c);
  RCHK(check_finite(Hk, 2 * nel * Nk, "Hk"));
  g->omega.release();
  double2* raw;
  RCHK(g->omega.alloc(&raw, nel * Nk));
  RCHK(g->omega.alloc(&g->d_Hk, nel * Nk));
  CUCHK(cudaMemcpyAsync(raw, Hk, sizeof(double2) * nel * Nk, cudaMemcpyHostToDevice, g->st));
  launch_nnn2lso(c.Nlat, c.Nspin, c.Norb, Nk, raw, g->d_Hk, g->st);
  CUCHK(cudaGetLastError());
  g->Nk = Nk;
  g->hk_spin_diag = hk_spin_diagonal(Hk, Nk);
  // k-independent entries of Hk (lso): where Hloc equals them the Omega
  // matrix M = Delta + Hloc - Hk has an exact zero
  {
    const int N = g->N;
    g->hk_const.assign((size_t)N * N, 0.0);
    g->hk_varying.assign((size_t)N * N, 0);
    for (int il = 0; il < c.Nlat; il++)
      for (int jl = 0; jl < c.Nlat; jl++)
        for (int is = 0; is < c.Nspin; is++)
          for (int js = 0; js < c.Nspin; js++)
            for (int io = 0; io < c.Norb; io++)
              for (int jo = 0; jo < c.Norb; jo++) {
                const int a = io + il * c.Norb + is * c.Norb * c.Nlat, b = jo + jl * c.Norb + js * c.Norb * c.Nlat;
                const int64_t x = idx_nnn(c, il, jl, is, js, io, jo);
                const double re = Hk[2 * x], im = Hk[2 * x + 1];
                bool var = false;
                for (int64_t k = 1; k < Nk && !var; k++)
                  if (Hk[2 * (k * nel + x)] != re || Hk[2 * (k * nel + x) + 1] != im) var = true;
                g->hk_const[a + (size_t)b * N] = cd(re, im);
                g->hk_varying[a + (size_t)b * N] = var ? 1 : 0;
              }
  }
  RCHK(pair_kpoints(Hk, Nk, nel));
  CUCHK(cudaStreamSynchronize(g->st));
  return VCA_OK;
}

double now_ms() {
  timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec * 1e3 + ts.tv_nsec * 1e-6;
}

// Hk must already be resident (upload_hk)
int solve_resident(const double* Hloc, const double* bath_h, const double* bath_v, double* omega_out) {
  if (!g || !g->basis.ptrs.size()) VFAIL(VCA_ERR_STATE, "vca_gpu_init has not been called");
  if (!g->d_Hk) VFAIL(VCA_ERR_STATE, "no Hk resident: call vca_gpu_solve or vca_gpu_upload_hk first");
  g->solved = false;
  gfm_drop();  // vca_solve rebuilds impGmatrix
  g->sigma_loaded = false;  // and impSmats / impSreal
  g->sigma_mats.clear();
  g->sigma_real.clear();
  double t0 = now_ms();
  RCHK(set_hamiltonian(Hloc, bath_h, bath_v));
  double t1 = now_ms();
  RCHK(diagonalize());
  double t2 = now_ms();
  RCHK(build_gf());
  if (g->fx && fx_take_wait_failures() != 0)
    VFAIL(VCA_ERR_TIMEOUT, "a bounded wait for a bulk copy in the column H x v ran out");
  double t3 = now_ms();
  RCHK(g->finiteT ? omega_integral_finite_t(&g->omega_int) : omega_integral(&g->omega_int));
  double t4 = now_ms();
  g->t_ms[0] = t1 - t0;
  g->t_ms[1] = t2 - t1;
  g->t_ms[2] = t3 - t2;
  g->t_ms[3] = t4 - t3;
  g->omega_prime = omega_prime();
  g->sft = g->omega_prime - g->omega_int;  // VCA_MAIN.f90:183-197
  g->solved = true;
  if (omega_out) *omega_out = g->sft;
  return VCA_OK;
}

int solve_one(const double* Hloc, const double* Hk, int64_t Nk, const double* bath_h,
              const double* bath_v, double* omega_out) {
  if (!g || !g->basis.ptrs.size()) VFAIL(VCA_ERR_STATE, "vca_gpu_init has not been called");
  RCHK(upload_hk(Hk, Nk));
  return solve_resident(Hloc, bath_h, bath_v, omega_out);
}

// One chain's table as the reference stores it, from the chain's n poles p
// and weights w (p = isign*(d_j - Ei), d ascending): a chain that stopped
// after n < nlanc steps also lists the eigenvalues 0 of its zero-padded
// coefficients (pole isign*(0 - Ei), weight 0) in ascending position
// (VCA_GF_NORMAL.f90:1006-1022).  Poles out as complex numbers.
void chain_table(const ChainRec& r, int n, int sg, const double* p, const double2* w, std::vector<double2>& P,
                 std::vector<double2>& W) {
  P.clear();
  W.clear();
  if (n <= 0) return;
  const int npad = n < r.nlanc ? r.nlanc - n : 0;
  const double Ei = g->gs[r.state].e;
  int q = 0;
  auto put = [&](double pole, double2 wt) {
    P.push_back(make_double2(pole, 0.0));
    W.push_back(wt);
  };
  for (int j = 0; j < n; j++) {
    const double dj = sg * p[j] + Ei;
    if (q == 0 && npad && dj > 0.0)
      for (; q < npad; q++) put(sg * (0.0 - Ei), make_double2(0.0, 0.0));
    put(p[j], w[j]);
  }
  for (; q < npad; q++) put(sg * (0.0 - Ei), make_double2(0.0, 0.0));
}

// file element of (il, jl, is, io, jo), 0-based: the loops of save_gfprime
// and read_gfprime, ilat outermost, jorb innermost (VCA_AUX_FUNX.f90:627-641)
inline int64_t gfm_elem(const vca_config& c, int il, int jl, int is, int io, int jo) {
  return jo + (int64_t)c.Norb * (io + (int64_t)c.Norb * (is + (int64_t)c.Nspin * (jl + (int64_t)c.Nlat * il)));
}

// The tables of the last solve in file order (impGmatrix as build_gf_normal
// fills it, VCA_GF_NORMAL.f90:57-80): every spin-diagonal element holds
// every kept state; 2 channels on the diagonal, 4 (chan4) or 2 (chan2) off
// it; a channel without target sector has no excitations.
static int solve_tables(GfmTable& t) {
  const vca_config& c = g->cfg;
  RCHK(ensure_poles());
  const int nch = (int)g->chains.size();
  const int nst = (int)g->gs.size();
  std::vector<int> nx(nch), sg(nch);
  std::vector<double> P((size_t)nch * g->ld);
  std::vector<double2> W((size_t)nch * g->ld);
  if (nch) {
    CUCHK(cudaMemcpy(nx.data(), g->d_nexc, sizeof(int) * nch, cudaMemcpyDeviceToHost));
    CUCHK(cudaMemcpy(sg.data(), g->cstore.isign, sizeof(int) * nch, cudaMemcpyDeviceToHost));
    CUCHK(cudaMemcpy(P.data(), g->d_poles, sizeof(double) * P.size(), cudaMemcpyDeviceToHost));
    CUCHK(cudaMemcpy(W.data(), g->d_weights, sizeof(double2) * W.size(), cudaMemcpyDeviceToHost));
  }
  const int nelem = c.Nlat * c.Nlat * c.Nspin * c.Norb * c.Norb;
  std::vector<int> which((size_t)nelem * nst * 4, -1);  // (elem, state, chan) -> chain
  for (int ch = 0; ch < nch; ch++) {
    const ChainRec& r = g->chains[ch];
    if (r.chan >= 1 && r.chan <= 4 && r.state >= 0 && r.state < nst && r.elem >= 0 && r.elem < nelem)
      which[((size_t)r.elem * nst + r.state) * 4 + r.chan - 1] = ch;
  }
  t = GfmTable{};
  std::vector<double2> tp, tw;
  for (int il = 0; il < c.Nlat; il++)
    for (int jl = 0; jl < c.Nlat; jl++)
      for (int is = 0; is < c.Nspin; is++)
        for (int io = 0; io < c.Norb; io++)
          for (int jo = 0; jo < c.Norb; jo++) {
            const int e = elem_index(c, il, jl, is, io, jo);
            const int nchan = (il == jl && io == jo) ? 2 : (c.vca_gf_symmetric ? 2 : 4);
            t.nstates.push_back(nst);
            for (int k = 0; k < nst; k++) {
              t.nchan.push_back(nchan);
              for (int ich = 1; ich <= nchan; ich++) {
                const int ch = which[((size_t)e * nst + k) * 4 + ich - 1];
                if (ch < 0) {
                  t.nexc.push_back(0);
                  continue;
                }
                chain_table(g->chains[ch], nx[ch], sg[ch], P.data() + (size_t)ch * g->ld,
                            W.data() + (size_t)ch * g->ld, tp, tw);
                t.nexc.push_back((int32_t)tp.size());
                for (size_t j = 0; j < tp.size(); j++) {
                  t.poles.push_back(tp[j].x);
                  t.poles.push_back(tp[j].y);
                  t.weights.push_back(tw[j].x);
                  t.weights.push_back(tw[j].y);
                }
              }
            }
          }
  return VCA_OK;
}

static std::string gfm_path(const char* file, const char* suffix, int32_t used) {
  const vca_config& c = g->cfg;
  const std::string sfx = suffix ? std::string(suffix) : std::string(c.file_suffix, strnlen(c.file_suffix, sizeof c.file_suffix));
  return std::string(file) + sfx + (used ? ".used" : ".restart");  // VCA_AUX_FUNX.f90:615-617
}

static void gfm_drop() {
  if (!g) return;
  g->gfm_dev.release();
  g->d_gfm_ptr = nullptr;
  g->d_gfm_p = g->d_gfm_w = nullptr;
  g->gfm = GfmTable{};
  g->gfm_state0.clear();
  g->gfm_chan0.clear();
  g->gfm_exc0.clear();
  g->gfm_loaded = false;
}

// ===========================================================================
// The batched form: B variational points in one pass.  The reference's
// drivers call vca_solve once per point (drivers/vca_hm_chain1d.f90:88-95,
// drivers/vca_bhz_2d.f90:244-305); here the points of a wave share every
// launch.  The FP64 multi-task Lanczos of vca_multi.cu runs one task list per
// stage, each task a (point, sector) or (point, chain) with that point's hop
// tables:
//   1. every point's one-body tables (set_hamiltonian, kept per point);
//   2. every (point, sector) lowest energy in one search (as the plain
//      path's batched search: same start vectors, recurrence and stopping);
//   3. per point the T=0 list (VCA_DIAG.f90:224-236) on the host;
//   4. the kept (point, sector) eigenvectors in one second pass;
//   5. every point's Green's-function chains in memory-bounded groups of
//      (point, chain) tasks (VCA_GF_NORMAL.f90:121-318,561-958);
//   6. per point Omega from its chain store (VCA_OMEGA.f90:37-146).
// T=0 only; the points share Hk.  The context is left as a solve of the last
// point leaves it (that point is solved once more on the plain path, which
// must agree with its batched Omega to 1e-10).
// ===========================================================================
// Eigenvalues of a complex Hermitian n x n matrix (column-major), ascending:
// cyclic Jacobi on the real symmetric 2n x 2n embedding [[Re, -Im], [Im, Re]],
// whose spectrum is each eigenvalue twice.
void herm_eigvals(int n, const std::vector<cd>& h, std::vector<double>& w) {
  const int m = 2 * n;
  std::vector<double> a((size_t)m * m);
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) {
      const cd z = h[i + (size_t)j * n];
      a[i + (size_t)j * m] = z.real();
      a[(i + n) + (size_t)(j + n) * m] = z.real();
      a[(i + n) + (size_t)j * m] = z.imag();
      a[i + (size_t)(j + n) * m] = -z.imag();
    }
  for (int sweep = 0; sweep < 100; sweep++) {
    double off = 0.0, tot = 0.0;
    for (int i = 0; i < m; i++)
      for (int j = 0; j < m; j++) {
        tot += a[i + (size_t)j * m] * a[i + (size_t)j * m];
        if (i != j) off += a[i + (size_t)j * m] * a[i + (size_t)j * m];
      }
    if (off <= 1e-30 * tot || off == 0.0) break;
    for (int p = 0; p < m; p++)
      for (int q = p + 1; q < m; q++) {
        const double apq = a[p + (size_t)q * m];
        if (apq == 0.0) continue;
        const double app = a[p + (size_t)p * m], aqq = a[q + (size_t)q * m];
        const double th = 0.5 * (aqq - app) / apq;
        const double t = (th >= 0 ? 1.0 : -1.0) / (std::fabs(th) + std::sqrt(th * th + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), sn = t * c;
        for (int k = 0; k < m; k++) {  // columns p, q
          const double akp = a[k + (size_t)p * m], akq = a[k + (size_t)q * m];
          a[k + (size_t)p * m] = c * akp - sn * akq;
          a[k + (size_t)q * m] = sn * akp + c * akq;
        }
        for (int k = 0; k < m; k++) {  // rows p, q
          const double apk = a[p + (size_t)k * m], aqk = a[q + (size_t)k * m];
          a[p + (size_t)k * m] = c * apk - sn * aqk;
          a[q + (size_t)k * m] = sn * apk + c * aqk;
        }
      }
  }
  std::vector<double> d(m);
  for (int i = 0; i < m; i++) d[i] = a[i + (size_t)i * m];
  std::sort(d.begin(), d.end());
  w.resize(n);
  for (int i = 0; i < n; i++) w[i] = d[2 * i];
}

// Lower bounds on the lowest energy of every sector of the loaded
// Hamiltonian, or an empty vector when none is available.  With every
// interaction coefficient non-negative (U, Ust, Ust - Jh), H = H1 + Hint
// with Hint >= 0, so E_min(n_up, n_dw) >= the ground energy of the one-body
// part H1 in that sector: the sum of the n_up lowest levels of the up
// one-body matrix (hops, level energies with -xmu and the HFMODE shifts) and
// the n_dw lowest of the down one, plus the HFMODE constant.
std::vector<double> sector_lower_bounds() {
  const vca_config& c = g->cfg;
  std::vector<double> out;
  for (int o = 0; o < c.Norb; o++)
    if (c.Uloc[o] < 0.0) return out;
  if (c.Norb > 1 && (c.Ust < 0.0 || c.Ust - c.Jh < 0.0)) return out;
  const int Ns = g->Ns, LC = c.Nlat * c.Norb;
  const int nsets = (c.Nspin == 2) ? 2 : 1;
  std::vector<double> lev[2];
  for (int set = 0; set < nsets; set++) {
    const int sidx = (set == 0) ? 0 : c.Nspin - 1;
    std::vector<cd> h((size_t)Ns * Ns, cd(0.0, 0.0));
    for (int il = 0; il < c.Nlat; il++)
      for (int io = 0; io < c.Norb; io++) {
        double e = g->Hloc[idx_nnn(c, il, il, sidx, sidx, io, io)].real() - c.xmu;
        if (c.hfmode) {
          e += -0.5 * c.Uloc[io];
          if (c.Norb > 1) e += -0.5 * (2.0 * c.Ust - c.Jh) * (c.Norb - 1);
        }
        const int l = io + il * c.Norb;
        h[l + (size_t)l * Ns] = e;
      }
    if (g->has_bath)
      for (int lb = 0; lb < c.Nlat_bath; lb++)
        for (int ob = 0; ob < c.Norb_bath; ob++) {
          const int l = LC + lb * c.Norb_bath + ob;
          h[l + (size_t)l * Ns] = g->bath_h[idx_bh(c, lb, lb, sidx, sidx, ob, ob)].real() - c.xmu;
        }
    // the hopping pairs of this spin set: set 0 owns [0, set0), set 1 the rest
    const size_t q0 = (set == 0) ? 0 : g->host_pairs_set0;
    const size_t q1 = (set == 0) ? g->host_pairs_set0 : g->host_pairs.size();
    for (size_t q = q0; q < q1; q++) {
      const HopPair& hp = g->host_pairs[q];
      h[hp.i + (size_t)hp.j * Ns] += cd(hp.re, hp.im);  // c^dag_i c_j
    }
    herm_eigvals(Ns, h, lev[set]);
  }
  if (nsets == 1) lev[1] = lev[0];
  std::vector<double> cum[2];
  for (int set = 0; set < 2; set++) {
    cum[set].assign(Ns + 1, 0.0);
    for (int k = 0; k < Ns; k++) cum[set][k + 1] = cum[set][k] + lev[set][k];
  }
  out.assign(g->Nsectors, 0.0);
  for (int s = 1; s <= g->Nsectors; s++) out[s - 1] = cum[0][sec_nup(s)] + cum[1][sec_ndw(s)] + g->md.c0;
  return out;
}

struct PointTabs {
  Arena ham;
  std::vector<SpinSpace> sp[2];
  std::vector<cd> Hloc, bath_h, bath_v;
  bool real_model = true;
};

SectorView view_tabs(const PointTabs& P, int nup, int ndw) {
  const SpinSpace& u = P.sp[0][nup];
  const SpinSpace& d = P.sp[g->dwset][ndw];
  SectorView v;
  v.dimup = u.dim;
  v.dimdw = d.dim;
  v.wup = u.width;
  v.wdw = d.width;
  v.up_words = u.words;
  v.dw_words = d.words;
  v.up_cnt = u.cnt;
  v.dw_cnt = d.cnt;
  v.up_src = u.src;
  v.dw_src = d.src;
  v.up_amp = u.amp;
  v.dw_amp = d.amp;
  v.up_e1 = u.e1;
  v.dw_e1 = d.e1;
  return v;
}

struct TaskList {  // tasks packed back to back, cut into MS_TILE tiles
  std::vector<MsSector> secs;
  std::vector<int> tsec;
  std::vector<int64_t> tstart;
  int64_t tot = 0;
  void add(const SectorView& sv, int64_t len, int isector, int ncomp) {
    MsSector m{};
    m.sv = sv;
    m.off = tot;
    m.D = len;
    m.tile0 = (int)tsec.size();
    m.isector = isector;
    m.ncomp = ncomp;
    for (int64_t s = 0; s < len; s += MS_TILE) {
      tsec.push_back((int)secs.size());
      tstart.push_back(s);
    }
    m.ntile = (int)tsec.size() - m.tile0;
    secs.push_back(m);
    tot += len;
  }
};

struct MtRun {  // device state of one multi-task run
  Arena ar;
  MsGroup gp{};
  Ms64Bufs b{};
  double* n2 = nullptr;
};

int mt_alloc(MtRun& R, const TaskList& T, int ld, size_t es, bool psi) {
  const int nsec = (int)T.secs.size(), ntiles = (int)T.tsec.size();
  MsSector* d_secs;
  int* d_tsec;
  int64_t* d_tstart;
  char *x0, *x1, *x2;
  Ms64Bufs& b = R.b;
  b.ld = ld;
  Arena& ar = R.ar;
  int rc = VCA_OK;
  if ((rc = ar.alloc(&d_secs, nsec)) || (rc = ar.alloc(&d_tsec, ntiles)) || (rc = ar.alloc(&d_tstart, ntiles)) ||
      (rc = ar.alloc(&x0, (size_t)T.tot * es)) || (rc = ar.alloc(&x1, (size_t)T.tot * es)) ||
      (rc = ar.alloc(&x2, (size_t)T.tot * es)) || (rc = ar.alloc(&b.tpart, ntiles)) ||
      (rc = ar.alloc(&b.meta, nsec)) || (rc = ar.alloc(&b.alpha, nsec)) || (rc = ar.alloc(&b.bnow, nsec)) ||
      (rc = ar.alloc(&b.invb, nsec)) || (rc = ar.alloc(&b.A, (size_t)nsec * ld)) ||
      (rc = ar.alloc(&b.Bt, (size_t)nsec * ld)) || (rc = ar.alloc(&b.theta, nsec)) ||
      (rc = ar.alloc(&b.resid, nsec)) || (rc = ar.alloc(&b.state, nsec)) || (rc = ar.alloc(&b.mconv, nsec)) ||
      (rc = ar.alloc(&b.undone, 1)) || (rc = ar.alloc(&R.n2, nsec)))
    return rc;
  if (!psi && (rc = ar.alloc(&b.svec, (size_t)nsec * 5 * ld))) return rc;
  b.X = x0;
  b.Xp = x1;
  b.Y = x2;
  CUCHK(cudaMemcpyAsync(d_secs, T.secs.data(), sizeof(MsSector) * nsec, cudaMemcpyHostToDevice, g->st));
  CUCHK(cudaMemcpyAsync(d_tsec, T.tsec.data(), sizeof(int) * ntiles, cudaMemcpyHostToDevice, g->st));
  CUCHK(cudaMemcpyAsync(d_tstart, T.tstart.data(), sizeof(int64_t) * ntiles, cudaMemcpyHostToDevice, g->st));
  CUCHK(cudaMemsetAsync(b.A, 0, sizeof(double) * nsec * ld, g->st));
  CUCHK(cudaMemsetAsync(b.Bt, 0, sizeof(double) * nsec * ld, g->st));
  CUCHK(cudaMemsetAsync(b.bnow, 0, sizeof(double) * nsec, g->st));
  CUCHK(cudaMemsetAsync(b.state, 0, sizeof(int) * nsec, g->st));
  R.gp = MsGroup{d_secs, d_tsec, d_tstart, nsec, ntiles};
  return VCA_OK;
}

// one chain task of the batched form, with the bookkeeping its store needs
struct BChain {
  int point, state;  // point within the wave, its kept state
  MtChain mc;
  ChainRec rec;
  int isign;
  cd wfac;
  int ncomp;
  int tup, tdw;
};

// Host tables of one group of column tasks (chains grouped by point, state,
// spin and particle/hole; rows cut into tiles of R rows)
struct McTaskRef {
  int point, c0, c1;  // chains [c0, c1) of that point's list
  int64_t D;
  int m;
};
struct McHost {
  std::vector<McTask> tasks;
  std::vector<int> tile_task, col_chain, col_part, isg, ch_point, ch_index;
  std::vector<int64_t> tile_row0, tile_row1;
  std::vector<McChain> chains;
  std::vector<ChainMeta> meta;
  std::vector<double2> wf;
  int64_t xoff = 0, part = 0;
  int nl_max = 1;
};
void mc_build(const std::vector<McTaskRef>& refs, size_t t0, size_t t1,
              const std::vector<std::vector<BChain>>& pch, const std::vector<PointTabs>& tabs, int R, int ngfiter,
              McHost& h) {
  for (size_t ti = t0; ti < t1; ti++) {
    const McTaskRef& r = refs[ti];
    const BChain& b0 = pch[r.point][r.c0];
    McTask tk{};
    tk.sv = view_tabs(tabs[r.point], b0.tup, b0.tdw);
    tk.D = r.D;
    tk.m = r.m;
    tk.col0 = (int)h.col_chain.size();
    tk.xoff = h.xoff;
    tk.tile0 = (int)h.tile_task.size();
    for (int64_t rr = 0; rr < r.D; rr += R) {
      h.tile_task.push_back((int)h.tasks.size());
      h.tile_row0.push_back(rr);
      h.tile_row1.push_back(std::min<int64_t>(rr + R, r.D));
    }
    tk.ntile = (int)h.tile_task.size() - tk.tile0;
    tk.part0 = h.part;
    h.part += (int64_t)tk.ntile * tk.m;
    h.xoff += r.D * r.m;
    const int nl = (int)std::min<int64_t>(r.D, ngfiter);
    h.nl_max = std::max(h.nl_max, nl);
    int col = 0;
    for (int ci = r.c0; ci < r.c1; ci++) {
      const BChain& b = pch[r.point][ci];
      McChain mc{};
      mc.task = (int)h.tasks.size();
      mc.col0 = col;
      mc.ncol = b.ncomp;
      mc.op = b.mc;
      for (int qq = 0; qq < b.ncomp; qq++) {
        h.col_chain.push_back((int)h.chains.size());
        h.col_part.push_back(qq);
      }
      col += b.ncomp;
      h.meta.push_back(ChainMeta{b.ncomp, 0, nl, 1, 0});
      h.isg.push_back(b.isign);
      h.wf.push_back(make_double2(b.wfac.real(), b.wfac.imag()));
      h.ch_point.push_back(r.point);
      h.ch_index.push_back(ci);
      h.chains.push_back(mc);
    }
    h.tasks.push_back(tk);
  }
}

// device copy of a group's tables; McGroup points into `ar`
int mc_upload(const McHost& h, int by, Arena& ar, McGroup& gp, ChainMeta** d_meta) {
  McTask* d_tasks;
  int *d_tt, *d_cc, *d_cp;
  int64_t *d_r0, *d_r1;
  McChain* d_ch;
  const int nch = (int)h.chains.size();
  RCHK(ar.alloc(&d_tasks, h.tasks.size()));
  RCHK(ar.alloc(&d_tt, h.tile_task.size()));
  RCHK(ar.alloc(&d_r0, h.tile_row0.size()));
  RCHK(ar.alloc(&d_r1, h.tile_row1.size()));
  RCHK(ar.alloc(&d_cc, h.col_chain.size()));
  RCHK(ar.alloc(&d_cp, h.col_part.size()));
  RCHK(ar.alloc(&d_ch, nch));
  RCHK(ar.alloc(d_meta, nch));
  CUCHK(cudaMemcpyAsync(d_tasks, h.tasks.data(), sizeof(McTask) * h.tasks.size(), cudaMemcpyHostToDevice, g->st));
  CUCHK(cudaMemcpyAsync(d_tt, h.tile_task.data(), sizeof(int) * h.tile_task.size(), cudaMemcpyHostToDevice, g->st));
  CUCHK(cudaMemcpyAsync(d_r0, h.tile_row0.data(), sizeof(int64_t) * h.tile_row0.size(), cudaMemcpyHostToDevice, g->st));
  CUCHK(cudaMemcpyAsync(d_r1, h.tile_row1.data(), sizeof(int64_t) * h.tile_row1.size(), cudaMemcpyHostToDevice, g->st));
  CUCHK(cudaMemcpyAsync(d_cc, h.col_chain.data(), sizeof(int) * h.col_chain.size(), cudaMemcpyHostToDevice, g->st));
  CUCHK(cudaMemcpyAsync(d_cp, h.col_part.data(), sizeof(int) * h.col_part.size(), cudaMemcpyHostToDevice, g->st));
  CUCHK(cudaMemcpyAsync(d_ch, h.chains.data(), sizeof(McChain) * nch, cudaMemcpyHostToDevice, g->st));
  CUCHK(cudaMemcpyAsync(*d_meta, h.meta.data(), sizeof(ChainMeta) * nch, cudaMemcpyHostToDevice, g->st));
  gp = McGroup{d_tasks, d_tt, d_r0, d_r1, d_cc, d_cp, d_ch, (int)h.tasks.size(), (int)h.tile_task.size(),
               (int)h.col_chain.size(), nch, by};
  return VCA_OK;
}

// Autotuner of the chains' tile shape: rows per tile R and row lanes per
// block by.  Each candidate runs one whole chain step (H x v, the two
// reductions, the update and the scaling) three times on the group's first
// tasks (up to 2^24 elements), timed by CUDA events; the fastest shape is
// kept per (real/complex, log2 mean dimension, log2 mean width) for the life
// of the process.  The shape changes the summation order of the chain's dot
// products (at the 1e-16 level), not what is summed.
struct McShape { int R = MC_ROWS, by = 8; double ms = 0.0; bool tuned = false; };
McShape mc_autotune(const std::vector<McTaskRef>& refs, size_t t0, size_t t1,
                    const std::vector<std::vector<BChain>>& pch, const std::vector<PointTabs>& tabs, bool cplx,
                    size_t es) {
  static std::vector<std::pair<long, McShape>> cache;
  McShape best;
  if (!g->autotune) return best;
  double sd = 0.0, sm = 0.0;
  size_t n = 0, t1s = t0;
  int64_t elems = 0;
  while (t1s < t1 && (t1s == t0 || elems + refs[t1s].D * refs[t1s].m <= ((int64_t)1 << 24))) {
    elems += refs[t1s].D * refs[t1s].m;
    sd += (double)refs[t1s].D;
    sm += refs[t1s].m;
    n++;
    t1s++;
  }
  const long key = (cplx ? 1L : 0L) | ((long)std::ilogb(std::max(1.0, sd / n)) << 1) |
                   ((long)std::ilogb(std::max(1.0, sm / n)) << 8);
  for (auto& kv : cache)
    if (kv.first == key) return kv.second;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  best.ms = INFINITY;
  for (int R : {64, 256, 1024}) {
    McHost h;
    mc_build(refs, t0, t1s, pch, tabs, R, g->cfg.lanc_ngfiter, h);
    Arena ar;
    McGroup gp;
    ChainMeta* d_meta;
    double *d_tp, *d_bn, *d_al;
    char *x0, *x1, *x2;
    const int nch = (int)h.chains.size();
    if (mc_upload(h, 8, ar, gp, &d_meta) || ar.alloc(&d_tp, (size_t)h.part) || ar.alloc(&d_bn, nch) ||
        ar.alloc(&d_al, nch) || ar.alloc(&x0, (size_t)h.xoff * es) || ar.alloc(&x1, (size_t)h.xoff * es) ||
        ar.alloc(&x2, (size_t)h.xoff * es)) {
      ar.release();
      continue;
    }
    cudaMemsetAsync(x0, 0, (size_t)h.xoff * es, g->st);
    cudaMemsetAsync(x1, 0, (size_t)h.xoff * es, g->st);
    cudaMemsetAsync(d_bn, 0, sizeof(double) * nch, g->st);
    cudaMemsetAsync(d_al, 0, sizeof(double) * nch, g->st);
    auto step = [&]() {
      mc_launch_hxv(gp, cplx, g->md, d_meta, d_bn, 1, x0, x1, x2, d_tp, g->st);
      mc_launch_reduce(gp, d_tp, d_al, g->st);
      mc_launch_update(gp, cplx, d_meta, d_bn, x0, x2, d_tp, g->st);
      mc_launch_reduce(gp, d_tp, d_al, g->st);
      mc_launch_scale(gp, cplx, d_meta, d_bn, x2, x2, g->st);
    };
    for (int by : {4, 8, 16}) {
      gp.by = by;
      step();  // warm-up
      cudaEventRecord(e0, g->st);
      for (int r = 0; r < 3; r++) step();
      cudaEventRecord(e1, g->st);
      float ms = 0.0f;
      if (cudaEventSynchronize(e1) == cudaSuccess && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess &&
          ms < best.ms) {
        best.R = R;
        best.by = by;
        best.ms = ms;
      }
    }
    ar.release();
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaGetLastError();
  if (!std::isfinite(best.ms)) return McShape{};
  best.tuned = true;
  cache.push_back({key, best});
  return best;
}

int solve_batch_fused(int B, const double* Hloc, int64_t sh, const double* bath_h, int64_t sbh, const double* bath_v,
                      int64_t sbv, double* omega_out) {
  const vca_config cfg0 = g->cfg;
  vca_config& c = g->cfg;
  c.arith = VCA_ARITH_FP64;  // the batched form runs the FP64 path
  auto restore = [&]() { g->cfg = cfg0; };
  auto hl = [&](int p) { return Hloc + 2 * (size_t)p * sh; };
  auto bh = [&](int p) { return bath_h ? bath_h + 2 * (size_t)p * sbh : nullptr; };
  auto bv = [&](int p) { return bath_v ? bath_v + 2 * (size_t)p * sbv : nullptr; };
  const int Ns = g->Ns, nsecs = g->Nsectors;
  int64_t sumD = 0;
  for (int s = 1; s <= nsecs; s++) sumD += (int64_t)g->dimn[sec_nup(s)] * g->dimn[sec_ndw(s)];
  const cd XI(0.0, 1.0);
  const int L = c.Nlat * c.Norb;
  for (double& t : g->bt_ms) t = 0.0;
  double tmark = now_ms();
  auto lap = [&](int stage) {
    cudaStreamSynchronize(g->st);
    const double t = now_ms();
    g->bt_ms[stage] += t - tmark;
    tmark = t;
  };
  int p0 = 0;
  while (p0 < B) {
    // ---- 1. tables of a wave of points ---------------------------------------
    size_t freeb = 0, totb = 0;
    if (cudaMemGetInfo(&freeb, &totb) != cudaSuccess) { restore(); VFAIL(VCA_ERR_CUDA, "cudaMemGetInfo failed"); }
    const size_t per_point = 3 * (size_t)sumD * sizeof(double2) + ((size_t)8 << 20);
    const int P = (int)std::max<int64_t>(1, std::min<int64_t>(B - p0, (int64_t)(0.35 * (double)freeb / per_point)));
    const int p1 = p0 + P;
    std::vector<PointTabs> tabs(P);
    std::vector<std::vector<double>> bnd(P);  // per point: lower bound of every sector's energy
    bool cplx = false;
    for (int q = 0; q < P; q++) {
      int rc = set_hamiltonian(hl(p0 + q), bh(p0 + q), bv(p0 + q));
      if (rc) { restore(); return rc; }
      if (!c.no_sector_screen) bnd[q] = sector_lower_bounds();
      PointTabs& T = tabs[q];
      T.ham.ptrs.swap(g->ham.ptrs);  // the point keeps its tables; set_hamiltonian starts a new arena
      T.sp[0] = g->sp[0];
      T.sp[1] = g->sp[1];
      T.Hloc = g->Hloc;
      T.bath_h = g->bath_h;
      T.bath_v = g->bath_v;
      T.real_model = g->real_model;
      if (q == 0) cplx = !g->real_model;
      if (cplx != !g->real_model) {
        for (auto& t : tabs) t.ham.release();
        restore();
        VFAIL(VCA_ERR_UNSUPPORTED, "a batch mixes real and complex Hamiltonians");
      }
    }
    g->ham_set = false;  // g->sp points into the wave's tables until the final plain solve
    const size_t es = cplx ? sizeof(double2) : sizeof(double);
    auto cleanup = [&]() { for (auto& t : tabs) t.ham.release(); };
    lap(0);
    // ---- 2. the (point, sector) lowest energies ------------------------------
    // Screened in two runs when a lower bound exists (sector_lower_bounds):
    // first each point's two lowest-bound sectors, whose Ritz values give an
    // upper bound E_up on its ground energy, then only the sectors whose
    // bound lies below E_up + 20 GS_THRESHOLD.  A skipped sector's lowest
    // level is above every level within 20 GS_THRESHOLD of the ground state,
    // so the T=0 list (VCA_DIAG.f90:224-236) is the one of a full scan.
    const int LDS = std::min(c.lanc_niter, 512) + 1;  // svec rows kept per (point, sector)
    std::vector<double> theta((size_t)P * nsecs, INFINITY);
    std::vector<int> mconv((size_t)P * nsecs, 0);
    std::vector<double> svec_h((size_t)P * nsecs * LDS, 0.0);
    std::vector<char> done((size_t)P * nsecs, 0);
    auto run_search = [&](const std::vector<int>& which /* q * nsecs + (s - 1) */) -> int {
      if (which.empty()) return VCA_OK;
      TaskList S;
      int nmaxg = 1;
      for (int t : which) {
        const int q = t / nsecs, sct = t % nsecs + 1;
        const int nu = sec_nup(sct), nd = sec_ndw(sct);
        const int64_t D = (int64_t)g->dimn[nu] * g->dimn[nd];
        S.add(view_tabs(tabs[q], nu, nd), D, sct, 1);
        nmaxg = std::max(nmaxg, (int)std::min<int64_t>(D, std::min(c.lanc_niter, 512)));
      }
      const int ldg = nmaxg + 1;
      MtRun R;
      int rc = mt_alloc(R, S, ldg, es, false);
      if (rc) { R.ar.release(); return rc; }
      std::vector<ChainMeta> meta(S.secs.size());
      for (size_t t = 0; t < S.secs.size(); t++)
        meta[t] = ChainMeta{1, (int)t, (int)std::min<int64_t>(S.secs[t].D, std::min(c.lanc_niter, 512)), 1, 0};
      cudaMemcpyAsync(R.b.meta, meta.data(), sizeof(ChainMeta) * meta.size(), cudaMemcpyHostToDevice, g->st);
      m64_launch_start(R.gp, cplx, c.start_seed, R.b, g->st);
      for (int k = 1; k <= nmaxg; k++) {
        m64_launch_step(R.gp, cplx, g->md, k, c.gs_beta_tol, R.b, g->st);
        if (k % std::max(1, c.gs_check_every) == 0 || k == nmaxg) {
          cudaMemsetAsync(R.b.undone, 0, sizeof(int), g->st);
          m64_launch_check(R.gp, R.b, c.gs_residual_tol, g->st);
          int undone = 0;
          cudaMemcpyAsync(&undone, R.b.undone, sizeof(int), cudaMemcpyDeviceToHost, g->st);
          if (cudaStreamSynchronize(g->st) != cudaSuccess) { R.ar.release(); VFAIL(VCA_ERR_CUDA, "batched search failed"); }
          if (undone == 0) break;
        }
      }
      std::vector<double> th(S.secs.size()), sv(S.secs.size() * 5 * (size_t)ldg);
      std::vector<int> mc(S.secs.size());
      cudaMemcpyAsync(th.data(), R.b.theta, sizeof(double) * th.size(), cudaMemcpyDeviceToHost, g->st);
      cudaMemcpyAsync(mc.data(), R.b.mconv, sizeof(int) * mc.size(), cudaMemcpyDeviceToHost, g->st);
      cudaMemcpyAsync(sv.data(), R.b.svec, sizeof(double) * sv.size(), cudaMemcpyDeviceToHost, g->st);
      cudaError_t e = cudaStreamSynchronize(g->st);
      R.ar.release();
      if (e != cudaSuccess) VFAIL(VCA_ERR_CUDA, cudaGetErrorString(e));
      for (size_t i = 0; i < which.size(); i++) {
        const int t = which[i];
        theta[t] = th[i];
        mconv[t] = mc[i];
        done[t] = 1;
        const int n = std::min(mc[i], LDS);
        std::copy(sv.begin() + i * 5 * (size_t)ldg, sv.begin() + i * 5 * (size_t)ldg + n,
                  svec_h.begin() + (size_t)t * LDS);
      }
      return VCA_OK;
    };
    {
      std::vector<int> stageA, stageB;
      bool screened = true;
      for (int q = 0; q < P; q++) screened = screened && !bnd[q].empty();
      for (int q = 0; q < P; q++) {
        if (!screened) {
          for (int s2 = 0; s2 < nsecs; s2++) stageA.push_back(q * nsecs + s2);
          continue;
        }
        std::vector<int> ord(nsecs);
        for (int s2 = 0; s2 < nsecs; s2++) ord[s2] = s2;
        std::sort(ord.begin(), ord.end(), [&](int a, int b) { return bnd[q][a] < bnd[q][b]; });
        for (int r = 0; r < std::min(2, nsecs); r++) stageA.push_back(q * nsecs + ord[r]);
      }
      int rc = run_search(stageA);
      if (rc) { cleanup(); restore(); return rc; }
      if (screened) {
        for (int q = 0; q < P; q++) {
          double eup = INFINITY;
          for (int s2 = 0; s2 < nsecs; s2++)
            if (done[(size_t)q * nsecs + s2]) eup = std::min(eup, theta[(size_t)q * nsecs + s2]);
          const double cut = eup + 20.0 * c.gs_threshold + 1e-9 * std::max(1.0, std::fabs(eup));
          for (int s2 = 0; s2 < nsecs; s2++)
            if (!done[(size_t)q * nsecs + s2] && !(bnd[q][s2] > cut)) stageB.push_back(q * nsecs + s2);
        }
        rc = run_search(stageB);
        if (rc) { cleanup(); restore(); return rc; }
      }
      g->bt_skipped = 0;
      for (char d : done) g->bt_skipped += d ? 0 : 1;
    }
    lap(1);
    // ---- 3. T=0 lists -------------------------------------------------------
    std::vector<std::vector<ListEntry>> lists(P);
    for (int q = 0; q < P; q++) {
      std::vector<double> E(theta.begin() + (size_t)q * nsecs, theta.begin() + (size_t)(q + 1) * nsecs);
      replay_t0(E, c.gs_threshold, lists[q]);  // skipped sectors are +inf: never listed
      if (lists[q].empty()) { cleanup(); restore(); VFAIL(VCA_ERR_NUMERIC, "no ground state found"); }
    }
    // ---- 4. eigenvectors of the kept (point, sector) tasks -------------------
    TaskList V;
    std::vector<int> vsrc;  // (point, sector) index of each eigenvector task
    for (int q = 0; q < P; q++)
      for (const ListEntry& x : lists[q]) {
        const int t = q * nsecs + (x.sector - 1);
        const int nu = sec_nup(x.sector), nd = sec_ndw(x.sector);
        V.add(view_tabs(tabs[q], nu, nd), (int64_t)g->dimn[nu] * g->dimn[nd], x.sector, 1);
        vsrc.push_back(t);
      }
    MtRun RV;  // holds the ground-state vectors (psi) until the chains are done
    char* psi = nullptr;
    {
      int mmax = 1;
      for (size_t v = 0; v < V.secs.size(); v++) mmax = std::max(mmax, mconv[vsrc[v]]);
      const int ldv = mmax + 1;
      int rc = mt_alloc(RV, V, ldv, es, true);
      if (!rc) rc = RV.ar.alloc(&psi, (size_t)V.tot * es);
      double* d_svec = nullptr;
      int* d_mc = nullptr;
      if (!rc) rc = RV.ar.alloc(&d_svec, V.secs.size() * 5 * (size_t)ldv);
      if (!rc) rc = RV.ar.alloc(&d_mc, V.secs.size());
      if (rc) { RV.ar.release(); cleanup(); restore(); return rc; }
      std::vector<double> sv(V.secs.size() * 5 * (size_t)ldv, 0.0);
      std::vector<int> mc(V.secs.size());
      std::vector<ChainMeta> meta(V.secs.size());
      for (size_t v = 0; v < V.secs.size(); v++) {
        mc[v] = mconv[vsrc[v]];
        std::copy(svec_h.begin() + (size_t)vsrc[v] * LDS, svec_h.begin() + (size_t)vsrc[v] * LDS + std::min(mc[v], LDS),
                  sv.begin() + v * 5 * (size_t)ldv);
        if (mc[v] < 1) { RV.ar.release(); cleanup(); restore(); VFAIL(VCA_ERR_NUMERIC, "Lanczos start vector has zero norm"); }
        meta[v] = ChainMeta{1, (int)v, mc[v], 1, 0};
      }
      cudaMemcpyAsync(d_svec, sv.data(), sizeof(double) * sv.size(), cudaMemcpyHostToDevice, g->st);
      cudaMemcpyAsync(d_mc, mc.data(), sizeof(int) * mc.size(), cudaMemcpyHostToDevice, g->st);
      cudaMemcpyAsync(RV.b.meta, meta.data(), sizeof(ChainMeta) * meta.size(), cudaMemcpyHostToDevice, g->st);
      cudaMemsetAsync(psi, 0, (size_t)V.tot * es, g->st);
      m64_launch_start(RV.gp, cplx, c.start_seed, RV.b, g->st);
      for (int k = 1; k <= mmax; k++) {  // psi = sum_k s_k x_k (sector_gs's second pass, every task at once)
        m64_launch_psi(RV.gp, cplx, d_svec, 5 * ldv, d_mc, k, RV.b.X, psi, g->st);
        if (k < mmax) m64_launch_step(RV.gp, cplx, g->md, k, c.gs_beta_tol, RV.b, g->st);
      }
      m64_launch_sqnorm(RV.gp, cplx, psi, RV.b.tpart, g->st);
      mt_launch_norm(RV.gp, RV.b.tpart, RV.b.meta, RV.n2, RV.b.invb, g->st);
      m64_launch_scale(RV.gp, cplx, RV.b.invb, psi, psi, g->st);
      if (cudaStreamSynchronize(g->st) != cudaSuccess || cudaGetLastError() != cudaSuccess) {
        RV.ar.release(); cleanup(); restore();
        VFAIL(VCA_ERR_CUDA, "batched eigenvector pass failed");
      }
    }
    lap(2);
    // ---- 5. chains of every point --------------------------------------------
    std::vector<std::vector<BChain>> pch(P);
    {
      int v = 0;
      for (int q = 0; q < P; q++)
        for (int k = 0; k < (int)lists[q].size(); k++, v++) {
          const ListEntry& st = lists[q][k];
          const int nup = sec_nup(st.sector), ndw = sec_ndw(st.sector);
          const void* gsv = psi + (size_t)V.secs[v].off * es;
          for (int is = 0; is < c.Nspin; is++)
            for (int dag = 1; dag >= 0; dag--) {  // the particle batch, then the hole batch (build_gf's order)
              const int tup = nup + (is == 0 ? (dag ? 1 : -1) : 0);
              const int tdw = ndw + (is == 1 ? (dag ? 1 : -1) : 0);
              if (tup < 0 || tup > Ns || tdw < 0 || tdw > Ns) continue;
              auto add = [&](int e, int chan, int p, cd cp, int qq, cd cq, int nterm, cd wfac) {
                BChain b{};
                b.point = q;
                b.state = k;
                b.mc.gs = gsv;
                b.mc.src_dimup = tabs[q].sp[0][nup].dim;
                b.mc.spin = is;
                b.mc.dag = dag;
                b.mc.nterm = nterm;
                b.mc.pos[0] = p;
                b.mc.cre[0] = cp.real();
                b.mc.cim[0] = cp.imag();
                b.mc.pos[1] = qq;
                b.mc.cre[1] = cq.real();
                b.mc.cim[1] = cq.imag();
                const bool imagcoef = (cp.imag() != 0.0) || (nterm > 1 && cq.imag() != 0.0);
                b.ncomp = (!cplx && imagcoef) ? 2 : 1;
                b.rec = ChainRec{e, k, chan, 0};
                b.isign = dag ? 1 : -1;
                b.wfac = wfac;
                b.tup = tup;
                b.tdw = tdw;
                pch[q].push_back(b);
              };
              for (int io = 0; io < c.Norb; io++)
                for (int il = 0; il < c.Nlat; il++) {
                  const int p = io + il * c.Norb;
                  add(elem_index(c, il, il, is, io, io), dag ? 1 : 2, p, 1.0, 0, 0.0, 1, 1.0);
                  for (int jl = 0; jl < c.Nlat; jl++)
                    for (int jo = 0; jo < c.Norb; jo++) {
                      if (il == jl && io == jo) continue;
                      const int qq = jo + jl * c.Norb;
                      const int e = elem_index(c, il, jl, is, io, jo);
                      add(e, dag ? 1 : 2, p, 1.0, qq, 1.0, 2, 1.0);
                      if (!c.vca_gf_symmetric) {
                        if (dag) add(e, 3, p, 1.0, qq, XI, 2, -XI);
                        else add(e, 4, p, 1.0, qq, -XI, 2, -XI);
                      }
                    }
                }
            }
        }
    }
    (void)L;
    g->ld = std::max(1, c.lanc_ngfiter);
    const int ld = g->ld;
    // per-point chain stores
    Arena stores;
    std::vector<ChainStore> cs(P);
    for (int q = 0; q < P; q++) {
      const size_t n = std::max<size_t>(1, pch[q].size());
      ChainStore& s = cs[q];
      s.ld = ld;
      int rc = VCA_OK;
      if ((rc = stores.alloc(&s.A, n * ld)) || (rc = stores.alloc(&s.B, n * ld)) || (rc = stores.alloc(&s.n, n)) ||
          (rc = stores.alloc(&s.pes, n)) || (rc = stores.alloc(&s.isign, n)) || (rc = stores.alloc(&s.wfac, n)) ||
          (rc = stores.alloc(&s.Ei, n))) {
        stores.release(); RV.ar.release(); cleanup(); restore();
        return rc;
      }
      cudaMemsetAsync(s.n, 0, sizeof(int) * n, g->st);
    }
    {
      // column tasks: the chains of one (point, state, spin, particle/hole)
      // share a target sector and run as one task of m columns; tasks are
      // grouped point-major under a memory budget
      std::vector<McTaskRef> trefs;
      for (int q = 0; q < P; q++) {
        int i = 0;
        const int n = (int)pch[q].size();
        while (i < n) {
          const BChain& b0 = pch[q][i];
          int j = i, m = 0;
          while (j < n && pch[q][j].state == b0.state && pch[q][j].mc.spin == b0.mc.spin &&
                 pch[q][j].mc.dag == b0.mc.dag) {
            m += pch[q][j].ncomp;
            j++;
          }
          trefs.push_back({q, i, j, (int64_t)g->dimn[b0.tup] * g->dimn[b0.tdw], m});
          i = j;
        }
      }
      size_t fb = 0;
      cudaMemGetInfo(&fb, &totb);
      const size_t gbudget = (size_t)(0.3 * (double)fb);
      size_t t0i = 0;
      while (t0i < trefs.size()) {
        size_t t1i = t0i;
        int64_t tot = 0;
        while (t1i < trefs.size()) {
          const int64_t add = trefs[t1i].D * trefs[t1i].m;
          if (t1i > t0i && 3 * (size_t)(tot + add) * es > gbudget) break;
          tot += add;
          t1i++;
        }
        const McShape shape = mc_autotune(trefs, t0i, t1i, pch, tabs, cplx, es);
        g->bt_shape[0] = shape.R;
        g->bt_shape[1] = shape.by;
        McHost h;
        mc_build(trefs, t0i, t1i, pch, tabs, shape.R, c.lanc_ngfiter, h);
        const int nch = (int)h.chains.size();
        const int nl_max = h.nl_max;
        const int64_t xoff = h.xoff, part = h.part;
        const std::vector<int>& ch_point = h.ch_point;
        const std::vector<int>& ch_index = h.ch_index;
        Arena ar;
        McGroup gp;
        ChainMeta* d_meta;
        int* d_isg;
        double *d_tp, *d_al, *d_b2, *d_bn, *d_ib, *d_A, *d_B, *d_n2, *d_in;
        double2* d_wf;
        char *x0, *x1, *x2;
        int rc = mc_upload(h, shape.by, ar, gp, &d_meta);
        if (!rc)
          (void)((rc = ar.alloc(&d_tp, (size_t)part)) || (rc = ar.alloc(&d_al, nch)) || (rc = ar.alloc(&d_b2, nch)) ||
                 (rc = ar.alloc(&d_bn, nch)) || (rc = ar.alloc(&d_ib, nch)) ||
                 (rc = ar.alloc(&d_A, (size_t)nch * ld)) || (rc = ar.alloc(&d_B, (size_t)nch * ld)) ||
                 (rc = ar.alloc(&d_n2, nch)) || (rc = ar.alloc(&d_in, nch)) || (rc = ar.alloc(&d_isg, nch)) ||
                 (rc = ar.alloc(&d_wf, nch)) || (rc = ar.alloc(&x0, (size_t)xoff * es)) ||
                 (rc = ar.alloc(&x1, (size_t)xoff * es)) || (rc = ar.alloc(&x2, (size_t)xoff * es)));
        if (rc) {
          ar.release(); stores.release(); RV.ar.release(); cleanup(); restore();
          return rc;
        }
        cudaMemcpyAsync(d_isg, h.isg.data(), sizeof(int) * nch, cudaMemcpyHostToDevice, g->st);
        cudaMemcpyAsync(d_wf, h.wf.data(), sizeof(double2) * nch, cudaMemcpyHostToDevice, g->st);
        cudaMemsetAsync(d_A, 0, sizeof(double) * nch * ld, g->st);
        cudaMemsetAsync(d_B, 0, sizeof(double) * nch * ld, g->st);
        cudaMemsetAsync(d_bn, 0, sizeof(double) * nch, g->st);
        void *X = x0, *Xp = x1, *Y = x2;
        // start vectors c^(dag)|gs>, normalised; norm^2 kept for the weights
        mc_launch_chain_init(gp, cplx, X, d_tp, g->st);
        mc_launch_reduce(gp, d_tp, d_n2, g->st);
        launch_chain_norm_init(nch, d_meta, d_n2, d_in, g->st);
        mc_launch_scale(gp, cplx, d_meta, d_in, X, X, g->st);
        for (int k = 1; k <= nl_max; k++) {
          mc_launch_hxv(gp, cplx, g->md, d_meta, d_bn, k > 1 ? 1 : 0, X, Xp, Y, d_tp, g->st);
          mc_launch_reduce(gp, d_tp, d_al, g->st);
          mc_launch_update(gp, cplx, d_meta, d_al, X, Y, d_tp, g->st);
          mc_launch_reduce(gp, d_tp, d_b2, g->st);
          launch_lanczos_record(nch, d_meta, k, d_al, d_b2, d_A, d_B, ld, c.gf_beta_tol, d_ib, d_bn, g->st);
          mc_launch_scale(gp, cplx, d_meta, d_ib, Y, Y, g->st);
          void* t = Xp;  // (X, Xp, Y) <- (Y, X, Xp)
          Xp = X;
          X = Y;
          Y = t;
        }
        // into the stores: runs of one (point, state)
        int r0 = 0;
        while (r0 < nch) {
          int r1 = r0;
          while (r1 < nch && ch_point[r1] == ch_point[r0] &&
                 pch[ch_point[r1]][ch_index[r1]].state == pch[ch_point[r0]][ch_index[r0]].state)
            r1++;
          const int q = ch_point[r0];
          const BChain& b0 = pch[q][ch_index[r0]];
          launch_chain_store(r1 - r0, d_meta + r0, d_A + (size_t)r0 * ld, d_B + (size_t)r0 * ld, ld, d_n2 + r0,
                             d_wf + r0, d_isg + r0, lists[q][b0.state].e, 1.0, (double)lists[q].size(), cs[q],
                             ch_index[r0], g->st);
          r0 = r1;
        }
        cudaError_t e = cudaStreamSynchronize(g->st);
        if (e == cudaSuccess) e = cudaGetLastError();
        ar.release();
        if (e != cudaSuccess) { stores.release(); RV.ar.release(); cleanup(); restore(); VFAIL(VCA_ERR_CUDA, cudaGetErrorString(e)); }
        t0i = t1i;
      }
    }
    RV.ar.release();  // the ground-state vectors are no longer needed
    lap(3);
    // ---- 6. Omega per point --------------------------------------------------
    for (int q = 0; q < P; q++) {
      g->Hloc = tabs[q].Hloc;
      g->bath_h = tabs[q].bath_h;
      g->bath_v = tabs[q].bath_v;
      g->real_model = tabs[q].real_model;
      g->gs.clear();
      for (const ListEntry& x : lists[q]) g->gs.push_back(GState{x.sector, x.e, nullptr});
      g->egs = INFINITY;
      for (auto& s : g->gs) g->egs = std::min(g->egs, s.e);
      g->zeta = (double)g->gs.size();
      g->chains.clear();
      for (const BChain& b : pch[q]) {
        ChainRec r = b.rec;
        const int64_t Dsec = (int64_t)g->dimn[b.tup] * g->dimn[b.tdw];
        r.nlanc = (int)std::min<int64_t>(Dsec, c.lanc_ngfiter);
        g->chains.push_back(r);
      }
      g->cstore = cs[q];
      g->poles_ready = false;
      g->nelem = c.Nlat * c.Nlat * c.Nspin * c.Norb * c.Norb;
      std::vector<std::vector<int>> lst(g->nelem);
      for (int ch = 0; ch < (int)g->chains.size(); ch++) lst[g->chains[ch].elem].push_back(ch);
      std::vector<int> ptr(g->nelem + 1, 0), flat;
      for (int e = 0; e < g->nelem; e++) {
        ptr[e + 1] = ptr[e] + (int)lst[e].size();
        flat.insert(flat.end(), lst[e].begin(), lst[e].end());
      }
      Arena csr;
      int rc = csr.alloc(&g->d_elem_ptr, ptr.size());
      if (!rc) rc = csr.alloc(&g->d_elem_chain, std::max<size_t>(1, flat.size()));
      if (!rc) {
        cudaMemcpyAsync(g->d_elem_ptr, ptr.data(), sizeof(int) * ptr.size(), cudaMemcpyHostToDevice, g->st);
        if (!flat.empty())
          cudaMemcpyAsync(g->d_elem_chain, flat.data(), sizeof(int) * flat.size(), cudaMemcpyHostToDevice, g->st);
        double oi = 0.0;
        rc = omega_integral(&oi);
        if (!rc) omega_out[p0 + q] = g->egs - oi;  // VCA_MAIN.f90:183-197 at T=0
      }
      csr.release();
      g->d_elem_ptr = g->d_elem_chain = nullptr;
      g->cstore = ChainStore{};
      g->chains.clear();
      if (rc) { stores.release(); cleanup(); restore(); return rc; }
    }
    stores.release();
    cleanup();
    lap(4);
    p0 = p1;
  }
  restore();
  // the context as a loop of vca_solve leaves it: the last point, plain path
  double last = 0.0;
  RCHK(solve_resident(hl(B - 1), bh(B - 1), bv(B - 1), &last));
  lap(5);
  if (std::fabs(last - omega_out[B - 1]) > 1e-10 * std::max(1.0, std::fabs(last)))
    VFAIL(VCA_ERR_NUMERIC, "batched and plain Omega of the last point disagree");
  return VCA_OK;
}

}  // namespace

namespace vca {
// error text of the last failed call of any entry point (vca_gpu_last_error)
void set_api_error(const std::string& m) { g_err = m; }
}  // namespace vca

// ===========================================================================
// C-ABI
// ===========================================================================
// Forgets the cached device addresses of the allocation-free entry point's
// static scratch (defined at the end of this file).
static void noalloc_forget();

extern "C" {

void vca_config_defaults(vca_config* c) {
  if (!c) return;
  std::memset(c, 0, sizeof(*c));
  c->Norb = 1;
  c->Nspin = 1;
  c->Nlat = 1;
  c->Nlat_bath = 0;
  c->Norb_bath = 0;
  c->Uloc[0] = 2.0;
  c->beta = 1000.0;
  c->xmu = 0.0;
  c->hfmode = 1;
  c->hfshift = 1;
  c->Lmats = 5000;
  c->Lreal = 5000;
  c->wini = -5.0;
  c->wfin = 5.0;
  c->eps = 0.01;
  c->vca_twin = 0;
  c->vca_sectors = 0;
  c->vca_sectors_shift = 1;
  c->vca_sparse_H = 1;
  c->vca_gf_symmetric = 0;
  c->lanc_method = VCA_LANC_ARPACK;
  c->lanc_nstates_sector = 6;
  c->lanc_nstates_total = 1;
  c->lanc_niter = 512;
  c->lanc_ngfiter = 200;
  c->lanc_tolerance = 1e-12;
  c->lanc_dim_threshold = 256;
  c->gs_threshold = 1e-9;
  c->verbose = 3;
  c->omega_nodes = 4096;
  c->gs_check_every = 10;
  c->omega_scale = 1.0;
  c->gs_residual_tol = 1e-11;
  c->gf_beta_tol = 1e-6;
  c->gs_beta_tol = 1e-12;
  c->start_seed = 20261203ull;
  c->lanc_nstates_step = 2;     // VCA_INPUT_VARS.f90:155
  c->lanc_niter_spectrum = 10;  // VCA_INPUT_VARS.f90:159
  c->cutoff = 1e-9;             // VCA_INPUT_VARS.f90:169
  c->bandwidth = 0.0;
  c->contour_nodes = 24;
  c->print_sigma = c->print_impg = c->print_impg0 = 0;  // on in the reference (VCA_INPUT_VARS.f90:137-139)
  c->file_suffix[0] = 0;
}

int vca_gpu_last_error(char* buf, int32_t len) {
  if (buf && len > 0) {
    std::strncpy(buf, g_err.c_str(), (size_t)len - 1);
    buf[len - 1] = 0;
  }
  return (int)g_err.size();
}

int vca_gpu_finalize(void) {
  noalloc_forget();
  if (!g) return VCA_OK;
  gfm_drop();
  g->work.release();
  g->nodes.release();
  g->omega.release();
  g->gf.release();
  g->states.release();
  g->ham.release();
  g->basis.release();
  if (g->st) cudaStreamDestroy(g->st);
  if (g->st2) cudaStreamDestroy(g->st2);
  delete g;
  g = nullptr;
  return VCA_OK;
}

int vca_gpu_init(const vca_config* cfg, const double* bath_h, const double* bath_v) {
  g_err.clear();
  if (!cfg) VFAIL(VCA_ERR_ARG, "cfg is NULL");
  vca_config c = *cfg;
  if ((bath_h == nullptr) != (bath_v == nullptr)) VFAIL(VCA_ERR_ARG, "bath_h and bath_v must be given together");
  const bool has_bath = bath_h != nullptr;
  if (has_bath && (c.Nlat_bath < 1 || c.Norb_bath < 1))
    VFAIL(VCA_ERR_CONFIG, "VCA_INIT_SOLVER error: wrong bath dimensions");  // VCA_MAIN.f90:61
  if (!has_bath) { c.Nlat_bath = 0; c.Norb_bath = 0; }  // VCA_MAIN.f90:64-66
  if (c.Nspin < 1 || c.Nspin > 2) VFAIL(VCA_ERR_CONFIG, "ED ERROR: Nspin > 2 is currently not supported");
  if (c.Norb < 1 || c.Norb > 5) VFAIL(VCA_ERR_CONFIG, "ED ERROR: Norb > 5 is currently not supported");
  if (c.Nlat < 1) VFAIL(VCA_ERR_CONFIG, "Nlat must be >= 1");
  const bool finiteT = c.lanc_nstates_total != 1;  // VCA_SETUP.f90:157-162
  if (finiteT) {
    if (c.lanc_nstates_total < 1) VFAIL(VCA_ERR_CONFIG, "LANC_NSTATES_TOTAL must be >= 1");
    if (c.lanc_niter_spectrum < 1) VFAIL(VCA_ERR_CONFIG, "LANC_NITER_SPECTRUM must be >= 1");
    if (c.lanc_nstates_step < 0) VFAIL(VCA_ERR_CONFIG, "LANC_NSTATES_STEP must be >= 0");
    if (!(c.beta > 0.0) || !std::isfinite(c.beta)) VFAIL(VCA_ERR_CONFIG, "BETA must be > 0");
    if (!(c.cutoff > 0.0 && c.cutoff < 1.0)) VFAIL(VCA_ERR_CONFIG, "CUTOFF must lie in (0,1)");
    if (c.contour_nodes < 2) VFAIL(VCA_ERR_CONFIG, "contour_nodes must be >= 2");
    if (!std::isfinite(c.bandwidth)) VFAIL(VCA_ERR_CONFIG, "bandwidth must be finite");
  }
  if (c.vca_twin) VFAIL(VCA_ERR_UNSUPPORTED, "VCA_TWIN is outside the GPU path");
  if (strnlen(c.file_suffix, sizeof c.file_suffix) == sizeof c.file_suffix)
    VFAIL(VCA_ERR_CONFIG, "file_suffix is not NUL-terminated within 64 characters");
  if (c.lanc_ngfiter < 1 || c.lanc_niter < 1) VFAIL(VCA_ERR_CONFIG, "LANC_NITER and LANC_NGFITER must be >= 1");
  if (c.omega_nodes < 2) VFAIL(VCA_ERR_CONFIG, "omega_nodes must be >= 2");
  if (!(c.omega_scale > 0.0)) VFAIL(VCA_ERR_CONFIG, "omega_scale must be > 0");
  if (c.gs_check_every < 1) c.gs_check_every = 1;
  const int Ns = c.Nlat * c.Norb + c.Nlat_bath * c.Norb_bath;  // VCA_SETUP.f90:82
  if (Ns > VCA_MAX_NS) VFAIL(VCA_ERR_UNSUPPORTED, "more than 24 levels per spin");
  vca_gpu_finalize();
  g = new Ctx();
  g->cfg = c;
  g->has_bath = has_bath;
  g->Ns = Ns;
  g->Nsectors = (Ns + 1) * (Ns + 1);  // VCA_SETUP.f90:93
  g->N = c.Nlat * c.Nspin * c.Norb;
  g->L = c.Nlat * c.Norb;
  g->Nb = c.Nlat_bath * c.Nspin * c.Norb_bath;
  g->finiteT = finiteT;
  g->nstates_total = c.lanc_nstates_total;
  if (finiteT && g->nstates_total % 2 != 0) g->nstates_total++;  // VCA_SETUP.f90:172-175
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev < 1) {
    g_err = "no CUDA device available: the GPU path has no CPU fallback";
    delete g;
    g = nullptr;
    cudaGetLastError();
    return VCA_ERR_CUDA;
  }
  // a blocking stream: the synchronous getters on the legacy stream order after it
  CUCHK(cudaStreamCreate(&g->st));
  CUCHK(cudaStreamCreate(&g->st2));
  set_binomials(Ns, g->st);
  g->dimn.resize(Ns + 1);
  g->words.resize(Ns + 1);
  for (int n = 0; n <= Ns; n++) {
    g->dimn[n] = (int)binom_h(Ns, n);
    RCHK(g->basis.alloc(&g->words[n], g->dimn[n]));
    launch_build_words(Ns, n, g->dimn[n], g->words[n], g->st);
  }
  RCHK(g->basis.alloc(&g->d_iscratch, 16));
  CUCHK(cudaGetLastError());
  CUCHK(cudaStreamSynchronize(g->st));
  return VCA_OK;
}

int vca_gpu_set_hamiltonian(const double* Hloc, const double* bath_h, const double* bath_v) {
  if (!g) VFAIL(VCA_ERR_STATE, "vca_gpu_init has not been called");
  return set_hamiltonian(Hloc, bath_h, bath_v);
}

static int print_after_solve();

int vca_gpu_solve(const double* Hloc, const double* Hk, int64_t Nk, const double* bath_h,
                  const double* bath_v, double* omega_out) {
  g_err.clear();
  if (!g) VFAIL(VCA_ERR_STATE, "vca_gpu_init has not been called");
  RCHK(solve_one(Hloc, Hk, Nk, bath_h, bath_v, omega_out));
  return print_after_solve();
}

int vca_gpu_solve_batch(int32_t B, const double* Hloc, int64_t stride_hloc, const double* Hk, int64_t Nk,
                        const double* bath_h, int64_t stride_bath_h, const double* bath_v,
                        int64_t stride_bath_v, double* omega_out) {
  g_err.clear();
  if (!g) VFAIL(VCA_ERR_STATE, "vca_gpu_init has not been called");
  if (B < 0 || !omega_out) VFAIL(VCA_ERR_ARG, "bad batch arguments");
  if (B == 0) return VCA_OK;
  RCHK(upload_hk(Hk, Nk));  // shared by every point: uploaded (and its k-pairs found) once
  if (B >= 2 && !g->finiteT && !g->cfg.batch_loop) {
    RCHK(solve_batch_fused(B, Hloc, stride_hloc, bath_h, stride_bath_h, bath_v, stride_bath_v, omega_out));
    return print_after_solve();
  }
  for (int b = 0; b < B; b++) {
    RCHK(solve_resident(Hloc + 2 * (size_t)b * stride_hloc,
                        bath_h ? bath_h + 2 * (size_t)b * stride_bath_h : nullptr,
                        bath_v ? bath_v + 2 * (size_t)b * stride_bath_v : nullptr, omega_out + b));
  }
  return print_after_solve();  // the files of the last point, as a loop of vca_solve leaves them
}

int vca_gpu_get_sft_potential(double* omega) {
  if (!g || !g->solved) VFAIL(VCA_ERR_STATE, "no completed vca_gpu_solve");
  if (!omega) VFAIL(VCA_ERR_ARG, "NULL output");
  *omega = g->sft;
  return VCA_OK;
}

int vca_gpu_get_energies(double* egs, double* omega_int) {
  if (!g || !g->solved) VFAIL(VCA_ERR_STATE, "no completed vca_gpu_solve");
  if (egs) *egs = g->egs;
  if (omega_int) *omega_int = g->omega_int;
  return VCA_OK;
}

int vca_gpu_get_state_count(int32_t* nstates) {
  if (!g || !g->solved) VFAIL(VCA_ERR_STATE, "no completed vca_gpu_solve");
  *nstates = (int32_t)g->gs.size();
  return VCA_OK;
}

int vca_gpu_get_state(int32_t istate, int32_t* isector, double* energy) {
  if (!g || !g->solved) VFAIL(VCA_ERR_STATE, "no completed vca_gpu_solve");
  if (istate < 1 || istate > (int)g->gs.size()) VFAIL(VCA_ERR_ARG, "state index out of range");
  if (isector) *isector = g->gs[istate - 1].sector;
  if (energy) *energy = g->gs[istate - 1].e;
  return VCA_OK;
}

int vca_gpu_get_sector_energies(double* e_out, int32_t n) {
  if (!g || g->sector_e.empty()) VFAIL(VCA_ERR_STATE, "no diagonalisation yet");
  if (!e_out || n < g->Nsectors) VFAIL(VCA_ERR_ARG, "output too small");
  for (int i = 0; i < g->Nsectors; i++) e_out[i] = g->sector_e[i];
  return VCA_OK;
}

int vca_gpu_get_gf_channel(int32_t ilat, int32_t jlat, int32_t ispin, int32_t iorb, int32_t jorb,
                           int32_t istate, int32_t ichan, int32_t* nexc, double* poles, double* weights,
                           int32_t cap) {
  if (!g || !(g->solved || g->gfm_loaded)) VFAIL(VCA_ERR_STATE, "no completed vca_gpu_solve");
  const vca_config& c = g->cfg;
  if (ilat < 1 || ilat > c.Nlat || jlat < 1 || jlat > c.Nlat || ispin < 1 || ispin > c.Nspin ||
      iorb < 1 || iorb > c.Norb || jorb < 1 || jorb > c.Norb)
    VFAIL(VCA_ERR_ARG, "element index out of range");
  if (nexc) *nexc = 0;  // channel absent (no target sector): Nexc=0 in the reference
  if (g->gfm_loaded) {
    const GfmTable& t = g->gfm;
    const int64_t f = gfm_elem(c, ilat - 1, jlat - 1, ispin - 1, iorb - 1, jorb - 1);
    if (istate < 1 || istate > t.nstates[f]) return VCA_OK;
    const int64_t st = g->gfm_state0[f] + istate - 1;
    if (ichan < 1 || ichan > t.nchan[st]) return VCA_OK;
    const int64_t ci = g->gfm_chan0[st] + ichan - 1;
    const int n = t.nexc[ci];
    const int64_t x0 = g->gfm_exc0[ci];
    if (nexc) *nexc = n;
    if (cap >= n) {
      if (poles) std::memcpy(poles, t.poles.data() + 2 * x0, sizeof(double) * 2 * n);
      if (weights) std::memcpy(weights, t.weights.data() + 2 * x0, sizeof(double) * 2 * n);
    }
    return VCA_OK;
  }
  const int e = elem_index(c, ilat - 1, jlat - 1, ispin - 1, iorb - 1, jorb - 1);
  RCHK(ensure_poles());
  for (int ch = 0; ch < (int)g->chains.size(); ch++) {
    const ChainRec& r = g->chains[ch];
    if (r.elem != e || r.state != istate - 1 || r.chan != ichan) continue;
    int n = 0, sg = 1;
    CUCHK(cudaMemcpy(&n, g->d_nexc + ch, sizeof(int), cudaMemcpyDeviceToHost));
    CUCHK(cudaMemcpy(&sg, g->cstore.isign + ch, sizeof(int), cudaMemcpyDeviceToHost));
    std::vector<double> p(std::max(n, 1));
    std::vector<double2> w(std::max(n, 1));
    if (n > 0) {
      CUCHK(cudaMemcpy(p.data(), g->d_poles + (size_t)ch * g->ld, sizeof(double) * n, cudaMemcpyDeviceToHost));
      CUCHK(cudaMemcpy(w.data(), g->d_weights + (size_t)ch * g->ld, sizeof(double2) * n, cudaMemcpyDeviceToHost));
    }
    std::vector<double2> P, W;
    chain_table(r, n, sg, p.data(), w.data(), P, W);
    if (nexc) *nexc = (int32_t)P.size();
    if (cap >= (int)P.size()) {
      if (poles) std::memcpy(poles, P.data(), sizeof(double2) * P.size());
      if (weights) std::memcpy(weights, W.data(), sizeof(double2) * W.size());
    }
    return VCA_OK;
  }
  return VCA_OK;
}

int vca_gpu_save_gfprime(const char* file, const char* suffix, int32_t used, int32_t formatted) {
  if (!g || !(g->solved || g->gfm_loaded))
    VFAIL(VCA_ERR_STATE, "vca_gf_cluster ERROR: impGmatrix not allocated!");  // VCA_AUX_FUNX.f90:614
  if (!file) VFAIL(VCA_ERR_ARG, "file is NULL");
  std::string err;
  if (g->gfm_loaded) {
    if (gfm_write(gfm_path(file, suffix, used), formatted != 0, g->gfm, err)) VFAIL(VCA_ERR_IO, err);
    return VCA_OK;
  }
  GfmTable t;
  RCHK(solve_tables(t));
  if (gfm_write(gfm_path(file, suffix, used), formatted != 0, t, err)) VFAIL(VCA_ERR_IO, err);
  return VCA_OK;
}

int vca_gpu_read_gfprime(const char* file, const char* suffix, int32_t used, int32_t formatted) {
  if (!g || !g->basis.ptrs.size()) VFAIL(VCA_ERR_STATE, "vca_gpu_init has not been called");
  if (!file) VFAIL(VCA_ERR_ARG, "file is NULL");
  const vca_config& c = g->cfg;
  const int64_t nelem = (int64_t)c.Nlat * c.Nlat * c.Nspin * c.Norb * c.Norb;
  GfmTable t;
  std::string err;
  if (gfm_read(gfm_path(file, suffix, used), formatted != 0, nelem, t, err)) VFAIL(VCA_ERR_IO, err);
  // offsets into the flattened counts, and each file element's excitations
  // (contiguous in file order)
  std::vector<int64_t> s0(nelem), c0(t.nchan.size()), x0(t.nexc.size()), ex0(nelem + 1);
  int64_t a = 0, b = 0, x = 0;
  for (int64_t f = 0; f < nelem; f++) {
    s0[f] = a;
    ex0[f] = x;
    for (int k = 0; k < t.nstates[f]; k++, a++) {
      c0[a] = b;
      for (int q = 0; q < t.nchan[a]; q++, b++) {
        x0[b] = x;
        x += t.nexc[b];
      }
    }
  }
  ex0[nelem] = x;
  // device layout: elements in elem_index order
  std::vector<int64_t> ptr(nelem + 1, 0);
  std::vector<int64_t> src(nelem);  // file element of each elem_index
  for (int il = 0; il < c.Nlat; il++)
    for (int jl = 0; jl < c.Nlat; jl++)
      for (int is = 0; is < c.Nspin; is++)
        for (int io = 0; io < c.Norb; io++)
          for (int jo = 0; jo < c.Norb; jo++) src[elem_index(c, il, jl, is, io, jo)] = gfm_elem(c, il, jl, is, io, jo);
  for (int64_t e = 0; e < nelem; e++) ptr[e + 1] = ptr[e] + (ex0[src[e] + 1] - ex0[src[e]]);
  std::vector<double2> hp((size_t)std::max<int64_t>(x, 1)), hw((size_t)std::max<int64_t>(x, 1));
  for (int64_t e = 0; e < nelem; e++) {
    const int64_t f = src[e], n = ex0[f + 1] - ex0[f];
    if (n) {
      std::memcpy(hp.data() + ptr[e], t.poles.data() + 2 * ex0[f], sizeof(double2) * n);
      std::memcpy(hw.data() + ptr[e], t.weights.data() + 2 * ex0[f], sizeof(double2) * n);
    }
  }
  gfm_drop();
  int rc;
  if ((rc = g->gfm_dev.alloc(&g->d_gfm_ptr, nelem + 1)) || (rc = g->gfm_dev.alloc(&g->d_gfm_p, hp.size())) ||
      (rc = g->gfm_dev.alloc(&g->d_gfm_w, hw.size()))) {
    gfm_drop();
    return rc;
  }
  cudaError_t ce = cudaMemcpy(g->d_gfm_ptr, ptr.data(), sizeof(int64_t) * ptr.size(), cudaMemcpyHostToDevice);
  if (ce == cudaSuccess) ce = cudaMemcpy(g->d_gfm_p, hp.data(), sizeof(double2) * hp.size(), cudaMemcpyHostToDevice);
  if (ce == cudaSuccess) ce = cudaMemcpy(g->d_gfm_w, hw.data(), sizeof(double2) * hw.size(), cudaMemcpyHostToDevice);
  if (ce != cudaSuccess) {
    gfm_drop();
    VFAIL(VCA_ERR_CUDA, cudaGetErrorString(ce));
  }
  g->gfm = std::move(t);
  g->gfm_state0 = std::move(s0);
  g->gfm_chan0 = std::move(c0);
  g->gfm_exc0 = std::move(x0);
  g->gfm_loaded = true;
  return VCA_OK;
}


// G'(z) at nz host points into the caller's (Nlat,Nlat,Nspin,Nspin,Norb,
// Norb,nz) array; solve_tables as in gf_lso
static int gf_cluster_host(const double* z, int64_t nz, double* gf_out, bool solve_tables) {
  if (!z || !gf_out || nz < 0) VFAIL(VCA_ERR_ARG, "bad arguments");
  if (nz == 0) return VCA_OK;
  const vca_config& c = g->cfg;
  const int N = g->N, NN = N * N;
  Arena ar;
  double2 *dz, *Glso;
  int rc;
  if ((rc = ar.alloc(&dz, nz)) || (rc = ar.alloc(&Glso, (size_t)nz * NN))) { ar.release(); return rc; }
  cudaMemcpyAsync(dz, z, sizeof(double2) * nz, cudaMemcpyHostToDevice, g->st);
  if ((rc = gf_lso((int)nz, dz, Glso, ar, solve_tables))) { ar.release(); return rc; }
  std::vector<double2> h((size_t)nz * NN);
  cudaMemcpyAsync(h.data(), Glso, sizeof(double2) * h.size(), cudaMemcpyDeviceToHost, g->st);
  cudaError_t e = cudaStreamSynchronize(g->st);
  ar.release();
  if (e != cudaSuccess) VFAIL(VCA_ERR_CUDA, cudaGetErrorString(e));
  // lso -> (Nlat,Nlat,Nspin,Nspin,Norb,Norb,nz)
  const size_t nel = hloc_len(c);
  for (int64_t q = 0; q < nz; q++)
    for (int il = 0; il < c.Nlat; il++)
      for (int jl = 0; jl < c.Nlat; jl++)
        for (int is = 0; is < c.Nspin; is++)
          for (int js = 0; js < c.Nspin; js++)
            for (int io = 0; io < c.Norb; io++)
              for (int jo = 0; jo < c.Norb; jo++) {
                int a = io + il * c.Norb + is * c.Norb * c.Nlat, b = jo + jl * c.Norb + js * c.Norb * c.Nlat;
                double2 v = h[(size_t)q * NN + a + (size_t)b * N];
                size_t o = (size_t)q * nel + idx_nnn(c, il, jl, is, js, io, jo);
                gf_out[2 * o] = v.x;
                gf_out[2 * o + 1] = v.y;
              }
  return VCA_OK;
}

int vca_gpu_gf_cluster(const double* z, int64_t nz, double* gf_out) {
  if (!g || !(g->solved || g->gfm_loaded)) VFAIL(VCA_ERR_STATE, "no completed vca_gpu_solve");
  return gf_cluster_host(z, nz, gf_out, false);
}

// the Matsubara (wm = pi/beta*(2n-1), VCA_GF_SHARED.f90:50) or real-axis
// (wr = linspace(wini,wfin,Lreal) + i*eps, VCA_GF_NORMAL.f90:1029) grid
static std::vector<double> freq_grid(bool mats) {
  const vca_config& c = g->cfg;
  const int L = mats ? c.Lmats : c.Lreal;
  std::vector<double> z(2 * (size_t)L);
  for (int i = 0; i < L; i++) {
    if (mats) {
      z[2 * i] = 0.0;
      z[2 * i + 1] = M_PI / c.beta * (2.0 * (i + 1) - 1.0);
    } else {
      z[2 * i] = (L > 1) ? c.wini + (c.wfin - c.wini) * i / (double)(L - 1) : c.wini;
      z[2 * i + 1] = c.eps;
    }
  }
  return z;
}

static int gimp_grid(bool mats, double* g_out) {
  if (!g || !g->solved) VFAIL(VCA_ERR_STATE, "no completed vca_gpu_solve");
  if (!g_out) VFAIL(VCA_ERR_ARG, "NULL output");
  const std::vector<double> z = freq_grid(mats);
  return gf_cluster_host(z.data(), (int64_t)(z.size() / 2), g_out, true);
}

// Sigma (want_g0 = false) or G0 on the Matsubara or real-axis grid, as
// build_sigma_normal (VCA_GF_NORMAL.f90:1045-1111), out in
// (Nlat,Nlat,Nspin,Nspin,Norb,Norb,L) order
static int sigma_grid(bool mats, bool want_g0, double* out) {
  if (g && !want_g0 && g->sigma_loaded) {  // read by vca_read_impSigma
    if (!out) VFAIL(VCA_ERR_ARG, "NULL output");
    const std::vector<double>& v = mats ? g->sigma_mats : g->sigma_real;
    std::copy(v.begin(), v.end(), out);
    return VCA_OK;
  }
  if (!g || !g->solved) VFAIL(VCA_ERR_STATE, "no completed vca_gpu_solve");
  if (!out) VFAIL(VCA_ERR_ARG, "NULL output");
  const vca_config& c = g->cfg;
  const int N = g->N, NN = N * N;
  if (N > 32) VFAIL(VCA_ERR_UNSUPPORTED, "self-energy supports up to 32 spin-orbitals");
  const std::vector<double> zh = freq_grid(mats);
  const int n = (int)(zh.size() / 2);
  if (n == 0) return VCA_OK;
  Arena ar;
  int rc;
  double2 *dz, *Glso = nullptr, *P, *Hl, *res;
  if ((rc = ar.alloc(&dz, n)) || (rc = ar.alloc(&Hl, NN)) || (rc = ar.alloc(&res, (size_t)n * NN))) {
    ar.release();
    return rc;
  }
  cudaMemcpyAsync(dz, zh.data(), sizeof(double2) * n, cudaMemcpyHostToDevice, g->st);
  if (!want_g0) {
    if ((rc = ar.alloc(&Glso, (size_t)n * NN)) || (rc = gf_lso(n, dz, Glso, ar, true))) { ar.release(); return rc; }
  }
  {
    double2* hraw;
    if ((rc = ar.alloc(&hraw, NN))) { ar.release(); return rc; }
    cudaMemcpyAsync(hraw, g->Hloc.data(), sizeof(double2) * NN, cudaMemcpyHostToDevice, g->st);
    launch_nnn2lso(c.Nlat, c.Nspin, c.Norb, 1, hraw, Hl, g->st);
  }
  bool per_z = false;
  P = Hl;
  if (g->has_bath) {  // P = Delta(z) + Hloc
    std::vector<double2> hb, V;
    bath_lso(hb, V);
    double2 *dhb, *dV, *work, *D;
    const int Nb = g->Nb;
    if ((rc = ar.alloc(&dhb, (size_t)Nb * Nb)) || (rc = ar.alloc(&dV, (size_t)N * Nb)) ||
        (rc = ar.alloc(&work, (size_t)n * 2 * Nb * Nb)) || (rc = ar.alloc(&D, (size_t)n * NN)) ||
        (rc = ar.alloc(&P, (size_t)n * NN))) {
      ar.release();
      return rc;
    }
    cudaMemcpyAsync(dhb, hb.data(), sizeof(double2) * hb.size(), cudaMemcpyHostToDevice, g->st);
    cudaMemcpyAsync(dV, V.data(), sizeof(double2) * V.size(), cudaMemcpyHostToDevice, g->st);
    launch_delta_bath(n, dz, N, Nb, dhb, dV, c.xmu, work, D, g->st);
    launch_add_hloc(n, NN, D, Hl, P, g->st);
    per_z = true;
  }
  launch_sigma_g0(n, N, dz, Glso, P, per_z, c.xmu, want_g0, res, g->st);
  std::vector<double2> h((size_t)n * NN);
  cudaMemcpyAsync(h.data(), res, sizeof(double2) * h.size(), cudaMemcpyDeviceToHost, g->st);
  cudaError_t e = cudaStreamSynchronize(g->st);
  ar.release();
  if (e != cudaSuccess) VFAIL(VCA_ERR_CUDA, cudaGetErrorString(e));
  const size_t nel = hloc_len(c);
  for (int q = 0; q < n; q++)
    for (int il = 0; il < c.Nlat; il++)
      for (int jl = 0; jl < c.Nlat; jl++)
        for (int is = 0; is < c.Nspin; is++)
          for (int js = 0; js < c.Nspin; js++)
            for (int io = 0; io < c.Norb; io++)
              for (int jo = 0; jo < c.Norb; jo++) {
                const int a = io + il * c.Norb + is * c.Norb * c.Nlat, b = jo + jl * c.Norb + js * c.Norb * c.Nlat;
                const double2 v = h[(size_t)q * NN + a + (size_t)b * N];
                const size_t o = (size_t)q * nel + idx_nnn(c, il, jl, is, js, io, jo);
                out[2 * o] = v.x;
                out[2 * o + 1] = v.y;
              }
  return VCA_OK;
}
int vca_gpu_get_gimp_matsubara(double* g_out) { return gimp_grid(true, g_out); }
int vca_gpu_get_gimp_realaxis(double* g_out) { return gimp_grid(false, g_out); }
// Ground-state observables (vca_lanc_observables, VCA_OBSERVABLES.f90:
// 185-316, T = 0: weight 1/zeta per kept state): which = 0 dens, 1 dens_up,
// 2 dens_dw, 3 docc, 4 mag = dens_up - dens_dw (VCA_IO/get_mag.f90), out in
// (Nlat,Norb) order
static int observable(int which, double* out) {
  if (!g || !g->solved) VFAIL(VCA_ERR_STATE, "no completed vca_gpu_solve");
  if (!out) VFAIL(VCA_ERR_ARG, "NULL output");
  const vca_config& c = g->cfg;
  const int nimp = c.Nlat * c.Norb;
  std::vector<double> up(nimp, 0.0), dw(nimp, 0.0), dd(nimp, 0.0);
  for (const GState& st : g->gs) {
    const SectorView sv = view_of(sec_nup(st.sector), sec_ndw(st.sector));
    const int nb = observables_blocks((int64_t)sv.dimup * sv.dimdw);
    Arena ar;
    double* part;
    RCHK(ar.alloc(&part, (size_t)3 * nimp * nb));
    const int fmt = g->fx ? 0 : (g->real_model ? 1 : 2);
    launch_observables(sv, fmt, st.vec, g->fxs.F, nimp, part, g->st);
    std::vector<double> h((size_t)3 * nimp * nb);
    cudaMemcpyAsync(h.data(), part, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, g->st);
    cudaError_t e = cudaStreamSynchronize(g->st);
    ar.release();
    if (e != cudaSuccess) VFAIL(VCA_ERR_CUDA, cudaGetErrorString(e));
    for (int l = 0; l < nimp; l++) {
      double a = 0.0, b = 0.0, d = 0.0;
      for (int x = 0; x < nb; x++) {
        a += h[((size_t)0 * nimp + l) * nb + x];
        b += h[((size_t)1 * nimp + l) * nb + x];
        d += h[((size_t)2 * nimp + l) * nb + x];
      }
      // peso = exp(-beta(Ei-Egs))/zeta at finite T (VCA_OBSERVABLES.f90:248-249)
      const double peso = (g->finiteT ? std::exp(-c.beta * (st.e - g->egs)) : 1.0) / g->zeta;
      up[l] += peso * a;
      dw[l] += peso * b;
      dd[l] += peso * d;
    }
  }
  for (int il = 0; il < c.Nlat; il++)
    for (int io = 0; io < c.Norb; io++) {
      const int l = io + il * c.Norb;  // imp_state_index (VCA_SETUP.f90:705-710)
      const double v[5] = {up[l] + dw[l], up[l], dw[l], dd[l], up[l] - dw[l]};
      out[il + io * c.Nlat] = v[which];
    }
  return VCA_OK;
}
int vca_gpu_get_dens(double* out) { return observable(0, out); }
int vca_gpu_get_dens_up(double* out) { return observable(1, out); }
int vca_gpu_get_dens_dw(double* out) { return observable(2, out); }
int vca_gpu_get_docc(double* out) { return observable(3, out); }
int vca_gpu_get_mag(double* out) { return observable(4, out); }

// ---- splot files (vca_print_impSigma / vca_print_impG / vca_print_impG0,
// VCA_IO.f90:112-205) -------------------------------------------------------
static std::string cfg_suffix() {
  const vca_config& c = g->cfg;
  return std::string(c.file_suffix, strnlen(c.file_suffix, sizeof c.file_suffix));
}

// one file per spin-diagonal element and grid:
// <name>_Isite<ilat:4>_Jsite<jlat:4>_l<iorb><jorb>_s<ispin>_<iw|realw><file_suffix>.vca
// (the suffix built at VCA_IO.f90:125-128), written as SciFortran's splot
// writes a complex function: one line per point, x, Im y, Re y; 17
// significant digits, so the text reads back bit-exact
static int print_function(int kind /* 0 G', 1 Sigma, 2 G0 */) {
  static const char* names[3] = {"impG", "impSigma", "impG0"};
  const vca_config& c = g->cfg;
  const std::string sfx = cfg_suffix();
  const size_t nel = hloc_len(c);
  for (int m = 0; m < 2; m++) {
    const bool mats = (m == 0);
    const int L = mats ? c.Lmats : c.Lreal;
    if (L <= 0) continue;
    std::vector<double> y(2 * nel * (size_t)L);
    RCHK(kind == 0 ? gimp_grid(mats, y.data()) : sigma_grid(mats, kind == 2, y.data()));
    const std::vector<double> z = freq_grid(mats);
    for (int il = 0; il < c.Nlat; il++)
      for (int jl = 0; jl < c.Nlat; jl++)
        for (int io = 0; io < c.Norb; io++)
          for (int jo = 0; jo < c.Norb; jo++)
            for (int is = 0; is < c.Nspin; is++) {
              char tag[96];
              std::snprintf(tag, sizeof tag, "_Isite%04d_Jsite%04d_l%d%d_s%d_%s", il + 1, jl + 1, io + 1, jo + 1,
                            is + 1, mats ? "iw" : "realw");
              const std::string path = std::string(names[kind]) + tag + sfx + ".vca";
              std::FILE* f = std::fopen(path.c_str(), "w");
              if (!f) VFAIL(VCA_ERR_IO, "cannot open " + path + ": " + std::strerror(errno));
              const int64_t off = idx_nnn(c, il, jl, is, is, io, jo);
              bool bad = false;
              for (int q = 0; q < L && !bad; q++) {
                const double x = mats ? z[2 * q + 1] : z[2 * q];
                const double* v = y.data() + 2 * ((size_t)q * nel + off);
                bad = std::fprintf(f, "%24.16E %24.16E %24.16E\n", x, v[1], v[0]) < 0;
              }
              if (std::fclose(f) != 0 || bad) VFAIL(VCA_ERR_IO, "write error on " + path);
            }
  }
  return VCA_OK;
}

// PRINT_SIGMA / PRINT_IMPG / PRINT_IMPG0 at the end of a solve, in the
// reference's order (VCA_GREENS_FUNCTIONS.f90:37-41)
static int print_after_solve() {
  const vca_config& c = g->cfg;
  if (c.print_sigma) RCHK(print_function(1));
  if (c.print_impg) RCHK(print_function(0));
  if (c.print_impg0) RCHK(print_function(2));
  return VCA_OK;
}

int vca_gpu_print_impSigma(void) {
  if (!g || !(g->solved || g->sigma_loaded)) VFAIL(VCA_ERR_STATE, "no completed vca_gpu_solve");
  return print_function(1);
}
int vca_gpu_print_impG(void) {
  if (!g || !g->solved) VFAIL(VCA_ERR_STATE, "no completed vca_gpu_solve");
  return print_function(0);
}
int vca_gpu_print_impG0(void) {
  if (!g || !g->solved) VFAIL(VCA_ERR_STATE, "no completed vca_gpu_solve");
  return print_function(2);
}

// One splot file of a complex function: n lines of x, Im y, Re y (blank- or
// comma-separated, D or E exponents).  Host only.
static int splot_read(const std::string& path, int64_t n, double* x, double* y) {
  std::FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) VFAIL(VCA_ERR_IO, "cannot open " + path + ": " + std::strerror(errno));
  std::string text;
  char buf[1 << 16];
  size_t got;
  while ((got = std::fread(buf, 1, sizeof buf, f)) > 0) text.append(buf, got);
  std::fclose(f);
  for (char& ch : text)
    if (ch == 'd' || ch == 'D') ch = 'e';
    else if (ch == ',') ch = ' ';
  const char* p = text.c_str();
  for (int64_t i = 0; i < n; i++) {
    double v[3];
    for (int k = 0; k < 3; k++) {
      char* end = nullptr;
      v[k] = std::strtod(p, &end);
      if (end == p) VFAIL(VCA_ERR_IO, path + ": expected " + std::to_string(n) + " lines of x, Im, Re");
      p = end;
    }
    if (x) x[i] = v[0];
    y[2 * i] = v[2];
    y[2 * i + 1] = v[1];
  }
  return VCA_OK;
}

int vca_splot_read(const char* path, int64_t n, double* x, double* y) {
  if (!path || n < 0 || (n > 0 && !y)) VFAIL(VCA_ERR_ARG, "bad arguments");
  return splot_read(path, n, x, y);
}

int vca_read_impSigma(void) {
  if (!g || !g->basis.ptrs.size()) VFAIL(VCA_ERR_STATE, "vca_gpu_init has not been called");
  const vca_config& c = g->cfg;
  const std::string sfx = cfg_suffix();
  const size_t nel = hloc_len(c);
  std::vector<double> sm(2 * nel * (size_t)std::max(c.Lmats, 0), 0.0), sr(2 * nel * (size_t)std::max(c.Lreal, 0), 0.0);
  for (int m = 0; m < 2; m++) {
    const bool mats = (m == 0);
    const int L = mats ? c.Lmats : c.Lreal;
    if (L <= 0) continue;
    std::vector<double>& dst = mats ? sm : sr;
    std::vector<double> y(2 * (size_t)L);
    for (int is = 0; is < c.Nspin; is++)
      for (int il = 0; il < c.Nlat; il++)
        for (int jl = 0; jl < c.Nlat; jl++)
          for (int io = 0; io < c.Norb; io++)
            for (int jo = 0; jo < c.Norb; jo++) {
              char tag[96];
              std::snprintf(tag, sizeof tag, "_Isite%04d_Jsite%04d_l%d%d_s%d_%s", il + 1, jl + 1, io + 1, jo + 1,
                            is + 1, mats ? "iw" : "realw");
              RCHK(splot_read(std::string("impSigma") + tag + sfx + ".vca", L, nullptr, y.data()));
              const int64_t off = idx_nnn(c, il, jl, is, is, io, jo);
              for (int q = 0; q < L; q++) {
                dst[2 * ((size_t)q * nel + off)] = y[2 * q];
                dst[2 * ((size_t)q * nel + off) + 1] = y[2 * q + 1];
              }
            }
  }
  g->sigma_mats.swap(sm);
  g->sigma_real.swap(sr);
  g->sigma_loaded = true;
  return VCA_OK;
}

int vca_gpu_get_sigma_matsubara(double* s_out) { return sigma_grid(true, false, s_out); }
int vca_gpu_get_sigma_realaxis(double* s_out) { return sigma_grid(false, false, s_out); }
int vca_gpu_get_g0_matsubara(double* g0_out) { return sigma_grid(true, true, g0_out); }
int vca_gpu_get_g0_realaxis(double* g0_out) { return sigma_grid(false, true, g0_out); }

int vca_gpu_sum_kmesh(const double* w, int64_t nw, double* f_out) {
  if (!g || !g->solved) VFAIL(VCA_ERR_STATE, "no completed vca_gpu_solve");
  if (!w || !f_out || nw < 1) VFAIL(VCA_ERR_ARG, "bad arguments");
  std::vector<double2> z(nw);
  for (int64_t i = 0; i < nw; i++) z[i] = make_double2(0.0, w[i]);
  return ksum_host((int)nw, z.data(), f_out, nullptr);
}

int vca_gpu_sum_kmesh_complex(const double* z, int64_t nz, double* f_out) {
  if (!g || !g->solved) VFAIL(VCA_ERR_STATE, "no completed vca_gpu_solve");
  if (!z || !f_out || nz < 1 || nz > (1 << 24)) VFAIL(VCA_ERR_ARG, "bad arguments");
  std::vector<double2> zh(nz);
  for (int64_t i = 0; i < nz; i++) zh[i] = make_double2(z[2 * i], z[2 * i + 1]);
  std::vector<double> re(nz), im(nz);
  RCHK(ksum_host((int)nz, zh.data(), re.data(), im.data()));
  for (int64_t i = 0; i < nz; i++) { f_out[2 * i] = re[i]; f_out[2 * i + 1] = im[i]; }
  return VCA_OK;
}

int vca_gpu_custom_observable(const double* s, int32_t kdep, double* value) {
  if (!g || !g->solved) VFAIL(VCA_ERR_STATE, "no completed vca_gpu_solve");
  if (!s || !value) VFAIL(VCA_ERR_ARG, "NULL argument");
  RCHK(check_finite(s, 2 * (size_t)g->N * g->N * (kdep ? (size_t)g->Nk : 1), "s"));
  return custom_observable(s, kdep != 0, value);
}

int vca_gpu_get_thermal(vca_thermal* out) {
  if (!g || !g->solved) VFAIL(VCA_ERR_STATE, "no completed vca_gpu_solve");
  if (!out) VFAIL(VCA_ERR_ARG, "NULL output");
  std::memset(out, 0, sizeof(*out));
  out->zeta = g->zeta;
  out->omega_prime = g->omega_prime;
  out->e_min = g->egs;
  out->nstates_total = g->nstates_total;
  out->finite_t = g->finiteT ? 1 : 0;
  if (g->finiteT) {
    out->max_exc = g->max_exc;
    out->integration_R = g->int_R;
    out->sum_part = g->sum_part;
    out->contour_part = g->contour_part;
    out->nmax = g->nmax;
    out->contour_points = g->contour_points;
  }
  return VCA_OK;
}

int vca_gpu_sector_info(int32_t isector, int32_t* nup, int32_t* ndw, int64_t* dimup, int64_t* dimdw) {
  if (!g) VFAIL(VCA_ERR_STATE, "vca_gpu_init has not been called");
  if (isector < 1 || isector > g->Nsectors) VFAIL(VCA_ERR_ARG, "sector out of range");
  const int u = sec_nup(isector), d = sec_ndw(isector);
  if (nup) *nup = u;
  if (ndw) *ndw = d;
  if (dimup) *dimup = g->dimn[u];
  if (dimdw) *dimdw = g->dimn[d];
  return VCA_OK;
}

int vca_gpu_sector_map(int32_t isector, int32_t spin, int64_t* map, int64_t cap) {
  if (!g) VFAIL(VCA_ERR_STATE, "vca_gpu_init has not been called");
  if (isector < 1 || isector > g->Nsectors || (spin != 1 && spin != 2)) VFAIL(VCA_ERR_ARG, "bad sector/spin");
  const int n = (spin == 1) ? sec_nup(isector) : sec_ndw(isector);
  const int dim = g->dimn[n];
  if (!map || cap < dim) VFAIL(VCA_ERR_ARG, "map buffer too small");
  std::vector<int> w(dim);
  CUCHK(cudaMemcpy(w.data(), g->words[n], sizeof(int) * dim, cudaMemcpyDeviceToHost));
  for (int i = 0; i < dim; i++) map[i] = w[i];
  return VCA_OK;
}

// Fixed-point view for the public column entry points: with hxv_variant 2
// the caller's rows of the up role are in hop-count order (the layout of the
// chain batches, vca_gpu_sector_row_order) and the position-ordered kernel
// runs.
static int api_fx_view(int nup, int ndw, int m, FxView* out) {
  FxView f = fx_view_of(nup, ndw);
  if (g->cfg.hxv_variant == 2) {
    if (!hxv_fx_r_ok(view_of(nup, ndw), f, m))
      VFAIL(VCA_ERR_UNSUPPORTED,
            "hxv_variant 2 needs >= 16 columns, at most 2 hopping classes and an up block that fits shared memory");
    f.rows_permuted = 1;
  }
  *out = f;
  return VCA_OK;
}

// apart: optional alpha-partial scratch of the fixed-point column kernels
// (hxv_fx_cols_rows rows of m int128), as the Lanczos chain steps pass it
static int hxv_cols(int32_t isector, const void* d_v, void* d_hv, int32_t is_complex, int32_t ncols,
                    i64* apart = nullptr) {
  if (!g || !g->ham_set) VFAIL(VCA_ERR_STATE, "no Hamiltonian loaded (vca_gpu_set_hamiltonian)");
  if (isector < 1 || isector > g->Nsectors) VFAIL(VCA_ERR_ARG, "sector out of range");
  if (ncols < 1) VFAIL(VCA_ERR_ARG, "ncols must be >= 1");
  if (!is_complex && !g->real_model) VFAIL(VCA_ERR_ARG, "real vectors need a real Hamiltonian");
  const int nup = sec_nup(isector), ndw = sec_ndw(isector);
  SectorView sv = view_of(nup, ndw);
  const int m = (is_complex && g->real_model) ? 2 * ncols : ncols;
  if ((((uintptr_t)d_v) | ((uintptr_t)d_hv)) & 15u) VFAIL(VCA_ERR_ARG, "device vectors must be 16-byte aligned");
  if (g->fx) {  // slab-major fixed-point columns (scale 2^-F, unit norm)
    if (m >= FX_SLAB && m % FX_SLAB)
      VFAIL(VCA_ERR_ARG, "fixed-point column batches of 8 or more columns need a multiple of 8 columns");
    if (m >= 16) {
      FxView fv;
      RCHK(api_fx_view(nup, ndw, m, &fv));
      launch_hxv_fx_cols(sv, fv, m, (const i64*)d_v, (i64*)d_hv, apart, g->cfg.hxv_variant == 1, g->st);
    } else if (g->cfg.hxv_variant == 2) {
      VFAIL(VCA_ERR_UNSUPPORTED, "hxv_variant 2 needs >= 16 columns");
    } else
      launch_hxv_fx(sv, fx_view_of(nup, ndw), m, (const i64*)d_v, (i64*)d_hv, g->st);
  } else if (is_complex && !g->real_model) {
    launch_hxv_cplx(sv, g->md, ncols, (const double2*)d_v, (double2*)d_hv, g->st);
  } else {
    launch_hxv_real(sv, g->md, m, (const double*)d_v, (double*)d_hv, g->st);
  }
  CUCHK(cudaGetLastError());
  return VCA_OK;
}

int vca_gpu_hxv_device(int32_t isector, const void* d_v, void* d_hv, int32_t is_complex) {
  return hxv_cols(isector, d_v, d_hv, is_complex, 1);
}

int vca_gpu_hxv(int32_t isector, const double* v, double* hv) {
  if (!g || !g->ham_set) VFAIL(VCA_ERR_STATE, "no Hamiltonian loaded (vca_gpu_set_hamiltonian)");
  if (isector < 1 || isector > g->Nsectors) VFAIL(VCA_ERR_ARG, "sector out of range");
  if (!v || !hv) VFAIL(VCA_ERR_ARG, "NULL vector");
  const int64_t D = (int64_t)g->dimn[sec_nup(isector)] * g->dimn[sec_ndw(isector)];
  Arena ar;
  double2 *dv, *dh;
  int rc;
  if ((rc = ar.alloc(&dv, D)) || (rc = ar.alloc(&dh, D))) { ar.release(); return rc; }
  if (g->fx) {
    // fixed point holds unit-norm vectors: scale by 1/||v||, convert, apply, undo
    double nrm = 0.0;
    for (int64_t i = 0; i < 2 * D; i++) nrm += v[i] * v[i];
    nrm = std::sqrt(nrm);
    if (nrm == 0.0) { ar.release(); std::memset(hv, 0, sizeof(double) * 2 * D); return VCA_OK; }
    std::vector<double> vs(2 * D);
    for (int64_t i = 0; i < 2 * D; i++) vs[i] = v[i] / nrm;
    cudaMemcpyAsync(dv, vs.data(), sizeof(double2) * D, cudaMemcpyHostToDevice, g->st);
    launch_fx_from_double(2 * D, (const double*)dv, g->fxs.F, (i64*)dh, g->st);
    rc = hxv_cols(isector, dh, dv, 1, 1);
    if (rc) { ar.release(); return rc; }
    launch_fx_to_double(2 * D, (const i64*)dv, g->fxs.G, (double*)dh, g->st);
    cudaMemcpyAsync(hv, dh, sizeof(double2) * D, cudaMemcpyDeviceToHost, g->st);
    cudaError_t e = cudaStreamSynchronize(g->st);
    ar.release();
    if (e != cudaSuccess) VFAIL(VCA_ERR_CUDA, cudaGetErrorString(e));
    for (int64_t i = 0; i < 2 * D; i++) hv[i] *= nrm;
    return VCA_OK;
  }
  cudaMemcpyAsync(dv, v, sizeof(double2) * D, cudaMemcpyHostToDevice, g->st);
  rc = vca_gpu_hxv_device(isector, dv, dh, 1);
  if (rc) { ar.release(); return rc; }
  cudaMemcpyAsync(hv, dh, sizeof(double2) * D, cudaMemcpyDeviceToHost, g->st);
  cudaError_t e = cudaStreamSynchronize(g->st);
  ar.release();
  if (e != cudaSuccess) VFAIL(VCA_ERR_CUDA, cudaGetErrorString(e));
  return VCA_OK;
}

int vca_gpu_hxv_timed(int32_t isector, const void* d_v, void* d_hv, int32_t is_complex, int32_t ncols,
                      int32_t reps, double* ms_per_call) {
  if (!g || !g->ham_set) VFAIL(VCA_ERR_STATE, "no Hamiltonian loaded (vca_gpu_set_hamiltonian)");
  if (reps < 1 || !ms_per_call) VFAIL(VCA_ERR_ARG, "bad arguments");
  cudaEvent_t e0, e1;
  Arena ar;
  if (isector < 1 || isector > g->Nsectors) VFAIL(VCA_ERR_ARG, "sector out of range");
  i64* apart = nullptr;
  const int mm = (is_complex && g->real_model) ? 2 * ncols : ncols;
  if (g->fx && mm >= 16) {  // the alpha partials the chain steps form with the product
    const int nup = sec_nup(isector), ndw = sec_ndw(isector);
    FxView fv;
    RCHK(api_fx_view(nup, ndw, mm, &fv));
    const int rows = hxv_fx_cols_rows(view_of(nup, ndw), fv, mm, g->cfg.hxv_variant == 1);
    RCHK(ar.alloc(&apart, 2 * (size_t)rows * mm));
  }
  CUCHK(cudaEventCreate(&e0));
  CUCHK(cudaEventCreate(&e1));
  RCHK(hxv_cols(isector, d_v, d_hv, is_complex, ncols, apart));  // warm-up
  CUCHK(cudaEventRecord(e0, g->st));
  for (int r = 0; r < reps; r++) RCHK(hxv_cols(isector, d_v, d_hv, is_complex, ncols, apart));
  CUCHK(cudaEventRecord(e1, g->st));
  CUCHK(cudaEventSynchronize(e1));
  float ms = 0.f;
  CUCHK(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  CUCHK(cudaStreamSynchronize(g->st));
  ar.release();
  if (g->fx && fx_take_wait_failures() != 0)
    VFAIL(VCA_ERR_TIMEOUT, "a bounded wait for a bulk copy in the column H x v ran out");
  *ms_per_call = ms / reps;
  return VCA_OK;
}

int vca_gpu_set_stage_extra_tx(int32_t bytes) {
  if (!g) VFAIL(VCA_ERR_STATE, "vca_gpu_init has not been called");
  if (bytes < 0 || bytes > (1 << 16) || bytes % 16) VFAIL(VCA_ERR_ARG, "0..65536 bytes, a multiple of 16");
  if (fx_set_stage_extra_tx(bytes) != 0) VFAIL(VCA_ERR_CUDA, "cannot set the test hook");
  return VCA_OK;
}

int vca_gpu_upload_hk(const double* Hk, int64_t Nk) {
  if (!g) VFAIL(VCA_ERR_STATE, "vca_gpu_init has not been called");
  return upload_hk(Hk, Nk);
}

int vca_gpu_solve_resident(const double* Hloc, const double* bath_h, const double* bath_v,
                           double* omega_out) {
  g_err.clear();
  RCHK(solve_resident(Hloc, bath_h, bath_v, omega_out));
  return print_after_solve();
}

int64_t vca_gpu_kernel_launches(void) { return (int64_t)launch_count(); }

int vca_gpu_sector_pairs(int32_t isector, int32_t k, double* energies, double* vecs, int32_t* n) {
  if (!g || !g->ham_set) VFAIL(VCA_ERR_STATE, "no Hamiltonian loaded (vca_gpu_set_hamiltonian)");
  if (isector < 1 || isector > g->Nsectors) VFAIL(VCA_ERR_ARG, "sector out of range");
  if (k < 1 || !energies || !n) VFAIL(VCA_ERR_ARG, "bad arguments");
  std::vector<double> e;
  std::vector<void*> v;
  Arena keep;
  int rc = sector_pairs(isector, k, e, v, keep, true);
  if (rc) { keep.release(); return rc; }
  const int64_t D = (int64_t)g->dimn[sec_nup(isector)] * g->dimn[sec_ndw(isector)];
  *n = (int32_t)e.size();
  for (size_t j = 0; j < e.size(); j++) {
    energies[j] = e[j];
    if (!vecs) continue;
    std::vector<double> h((size_t)D * (g->real_model ? 1 : 2));
    cudaMemcpy(h.data(), v[j], h.size() * sizeof(double), cudaMemcpyDeviceToHost);
    for (int64_t i = 0; i < D; i++) {
      vecs[2 * (j * D + i)] = g->real_model ? h[i] : h[2 * i];
      vecs[2 * (j * D + i) + 1] = g->real_model ? 0.0 : h[2 * i + 1];
    }
  }
  keep.release();
  CUCHK(cudaGetLastError());
  return VCA_OK;
}

int vca_gpu_get_timings(double* ms, int32_t n) {
  if (!g) VFAIL(VCA_ERR_STATE, "vca_gpu_init has not been called");
  if (!ms) VFAIL(VCA_ERR_ARG, "NULL output");
  for (int i = 0; i < n && i < 4; i++) ms[i] = g->t_ms[i];
  for (int i = 4; i < n && i < 10; i++) ms[i] = g->bt_ms[i - 4];
  if (n > 10) ms[10] = (double)g->bt_skipped;
  if (n > 12) { ms[11] = g->bt_shape[0]; ms[12] = g->bt_shape[1]; }
  for (int i = 13; i < n && i < 16; i++) ms[i] = g->chain_ms[i - 13];
  return VCA_OK;
}

static cudaEvent_t g_t0 = nullptr, g_t1 = nullptr;
int vca_gpu_timer_start(void) {
  if (!g) VFAIL(VCA_ERR_STATE, "vca_gpu_init has not been called");
  if (!g_t0) { CUCHK(cudaEventCreate(&g_t0)); CUCHK(cudaEventCreate(&g_t1)); }
  CUCHK(cudaEventRecord(g_t0, g->st));
  return VCA_OK;
}
int vca_gpu_timer_stop(double* ms) {
  if (!g || !g_t0) VFAIL(VCA_ERR_STATE, "vca_gpu_timer_start has not been called");
  CUCHK(cudaEventRecord(g_t1, g->st));
  CUCHK(cudaEventSynchronize(g_t1));
  float f = 0.f;
  CUCHK(cudaEventElapsedTime(&f, g_t0, g_t1));
  if (ms) *ms = f;
  return VCA_OK;
}

int vca_gpu_sector_row_order(int32_t isector, int64_t* order, int64_t cap) {
  if (!g || !g->ham_set) VFAIL(VCA_ERR_STATE, "no Hamiltonian loaded");
  if (isector < 1 || isector > g->Nsectors) VFAIL(VCA_ERR_ARG, "sector out of range");
  if (!g->fx) VFAIL(VCA_ERR_UNSUPPORTED, "row orders exist in the fixed-point path only");
  const int nup = sec_nup(isector), ndw = sec_ndw(isector);
  const int64_t du = g->dimn[nup], dd = g->dimn[ndw];
  if (!order || cap < du * dd) VFAIL(VCA_ERR_ARG, "order buffer too small");
  std::vector<int> perm(du);
  CUCHK(cudaMemcpy(perm.data(), g->fx_perm[0][nup], sizeof(int) * du, cudaMemcpyDeviceToHost));
  for (int64_t b = 0; b < dd; b++)
    for (int64_t p = 0; p < du; p++) order[p + b * du] = perm[p] + b * du;
  return VCA_OK;
}

int vca_gpu_arith_info(int32_t* fx, int32_t* F, int32_t* G) {
  if (!g || !g->ham_set) VFAIL(VCA_ERR_STATE, "no Hamiltonian loaded");
  if (fx) *fx = g->fx ? 1 : 0;
  if (F) *F = g->fxs.F;
  if (G) *G = g->fxs.G;
  return VCA_OK;
}

int vca_gpu_synchronize(void) {
  if (!g) VFAIL(VCA_ERR_STATE, "vca_gpu_init has not been called");
  CUCHK(cudaStreamSynchronize(g->st));
  return VCA_OK;
}

int vca_hop_schedule(int32_t dim, int32_t width, int32_t K, const int32_t* cnt, const uint32_t* hop, uint32_t* sched,
                     int64_t sched_cap, int32_t* wround, int32_t* wgrp, int64_t* nrounds, int64_t* conflicts) {
  if (dim < 1 || width < 0 || K < 1 || K > VCA_FX_KMAX || !cnt || (width > 0 && !hop) || !wround || !wgrp ||
      !nrounds || sched_cap < 0 || (sched_cap > 0 && !sched))
    return set_error(VCA_ERR_ARG, "bad arguments");
  std::vector<unsigned> sc;
  std::vector<int> wr, wg;
  const int64_t nc = fx_pair_schedule(dim, width, K, cnt, hop, sc, wr, wg);
  if (nc < 0) return set_error(VCA_ERR_NUMERIC, "a hop was left unplaced");
  *nrounds = wr.back();
  if (conflicts) *conflicts = nc;
  std::memcpy(wround, wr.data(), sizeof(int) * wr.size());
  std::memcpy(wgrp, wg.data(), sizeof(int) * wg.size());
  std::memcpy(sched, sc.data(), sizeof(unsigned) * std::min<size_t>(sc.size(), (size_t)sched_cap));
  return VCA_OK;
}

int vca_hop_parity_order(int32_t dim, int32_t width, const int32_t* cnt, const int32_t* npos, uint32_t* rhop) {
  if (dim < 1 || width < 0 || !cnt || !npos || (width > 0 && !rhop)) return set_error(VCA_ERR_ARG, "bad arguments");
  fx_rhop_parity_order(dim, width, cnt, npos, rhop);
  return VCA_OK;
}

int vca_gpu_set_chain_streams(int32_t n) {
  if (!g) VFAIL(VCA_ERR_STATE, "vca_gpu_init has not been called");
  if (n < 1 || n > 2) VFAIL(VCA_ERR_ARG, "1 or 2 chain streams");
  g->chain_streams = n;
  return VCA_OK;
}

int vca_gpu_set_hop_pairing(int32_t on) {
  if (!g) VFAIL(VCA_ERR_STATE, "vca_gpu_init has not been called");
  g->rhop_order = on != 0;  // takes effect when the next Hamiltonian's tables are built
  return VCA_OK;
}

int vca_gpu_set_autotune(int32_t on) {
  if (!g) VFAIL(VCA_ERR_STATE, "vca_gpu_init has not been called");
  g->autotune = on != 0;
  return VCA_OK;
}

int vca_gpu_set_omega_inverse_form(int32_t on) {
  if (!g) VFAIL(VCA_ERR_STATE, "vca_gpu_init has not been called");
  g->omega_inverse_form = on != 0;
  return VCA_OK;
}

int vca_gpu_sector_bounds(double* out, int32_t n) {
  if (!g || !g->ham_set) VFAIL(VCA_ERR_STATE, "no Hamiltonian loaded (vca_gpu_set_hamiltonian or a solve)");
  if (!out || n < g->Nsectors) VFAIL(VCA_ERR_ARG, "output too small");
  const std::vector<double> b = sector_lower_bounds();
  if (b.empty()) VFAIL(VCA_ERR_UNSUPPORTED, "no bound: an interaction coefficient is negative");
  for (int i = 0; i < g->Nsectors; i++) out[i] = b[i];
  return VCA_OK;
}

int vca_gpu_set_ql_max_iter(int32_t max_iter) {
  if (!g) VFAIL(VCA_ERR_STATE, "vca_gpu_init has not been called");
  if (max_iter < 1) VFAIL(VCA_ERR_ARG, "max_iter must be >= 1");
  g->ql_max_iter = max_iter;
  g->poles_ready = false;  // the next pole request reruns the QL under the new cap
  return VCA_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free column H x v with the per-column Rayleigh numerator.
//
// Some callers cannot call cudaMalloc while they run: a host code whose
// device memory belongs to its own pool allocator sized at start-up, or a
// sweep loop that must not reach the driver's allocator mid-run (cudaMalloc
// can stall the device and can fail when memory is tight).  For them,
// vca_gpu_hxv_alpha_noalloc does the column H x v of vca_gpu_hxv_timed and
// also forms alpha[c] = <x_c, H x_c>, keeping its partial sums in the
// file-scope device array below instead of allocated scratch.
//
// The array's device address is looked up once per device, by the first call
// made while that device is current; make that first call before any stream
// capture.  The address is cached only as long as the CUDA context: a
// vca_gpu_finalize forgets it, so a caller that resets the device (or makes a
// new primary context) must finalize and init again before the next call.
// Every call on a device shares the array and the array keeps the last call's
// contents: each partial is overwritten before it is read, so nothing needs
// clearing, but calls whose work overlaps on the GPU race.
// ---------------------------------------------------------------------------
#define VCA_NOALLOC_SCRATCH_BYTES (8u << 20)
#define VCA_NOALLOC_MAX_DEVICES 64
static __device__ __align__(256) unsigned char g_noalloc_scratch[VCA_NOALLOC_SCRATCH_BYTES];
static void* g_noalloc_addr[VCA_NOALLOC_MAX_DEVICES];
static std::mutex g_noalloc_mu;

static void noalloc_forget() {
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  for (auto& a : g_noalloc_addr) a = nullptr;
}

static int noalloc_scratch(void** out) {
  int dev = 0;
  CUCHK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= VCA_NOALLOC_MAX_DEVICES) VFAIL(VCA_ERR_CUDA, "device ordinal beyond the scratch table");
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_addr[dev]) {
    void* p = nullptr;
    CUCHK(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    g_noalloc_addr[dev] = p;
  }
  *out = g_noalloc_addr[dev];
  return VCA_OK;
}

extern "C" int vca_gpu_hxv_alpha_noalloc(int32_t isector, const void* d_v, void* d_hv, int32_t ncols,
                                         double* d_alpha) {
  if (!g || !g->ham_set) VFAIL(VCA_ERR_STATE, "no Hamiltonian loaded (vca_gpu_set_hamiltonian)");
  if (isector < 1 || isector > g->Nsectors) VFAIL(VCA_ERR_ARG, "sector out of range");
  if (ncols < 1 || !d_v || !d_hv || !d_alpha) VFAIL(VCA_ERR_ARG, "bad arguments");
  if ((((uintptr_t)d_v) | ((uintptr_t)d_hv)) & 15u) VFAIL(VCA_ERR_ARG, "device vectors must be 16-byte aligned");
  if (!g->real_model) VFAIL(VCA_ERR_UNSUPPORTED, "real columns need a real Hamiltonian");
  const int nup = sec_nup(isector), ndw = sec_ndw(isector);
  const SectorView sv = view_of(nup, ndw);
  const int64_t D = (int64_t)sv.dimup * sv.dimdw;
  const int m = ncols;
  const bool warp_only = g->cfg.hxv_variant == 1;
  // partial rows of the reduction behind alpha, as the Lanczos steps size them
  const int nblk = (int)std::min<int64_t>(std::max<int64_t>(1, D / 256), 608);
  int rows = nblk;
  size_t need;
  if (g->fx) {
    if (m >= FX_SLAB && m % FX_SLAB)
      VFAIL(VCA_ERR_ARG, "fixed-point column batches of 8 or more columns need a multiple of 8 columns");
    if (m >= 16) {
      FxView fv;
      RCHK(api_fx_view(nup, ndw, m, &fv));
      rows = hxv_fx_cols_rows(sv, fv, m, warp_only);
    } else if (g->cfg.hxv_variant == 2) {
      VFAIL(VCA_ERR_UNSUPPORTED, "hxv_variant 2 needs >= 16 columns");
    }
    need = (size_t)rows * m * 2 * sizeof(i64);
  } else {
    need = (size_t)rows * m * sizeof(double);
  }
  if (need > VCA_NOALLOC_SCRATCH_BYTES)
    VFAIL(VCA_ERR_ARG, "this batch needs " + std::to_string(need) +
                           " bytes of partial sums; the static scratch holds " +
                           std::to_string((size_t)VCA_NOALLOC_SCRATCH_BYTES) + " (use fewer columns)");
  void* scr = nullptr;
  RCHK(noalloc_scratch(&scr));
  const ColBatch cb{D, m, false, 0, nullptr, nullptr};
  if (g->fx) {
    FxView fv = fx_view_of(nup, ndw);
    if (m >= 16) RCHK(api_fx_view(nup, ndw, m, &fv));
    const int sexp = g->fxs.F + g->fxs.G;
    if (m >= 16) {
      launch_hxv_fx_cols(sv, fv, m, (const i64*)d_v, (i64*)d_hv, (i64*)scr, warp_only, g->st);
      launch_fx_partial_reduce(m, rows, (const i64*)scr, sexp, d_alpha, g->st);
    } else {
      launch_hxv_fx(sv, fv, m, (const i64*)d_v, (i64*)d_hv, g->st);
      launch_fx_dot(cb, (const i64*)d_v, (const i64*)d_hv, g->fxs.F, g->fxs.G, (i64*)scr, rows, d_alpha, g->st);
    }
  } else {
    launch_hxv_real(sv, g->md, m, (const double*)d_v, (double*)d_hv, g->st);
    launch_col_dot(cb, d_v, d_hv, (double*)scr, rows, d_alpha, g->st);
  }
  CUCHK(cudaGetLastError());
  return VCA_OK;
}

int vca::set_error(int code, const std::string& msg) {
  g_err = msg;
  return code;
}
