// vca_fx.cuh -- exact 64-bit fixed-point ("FX") Lanczos arithmetic for real
// Hamiltonians.
//
// GB300 issues FP64 at ~0.5 T instructions/s but 64-bit integer adds ~50x
// faster, so the real-Hamiltonian path keeps every Lanczos vector as int64
// fixed point and does all per-element arithmetic on the integer pipes:
//   * vectors v (norm 1):           V = round(v * 2^F)
//   * H v, Lanczos residuals w:      Y = round(y * 2^G), G set from a bound on
//                                    max_i sum_j |H_ij| so |Y| < 2^61
//   * hop sums: amplitudes fall in K <= 4 magnitude classes; per element
//     S_k = sum_{hops in k} (+/-)V[src] is an exact int64 sum, then
//     Y = round((d_fx*V + sum_k a_fx[k]*S_k) / 2^(A+F-G)) with one rounding
//     (int64 x int64 -> int128 products)
//   * dot products are exact int128 sums (order independent, reproducible)
// Scalars (alpha, beta) stay FP64; they enter the element updates as int64
// fixed-point coefficients.
#pragma once

#include <vector>

#include "vca_common.cuh"
#include "vca_kernels.cuh"

namespace vca {

#define VCA_FX_KMAX 4

typedef long long i64;

struct FxScales {
  int F;   // vector scale 2^-F
  int G;   // H v / residual scale 2^-G
  int A;   // diagonal and amplitude coefficients 2^-A
  int C;   // alpha/beta coefficients 2^-C
};

struct FxView {
  const signed char* up_code;  // [width*dim]: class (bits 0-1), sign (bit 7)
  const signed char* dw_code;
  const unsigned* up_hop;      // [width*dim]: src (bits 0-23) | class << 24 | sign << 31
  const unsigned* dw_hop;
  const i64* up_e1;            // one-body + same-spin diagonal, scale 2^-A
  const i64* dw_e1;
  const int* up_npos;          // [dim]: leading positive hops of each row (hops sign sorted)
  const int* dw_npos;
  const int* up_perm;          // [dim]: up rows in order of decreasing hop count
  // up-spin tables re-indexed by position in up_perm (coalesced for the
  // staged column kernel): hop words [width*dim] k-major with the source as
  // its first swizzled shared-memory unit (4 src + ((src >> 1) & 3)) and the
  // class in bits 24-25, counts, positive counts, configurations, one-body
  // energies
  const unsigned* up_phop;
  const unsigned* up_rhop;     // the same hops with the source as its position in up_perm
  const int* up_pinv;          // position of each up configuration in up_perm
  int rows_permuted;           // 1: the batch's fast-index rows are in up_perm order
  const int* up_pcnt;
  const int* up_pnpos;
  const int* up_pword;
  const i64* up_pe1;
  // bank schedule of the paired-column single-vector kernel (fx_pair_schedule):
  // shared-memory byte offsets, warp w's round r, lane l at
  // up_sched[(up_wround[w] + r)*32 + l], rounds in groups of one class and
  // sign (up_wgrp[w*2K + g] rounds in group g); nullptr: the one-column form runs
  const unsigned* up_sched;
  const int* up_wround;
  const int* up_wgrp;
  int K;
  i64 afx[VCA_FX_KMAX];        // class amplitudes, scale 2^-A
  int norb;
  unsigned int omask[VCA_MAX_NORB];
  i64 Ufx[VCA_MAX_NORB];
  i64 Ustfx;
  i64 c0fx;
  int shift;                   // A + F - G
};

// Column batches of the fixed-point path are slab-major: slabs of W =
// fx_slab_w(m) adjacent columns, each slab one contiguous [D][W] block, so
// element (row i, column c) sits at ((c / W) * D + i) * W + c % W.  W = 8
// once m >= 8 (memory holds fx_cols_alloc(m) columns, the pad columns stay
// zero); below 8 columns W = m, plain row-major.  A slab of a 4x3-cluster
// sector is 47 MB, so the slab an H x v kernel works on stays in L2.
#define FX_SLAB 8
__host__ __device__ __forceinline__ int fx_slab_w(int m) { return m >= FX_SLAB ? FX_SLAB : m; }
__host__ __device__ __forceinline__ int fx_cols_alloc(int m) {
  return m >= FX_SLAB ? (m + FX_SLAB - 1) / FX_SLAB * FX_SLAB : m;
}
__host__ __device__ __forceinline__ int64_t fx_off(int64_t D, int W, int64_t i, int c) {
  return ((int64_t)(c / W) * D + i) * W + c % W;
}

// up-spin tables in the order of perm (see FxView::up_phop)
void launch_fx_perm_tables(int dim, int width, const int* perm, const int* pinv, const unsigned* hop,
                           const int* cnt, const int* npos, const int* words, const i64* e1, unsigned* phop,
                           unsigned* rhop, int* pcnt, int* pnpos, int* pword, i64* pe1, cudaStream_t st);
// partition each row's hop words positive-first in place; npos[row] counts them
void launch_fx_sign_sort(int dim, int width, const int* cnt, unsigned* hop, int* npos, cudaStream_t st);
// packed hop words src | class<<24 | sign<<31 from the FP64 tables
void launch_fx_pack(int dim, int width, const int* src, const double2* amp, const double* classes, int K,
                    unsigned* hop, cudaStream_t st);
// Y = H X on a slab-major column batch (m >= 16), one warp per row and
// 128-column slice; with apart != nullptr also the exact alpha partials
// <X,Y> per (row block, column), hxv_fx_w_rowblocks(D) rows of m int128
void launch_hxv_fx_w(const SectorView& sv, const FxView& fv, int m, const i64* X, i64* Y, i64* apart,
                     cudaStream_t st);
int hxv_fx_w_rowblocks(int64_t D);
// Y = H X on a slab-major column batch (m >= 16): the position-ordered
// form when fv.rows_permuted (rows of the fast spin role in up_perm order),
// else the shared-memory staged form while DimUp*128 bytes fit and
// warp_only is false, else the warp form; apart, when given, needs
// hxv_fx_cols_rows(...) rows of m int128
int hxv_fx_cols_rows(const SectorView& sv, const FxView& fv, int m, bool warp_only);
// the position-ordered form (fv.rows_permuted) applies: K <= 2, m >= 16 and
// the up block fits shared memory
bool hxv_fx_r_ok(const SectorView& sv, const FxView& fv, int m);
void launch_hxv_fx_cols(const SectorView& sv, const FxView& fv, int m, const i64* X, i64* Y, i64* apart,
                        bool warp_only, cudaStream_t st);
// per-hop class/sign codes from the FP64 amplitude tables
void launch_fx_codes(int dim, int width, const double2* amp, const double* classes, int K,
                     signed char* code, cudaStream_t st);
// FP64 one-body table -> fixed point
void launch_fx_e1(int dim, const double2* e1, int A, i64* e1fx, cudaStream_t st);
// Bank schedule of the paired-column staged up kernel.  Rows are taken in
// warps of 32, and a warp's hops in groups g = 2*class + (amplitude < 0);
// group g of warp w gets wgrp[w*2K + g] rounds (the most hops of that group
// in any of its rows), the groups' rounds follow one another from round
// wround[w], and each round holds one word per lane: the byte offset in the
// kernel's shared memory of the 16-byte unit the lane reads (a hop's source
// unit, or for a lane without a hop in that round a zero unit).  Within every
// quarter warp (8 lanes: one 128-byte shared-memory wavefront of 16-byte
// reads) a round's sources are chosen by bipartite matching (lanes by
// remaining hops, most first, against the bank groups src mod 8) so that
// they fall in distinct groups, and the zero unit read by idle lanes lies in
// a group no real lane of that round uses.  hop: the packed hop words
// [width*dim] (host copy); cnt: hop counts [dim].  The fixed-point hop sums
// are exact, so the order of a row's hops changes no result.  Returns the
// number of quarter-warp rounds that could not be made conflict free, or -1
// if a hop was left unplaced.
int64_t fx_pair_schedule(int dim, int width, int K, const int* cnt, const unsigned* hop,
                         std::vector<unsigned>& sched, std::vector<int>& wround, std::vector<int>& wgrp);
// bounded waits of the position-ordered kernel's bulk copies that ran out
// since the last call (the count is reset), -1 if it cannot be read
int fx_take_wait_failures();
// test hook: bytes the position-ordered kernel's copy barrier expects beyond
// those it copies (0: none), so that its bounded wait runs out
int fx_set_stage_extra_tx(int bytes);
// re-order the position-ordered kernel's up hops so the two rows of a
// quarter warp read sources of opposite parity where the counts allow
void fx_rhop_parity_order(int dim, int width, const int* cnt, const int* npos, unsigned* rhop);
// the paired-column form's shared memory: dim + FX1_ZERO_UNITS 16-byte units
// (the last ones zero, one per bank group)
#define FX1_ZERO_UNITS 8
#define FX1_SMEM_MAX (227 * 1024)
// single vectors of sectors from this dimension on take the staged two-kernel form
#define FX1_MIN_DIM (1 << 22)
inline bool fx_pair_fits(int dim) { return (size_t)(dim + FX1_ZERO_UNITS) * 16 <= FX1_SMEM_MAX; }
// Y = H X (FX) on a slab-major column batch, any m (the small-batch form)
void launch_hxv_fx(const SectorView& sv, const FxView& fv, int m, const i64* X, i64* Y, cudaStream_t st);
// per-column exact dot: out_col[c] = (sum X*Y) * 2^-(sx+sy) (double)
void launch_fx_dot(const ColBatch& b, const i64* X, const i64* Y, int sx, int sy, i64* partial, int nblk,
                   double* out_col, cudaStream_t st);
// per-chain coefficient to fixed point: cfx[ch] = round(scale * x[ch] * 2^C)
void launch_fx_coef(int nch, const double* x, double scale, int C, i64* cfx, cudaStream_t st);
// W = Y - (afx*X + bfx*Xp) >> (C+F-G)  (bfx ignored when use_b == 0)
void launch_fx_update(const ColBatch& b, const FxScales& s, const i64* afx, const i64* bfx, bool use_b,
                      const i64* X, const i64* Xp, const i64* Y, i64* W, cudaStream_t st);
// normalisation: X = W / beta per chain (scale 2^-G -> 2^-F), zero for retired chains
void launch_fx_normalize(const ColBatch& b, const FxScales& s, const double* invbeta, const i64* W,
                         i64* X, i64* scratch2nch, cudaStream_t st);
// generic per-chain scaling between scales: Xo = round(Xi * f[ch] * 2^(so - si))
void launch_fx_rescale(const ColBatch& b, const double* f, int si, int so, const i64* Xi, i64* Xo,
                       i64* scratch2nch, cudaStream_t st);
// psi += s[k] * X (single column, scale 2^-F)
void launch_fx_psi_accum(int64_t n, const double* s, int k, const i64* X, i64* psi, cudaStream_t st);
// FP64 <-> fixed point (one-time conversions)
void launch_fx_from_double(int64_t n, const double* x, int F, i64* X, cudaStream_t st);
void launch_fx_to_double(int64_t n, const i64* X, int F, double* x, cudaStream_t st);
// chain start vectors by exact gather (+/- psi, re/im columns) from a FX
// ground state, into a slab-major batch of m columns; swapped: batch row of
// element (iup, idw) is idw + iup*DimDw instead of iup + idw*DimUp; pinv
// (optional): the fast index is replaced by its position pinv[.]
void launch_chain_init_fx(const SectorView& tgt, int src_dimup, const i64* gs, int nchain,
                          const ChainInit* d_ci, int m, bool swapped, const int* pinv, i64* X,
                          cudaStream_t st);

// out[c] = (sum over `rows` int128 partials of column c) * 2^-sexp
void launch_fx_partial_reduce(int m, int rows, const i64* partial, int sexp, double* out, cudaStream_t st);
// fused W = Y - a X - b Xp and beta^2 partials (out_col = <W,W> per column)
void launch_fx_update_dot(const ColBatch& b, const FxScales& s, const i64* afx, const i64* bfx, bool use_b,
                          const i64* X, const i64* Xp, i64* YW, i64* partial, int nblk, double* out_col,
                          cudaStream_t st);

// start vector R = round(v * 2^40), v the splitmix64 values of the FP64 path
void launch_fx_start_raw(int64_t n, uint64_t seed, int isector, i64* R, cudaStream_t st);

}  // namespace vca
