// vca_fx.cu -- fixed-point (int64 / int128) Lanczos kernels for real
// Hamiltonians on GB300.  See vca_fx.cuh for the number format.
#include "vca_fx.cuh"

#include <atomic>
#include <algorithm>
#include <cmath>

namespace vca {

void count_launch_external();

typedef __int128 i128;
typedef unsigned long long u64;

static inline int nblk_fx(int64_t n, int threads, int cap = 152 * 16) {
  int64_t b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > cap) b = cap;
  return (int)b;
}

// Block shape of the per-column kernels on a slab-major batch: the W
// columns of one slab across threadIdx.x, a power of two RB of rows across
// threadIdx.y (W*RB <= 256), one slab per blockIdx.y.  A warp then covers
// 32/W consecutive rows of one slab: contiguous 256-byte runs.
static void slab_shape(int m, dim3& blk, int& nslab) {
  const int W = fx_slab_w(m);
  int rb = 1;
  while (rb * 2 * W <= 256) rb <<= 1;
  blk = dim3(W, rb, 1);
  nslab = (m + W - 1) / W;
}

// round-half-up arithmetic shift of an int128 by s >= 0
__device__ __forceinline__ i64 rshift_round(i128 p, int s) {
  if (s <= 0) return (i64)p;
  p += ((i128)1) << (s - 1);
  return (i64)(p >> s);
}

// the same for 1 <= s <= 63 on the two 64-bit words (no int128 shift)
__device__ __forceinline__ i64 rshift_round63(i128 p, int s) {
  u64 lo = (u64)p, hi = (u64)(p >> 64);
  const u64 r = 1ull << (s - 1);
  lo += r;
  hi += (lo < r) ? 1ull : 0ull;
  return (i64)((lo >> s) | (hi << (64 - s)));
}

// either form by a uniform flag (sh63: 1 <= s <= 63, the two-word form)
__device__ __forceinline__ i64 rshift_round_u(i128 p, int s, bool sh63) {
  if (sh63) return rshift_round63(p, s);
  return rshift_round(p, s);
}

__device__ __forceinline__ double i128_to_double(i128 v, int scale_exp) {
  const bool neg = v < 0;
  unsigned __int128 u = neg ? (unsigned __int128)(-v) : (unsigned __int128)v;
  const u64 hi = (u64)(u >> 64), lo = (u64)u;
  double d = (double)hi * 18446744073709551616.0 + (double)lo;
  d = ldexp(d, -scale_exp);
  return neg ? -d : d;
}

// ---------------------------------------------------------------------------
// tables
// ---------------------------------------------------------------------------
__global__ void k_fx_codes(int64_t n, const double2* amp, const double* classes, int K, signed char* code) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const double a = amp[t].x;
    const double mag = fabs(a);
    int cls = 0;
    for (int k = 0; k < K; k++)
      if (classes[k] == mag) cls = k;
    code[t] = (signed char)(cls | (a < 0.0 ? 0x80 : 0));
  }
}
void launch_fx_codes(int dim, int width, const double2* amp, const double* classes, int K,
                     signed char* code, cudaStream_t st) {
  count_launch_external();
  int64_t n = (int64_t)dim * width;
  if (n == 0) return;
  k_fx_codes<<<nblk_fx(n, 256), 256, 0, st>>>(n, amp, classes, K, code);
}

__global__ void k_fx_e1(int dim, const double2* e1, int A, i64* e1fx) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < dim; r += gridDim.x * blockDim.x)
    e1fx[r] = __double2ll_rn(ldexp(e1[r].x, A));
}
void launch_fx_e1(int dim, const double2* e1, int A, i64* e1fx, cudaStream_t st) {
  count_launch_external();
  k_fx_e1<<<nblk_fx(dim, 256), 256, 0, st>>>(dim, e1, A, e1fx);
}

// ---------------------------------------------------------------------------
// H x v in fixed point.  Same row/column mapping as the FP64 kernel; every hop
// is an exact int64 add into the accumulator of its amplitude class.
// ---------------------------------------------------------------------------
__device__ __forceinline__ i64 mixed_fx(const FxView& f, unsigned u, unsigned d) {
  if (f.norb == 1) return f.c0fx + f.Ufx[0] * (i64)__popc(u & d & f.omask[0]);
  i64 s = f.c0fx;
  for (int o = 0; o < f.norb; o++) s += f.Ufx[o] * (i64)__popc(u & d & f.omask[o]);
  int c = 0;
  for (int o = 0; o < f.norb; o++)
    for (int q = o + 1; q < f.norb; q++)
      c += __popc(u & f.omask[o] & (d >> (q - o))) + __popc(u & f.omask[q] & (d << (q - o)));
  return s + f.Ustfx * (i64)c;
}

template <int K>
__device__ __forceinline__ void acc_hop(i64 (&S)[K], signed char code, i64 v) {
  const i64 sv = (code < 0) ? -v : v;
  if (K == 1) {
    S[0] += sv;
  } else {
    const int cls = code & 3;
#pragma unroll
    for (int k = 0; k < K; k++) S[k] += (cls == k) ? sv : 0;
  }
}

// Small-batch form: column c of slab blockIdx.y on threadIdx.x, rows on
// threadIdx.y and the grid.
template <int K>
__global__ void k_hxv_fx(SectorView sv, FxView fv, int m, const i64* __restrict__ X, i64* __restrict__ Y) {
  const int64_t D = (int64_t)sv.dimup * sv.dimdw;
  const int W = blockDim.x;
  if ((int)(blockIdx.y * W + threadIdx.x) >= m) return;
  const int64_t sb = (int64_t)blockIdx.y * D * W + threadIdx.x;
  const i64* Xs = X + sb;
  i64* Ys = Y + sb;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.y + threadIdx.y; i < D;
       i += (int64_t)gridDim.x * blockDim.y) {
    const int idw = (int)(i / sv.dimup);
    const int iup = (int)(i - (int64_t)idw * sv.dimup);
    const i64 dfx = fv.up_e1[iup] + fv.dw_e1[idw] +
                    mixed_fx(fv, (unsigned)sv.up_words[iup], (unsigned)sv.dw_words[idw]);
    const int nu = sv.up_cnt[iup], nd = sv.dw_cnt[idw];
    const int64_t colbase = (int64_t)idw * sv.dimup;
    i64 S[K];
#pragma unroll
    for (int k = 0; k < K; k++) S[k] = 0;
    for (int h = 0; h < nu; h++) {
      const int64_t o = (int64_t)h * sv.dimup + iup;
      acc_hop<K>(S, fv.up_code[o], Xs[(colbase + sv.up_src[o]) * W]);
    }
    for (int h = 0; h < nd; h++) {
      const int64_t o = (int64_t)h * sv.dimdw + idw;
      acc_hop<K>(S, fv.dw_code[o], Xs[((int64_t)iup + (int64_t)sv.dw_src[o] * sv.dimup) * W]);
    }
    i128 p = (i128)dfx * Xs[i * W];
#pragma unroll
    for (int k = 0; k < K; k++) p += (i128)fv.afx[k] * S[k];
    Ys[i * W] = rshift_round(p, fv.shift);
  }
}


// Single-vector H x v for large sectors, in two kernels.
// Up part (+ diagonal): one CTA per down configuration idw stages its
// column X[:, idw] (DimUp contiguous int64) in shared memory; every up hop
// is a shared-memory read.  Y = round((d x + sum_k a_k S_k^up) 2^-shift).
template <int K>
__global__ void __launch_bounds__(1024, 2) k_hxv1_up(SectorView sv, FxView fv, const i64* __restrict__ X,
                                                 i64* __restrict__ Y) {
  extern __shared__ __align__(16) i64 x1s[];
  const int DU = sv.dimup;
  const int idw = blockIdx.x;
  const int64_t base = (int64_t)idw * DU;
  for (int t = threadIdx.x; t < DU; t += blockDim.x) x1s[t] = (i64)__ldcg((const long long*)X + base + t);
  __syncthreads();
  const i64 e1d = fv.dw_e1[idw];
  const unsigned wdw = (unsigned)sv.dw_words[idw];
  for (int iup = threadIdx.x; iup < DU; iup += blockDim.x) {
    u64 S[K];
#pragma unroll
    for (int k = 0; k < K; k++) S[k] = 0;
    const int nu = sv.up_cnt[iup], np = fv.up_npos[iup];
    int h = 0, o = iup;
    for (; h < np; h++, o += DU) {
      const unsigned hw = fv.up_hop[o];
      const i64 v = x1s[hw & 0xFFFFFFu];
      const int cls = (K == 1) ? 0 : (int)((hw >> 24) & 3u);
#pragma unroll
      for (int k = 0; k < K; k++)
        if (k == cls) S[k] += (u64)v;
    }
    for (; h < nu; h++, o += DU) {
      const unsigned hw = fv.up_hop[o];
      const i64 v = x1s[hw & 0xFFFFFFu];
      const int cls = (K == 1) ? 0 : (int)((hw >> 24) & 3u);
#pragma unroll
      for (int k = 0; k < K; k++)
        if (k == cls) S[k] -= (u64)v;
    }
    const i64 dfx = fv.up_e1[iup] + e1d + mixed_fx(fv, (unsigned)sv.up_words[iup], wdw);
    i128 p = (i128)dfx * x1s[iup];
#pragma unroll
    for (int k = 0; k < K; k++) p += (i128)fv.afx[k] * (i64)S[k];
    __stcg((long long*)Y + base + iup, (long long)rshift_round(p, fv.shift));
  }
}

// Down part: Y[chunk, idw] += round(sum_k a_k S_k^dw 2^-shift), S^dw the
// signed sum of rows `chunk` of the neighbour columns X[:, idw'] (the hop
// list of idw, the same for every row).  CTAs are ordered chunk-major, so
// the rows of one chunk of every column (chunk * DimDw * 8 bytes, <= 64 MB)
// stay in L2 while the CTAs of that chunk run; every row read is a
// coalesced stream.
#define FX1_CHUNK_BYTES (64u << 20)
template <int K>
__global__ void __launch_bounds__(256) k_hxv1_dw(SectorView sv, FxView fv, int chunk_rows,
                                                 const i64* __restrict__ X, i64* __restrict__ Y) {
  extern __shared__ __align__(16) unsigned char x1d_smem[];
  const int DU = sv.dimup, DD = sv.dimdw;
  const int ck = blockIdx.x / DD;
  const int idw = blockIdx.x - ck * DD;
  int64_t* doff = (int64_t*)x1d_smem;
  unsigned char* dcl = (unsigned char*)(doff + sv.wdw);
  const int nd = sv.dw_cnt[idw], ndp = fv.dw_npos[idw];
  for (int h = threadIdx.x; h < nd; h += blockDim.x) {
    const unsigned hw = fv.dw_hop[idw + h * DD];
    doff[h] = ((int64_t)(hw & 0xFFFFFFu) - idw) * DU;
    dcl[h] = (unsigned char)((hw >> 24) & 3u);
  }
  __syncthreads();
  const int64_t base = (int64_t)idw * DU;
  const int r0 = ck * chunk_rows, r1 = min(DU, r0 + chunk_rows);
  const long long* Xb = (const long long*)X + base;
  for (int iup = r0 + threadIdx.x; iup < r1; iup += blockDim.x) {
    u64 S[K];
#pragma unroll
    for (int k = 0; k < K; k++) S[k] = 0;
    int h = 0;
#pragma unroll 4
    for (; h < ndp; h++) {
      const i64 v = (i64)__ldcg(Xb + iup + doff[h]);
      const int cls = (K == 1) ? 0 : (int)dcl[h];
#pragma unroll
      for (int k = 0; k < K; k++)
        if (k == cls) S[k] += (u64)v;
    }
#pragma unroll 4
    for (; h < nd; h++) {
      const i64 v = (i64)__ldcg(Xb + iup + doff[h]);
      const int cls = (K == 1) ? 0 : (int)dcl[h];
#pragma unroll
      for (int k = 0; k < K; k++)
        if (k == cls) S[k] -= (u64)v;
    }
    i128 p = 0;
#pragma unroll
    for (int k = 0; k < K; k++) p += (i128)fv.afx[k] * (i64)S[k];
    long long* yo = (long long*)Y + base + iup;
    __stcg(yo, (long long)((i64)__ldcg(yo) + rshift_round(p, fv.shift)));
  }
}

// The rounds of warp-row w of the bank schedule (fx_pair_schedule) over the
// staged 16-byte units at smem: A[k], B[k] = signed class-k hop sums of the
// lane's row in the units' first and second words.  Every round of the warp
// is one 16-byte read per lane; 8 schedule words are loaded ahead.
template <int K>
__device__ __forceinline__ void up2_rounds(const FxView& fv, int w, int lane, int DU,
                                           const unsigned char* __restrict__ x1p_smem, u64 (&A)[K], u64 (&B)[K]) {
#pragma unroll
  for (int k = 0; k < K; k++) A[k] = B[k] = 0;
  const unsigned* sp = fv.up_sched + (size_t)fv.up_wround[w] * 32 + lane;
  const int* gr = fv.up_wgrp + w * 2 * K;
#pragma unroll
  for (int g = 0; g < 2 * K; g++) {
    const int Rg = gr[g];
    u64 a = 0, b = 0;
    int r = 0;
    for (; r + 8 <= Rg; r += 8) {  // 8 schedule loads in flight, then 8 unit reads
      unsigned o[8];
#pragma unroll
      for (int u = 0; u < 8; u++) o[u] = __ldg(sp + (r + u) * 32);
#pragma unroll
      for (int u = 0; u < 8; u += 2) {
        const longlong2 v0 = *(const longlong2*)(x1p_smem + o[u]);
        const longlong2 v1 = *(const longlong2*)(x1p_smem + o[u + 1]);
        a += (u64)v0.x + (u64)v1.x;
        b += (u64)v0.y + (u64)v1.y;
      }
    }
    if (r + 4 <= Rg) {
      unsigned o[4];
#pragma unroll
      for (int u = 0; u < 4; u++) o[u] = __ldg(sp + (r + u) * 32);
#pragma unroll
      for (int u = 0; u < 4; u += 2) {
        const longlong2 v0 = *(const longlong2*)(x1p_smem + o[u]);
        const longlong2 v1 = *(const longlong2*)(x1p_smem + o[u + 1]);
        a += (u64)v0.x + (u64)v1.x;
        b += (u64)v0.y + (u64)v1.y;
      }
      r += 4;
    }
    if (r < Rg) {  // 1..3 rounds left: their loads together
      const unsigned o0 = __ldg(sp + r * 32);
      const unsigned o1 = r + 1 < Rg ? __ldg(sp + (r + 1) * 32) : 16u * (unsigned)DU;
      const unsigned o2 = r + 2 < Rg ? __ldg(sp + (r + 2) * 32) : 16u * (unsigned)DU;
      const longlong2 v0 = *(const longlong2*)(x1p_smem + o0);
      a += (u64)v0.x;
      b += (u64)v0.y;
      if (r + 1 < Rg) {
        const longlong2 v1 = *(const longlong2*)(x1p_smem + o1);
        a += (u64)v1.x;
        b += (u64)v1.y;
      }
      if (r + 2 < Rg) {
        const longlong2 v2 = *(const longlong2*)(x1p_smem + o2);
        a += (u64)v2.x;
        b += (u64)v2.y;
      }
    }
    sp += Rg * 32;
    if (g & 1) {
      A[g >> 1] -= a;
      B[g >> 1] -= b;
    } else {
      A[g >> 1] += a;
      B[g >> 1] += b;
    }
  }
}

// Paired-column up part (+ diagonal): one CTA stages columns idw0 = 2*bx and
// idw0 + 1 interleaved, one 16-byte unit (X[iup, idw0], X[iup, idw0+1]) per
// up configuration (then FX1_ZERO_UNITS zero units), and walks the bank
// schedule (fx_pair_schedule).  A warp's rounds come in groups of one
// amplitude class and one sign, so a round is one 16-byte shared-memory read
// and a plain 64-bit add per column: no per-hop class or sign logic.  Each
// schedule word (the unit's byte offset) serves both columns, the 8 lanes of
// a quarter warp read distinct units, and the schedule is read from L2 once
// per two columns.  The int128 sum and its single rounding are those of the
// one-column form, bit for bit.
#define FX1_UP2_THREADS 1024
template <int K>
__global__ void __launch_bounds__(FX1_UP2_THREADS, 1) k_hxv1_up2(SectorView sv, FxView fv, const i64* __restrict__ X,
                                                             i64* __restrict__ Y) {
  extern __shared__ __align__(16) unsigned char x1p_smem[];
  longlong2* xs = (longlong2*)x1p_smem;
  const int DU = sv.dimup, DD = sv.dimdw;
  const int idw0 = 2 * blockIdx.x;
  const bool two = idw0 + 1 < DD;
  const long long* c0 = (const long long*)X + (int64_t)idw0 * DU;
  const long long* c1 = c0 + DU;
  constexpr int U = 8;  // loads in flight per thread and column
  for (int t0 = threadIdx.x; t0 < DU; t0 += U * FX1_UP2_THREADS) {
    long long a[U], b[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int t = t0 + u * FX1_UP2_THREADS;
      a[u] = t < DU ? __ldcs(c0 + t) : 0ll;
      b[u] = (two && t < DU) ? __ldcs(c1 + t) : 0ll;
    }
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int t = t0 + u * FX1_UP2_THREADS;
      if (t < DU) xs[t] = make_longlong2(a[u], b[u]);
    }
  }
  if (threadIdx.x < FX1_ZERO_UNITS) xs[DU + threadIdx.x] = make_longlong2(0ll, 0ll);
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int nw = (DU + 31) >> 5;
  const bool sh63 = fv.shift >= 1 && fv.shift <= 63;
  const i64 e1d0 = fv.dw_e1[idw0], e1d1 = two ? fv.dw_e1[idw0 + 1] : 0;
  const unsigned wd0 = (unsigned)sv.dw_words[idw0], wd1 = two ? (unsigned)sv.dw_words[idw0 + 1] : 0u;
  for (int w = threadIdx.x >> 5; w < nw; w += FX1_UP2_THREADS / 32) {
    const int iup = w * 32 + lane;
    const bool row = iup < DU;
    const i64 eu = row ? fv.up_e1[iup] : 0;  // the epilogue's tables, ahead of the rounds
    const unsigned wu = row ? (unsigned)sv.up_words[iup] : 0u;
    u64 A[K], B[K];
    up2_rounds<K>(fv, w, lane, DU, x1p_smem, A, B);
    if (!row) continue;
    const longlong2 xi = xs[iup];
    i128 p0 = (i128)(eu + e1d0 + mixed_fx(fv, wu, wd0)) * xi.x;
#pragma unroll
    for (int k = 0; k < K; k++) p0 += (i128)fv.afx[k] * (i64)A[k];
    __stcs((long long*)Y + (int64_t)idw0 * DU + iup, (long long)rshift_round_u(p0, fv.shift, sh63));
    if (two) {
      i128 p1 = (i128)(eu + e1d1 + mixed_fx(fv, wu, wd1)) * xi.y;
#pragma unroll
      for (int k = 0; k < K; k++) p1 += (i128)fv.afx[k] * (i64)B[k];
      __stcs((long long*)Y + (int64_t)(idw0 + 1) * DU + iup, (long long)rshift_round_u(p1, fv.shift, sh63));
    }
  }
}

// Down part on row pairs (DimUp even): as k_hxv1_dw, each thread two
// adjacent rows of one chunk, every neighbour row pair one 16-byte L2 read;
// chunks of FX1_DW2_ROWS-row multiples (one pair per thread).
#define FX1_DW2_ROWS 512
template <int K>
__global__ void __launch_bounds__(FX1_DW2_ROWS / 2) k_hxv1_dw2(SectorView sv, FxView fv, int chunk_rows,
                                                          const i64* __restrict__ X, i64* __restrict__ Y) {
  extern __shared__ __align__(16) unsigned char x1d_smem[];
  const int DU = sv.dimup, DD = sv.dimdw;
  const int ck = blockIdx.x / DD;
  const int idw = blockIdx.x - ck * DD;
  const int64_t DU2 = DU / 2;
  int64_t* doff = (int64_t*)x1d_smem;  // neighbour column offsets in row pairs
  unsigned char* dcl = (unsigned char*)(doff + sv.wdw);
  const int nd = sv.dw_cnt[idw], ndp = fv.dw_npos[idw];
  for (int h = threadIdx.x; h < nd; h += blockDim.x) {
    const unsigned hw = fv.dw_hop[idw + h * DD];
    doff[h] = ((int64_t)(hw & 0xFFFFFFu) - idw) * DU2;
    dcl[h] = (unsigned char)((hw >> 24) & 3u);
  }
  __syncthreads();
  const int64_t base2 = (int64_t)idw * DU2;
  const int q0 = ck * (chunk_rows / 2), q1 = (int)min((int64_t)DU2, (int64_t)(ck + 1) * (chunk_rows / 2));
  const longlong2* Xb = (const longlong2*)X + base2;
  longlong2* Yb = (longlong2*)Y + base2;
  for (int q = q0 + threadIdx.x; q < q1; q += blockDim.x) {
    const longlong2 y = __ldcs(Yb + q);
    u64 A[K], B[K];
#pragma unroll
    for (int k = 0; k < K; k++) A[k] = B[k] = 0;
    int h = 0;
#pragma unroll 4
    for (; h < ndp; h++) {
      const longlong2 v = __ldcg(Xb + q + doff[h]);
      const int cls = (K == 1) ? 0 : (int)dcl[h];
#pragma unroll
      for (int k = 0; k < K; k++)
        if (k == cls) A[k] += (u64)v.x, B[k] += (u64)v.y;
    }
#pragma unroll 4
    for (; h < nd; h++) {
      const longlong2 v = __ldcg(Xb + q + doff[h]);
      const int cls = (K == 1) ? 0 : (int)dcl[h];
#pragma unroll
      for (int k = 0; k < K; k++)
        if (k == cls) A[k] -= (u64)v.x, B[k] -= (u64)v.y;
    }
    i128 pa = 0, pb = 0;
#pragma unroll
    for (int k = 0; k < K; k++) pa += (i128)fv.afx[k] * (i64)A[k], pb += (i128)fv.afx[k] * (i64)B[k];
    const bool sh63 = fv.shift >= 1 && fv.shift <= 63;
    __stcs(Yb + q, make_longlong2((long long)((i64)y.x + rshift_round_u(pa, fv.shift, sh63)),
                                  (long long)((i64)y.y + rshift_round_u(pb, fv.shift, sh63))));
  }
}

// ---- host: the bank schedule of k_hxv1_up2 ----
namespace {
struct QuarterMatch {  // lanes of one quarter warp against the 8 bank groups of 16-byte units
  const std::vector<unsigned>* rem;
  int unit_lane[8], lane_unit[8];
  bool seen[8];
  bool augment(int j) {
    for (unsigned src : rem[j]) {
      const int u = (int)(src & 7u);
      if (seen[u]) continue;
      seen[u] = true;
      if (unit_lane[u] < 0 || augment(unit_lane[u])) {
        unit_lane[u] = j;
        lane_unit[j] = u;
        return true;
      }
    }
    return false;
  }
};
}  // namespace

int64_t fx_pair_schedule(int dim, int width, int K, const int* cnt, const unsigned* hop,
                         std::vector<unsigned>& sched, std::vector<int>& wround, std::vector<int>& wgrp) {
  const int nw = (dim + 31) / 32, NG = 2 * K;
  auto group = [&](unsigned hw) { return 2 * (int)((hw >> 24) & 3u) + (int)(hw >> 31); };
  wround.assign(nw + 1, 0);
  wgrp.assign((size_t)nw * NG, 0);
  for (int w = 0; w < nw; w++) {
    for (int l = 0; l < 32 && w * 32 + l < dim; l++) {
      const int r = w * 32 + l;
      int c[2 * VCA_FX_KMAX] = {0};
      for (int h = 0; h < cnt[r] && h < width; h++) {
        const int gg = group(hop[(size_t)h * dim + r]);
        if (gg >= NG) return -1;
        c[gg]++;
      }
      for (int gg = 0; gg < NG; gg++) wgrp[(size_t)w * NG + gg] = std::max(wgrp[(size_t)w * NG + gg], c[gg]);
    }
    int R = 0;
    for (int gg = 0; gg < NG; gg++) R += wgrp[(size_t)w * NG + gg];
    wround[w + 1] = wround[w] + R;
  }
  sched.assign((size_t)wround[nw] * 32, 0u);
  int64_t conflicts = 0;
  std::vector<unsigned> rem[8];
  for (int w = 0; w < nw; w++) {
    for (int q = 0; q < 4; q++) {
      int rd0 = wround[w];
      for (int gg = 0; gg < NG; gg++) {
        const int R = wgrp[(size_t)w * NG + gg];
        for (int j = 0; j < 8; j++) {
          rem[j].clear();
          const int r = w * 32 + q * 8 + j;
          if (r < dim)
            for (int h = 0; h < cnt[r] && h < width; h++) {
              const unsigned hw = hop[(size_t)h * dim + r];
              if (group(hw) == gg) rem[j].push_back(hw & 0xFFFFFFu);
            }
        }
        for (int rd = 0; rd < R; rd++) {
          int ord[8];
          for (int j = 0; j < 8; j++) ord[j] = j;
          std::stable_sort(ord, ord + 8, [&](int a, int b) { return rem[a].size() > rem[b].size(); });
          QuarterMatch qm;
          qm.rem = rem;
          for (int u = 0; u < 8; u++) qm.unit_lane[u] = qm.lane_unit[u] = -1;
          for (int t = 0; t < 8; t++) {
            const int j = ord[t];
            if (rem[j].empty()) break;
            for (int u = 0; u < 8; u++) qm.seen[u] = false;
            qm.augment(j);
          }
          int load[8] = {0, 0, 0, 0, 0, 0, 0, 0};
          unsigned src[8];
          bool real[8];
          for (int j = 0; j < 8; j++) {
            real[j] = false;
            if (qm.lane_unit[j] < 0) continue;
            for (size_t i = 0; i < rem[j].size(); i++)
              if ((int)(rem[j][i] & 7u) == qm.lane_unit[j]) {
                src[j] = rem[j][i];
                rem[j].erase(rem[j].begin() + (std::ptrdiff_t)i);
                break;
              }
            real[j] = true;
            load[qm.lane_unit[j]]++;
          }
          bool conflict = false;
          for (int j = 0; j < 8; j++) {  // lanes that must take a hop in every remaining round
            if (real[j] || (int)rem[j].size() < R - rd) continue;
            size_t best = 0;
            for (size_t i = 1; i < rem[j].size(); i++)
              if (load[rem[j][i] & 7u] < load[rem[j][best] & 7u]) best = i;
            src[j] = rem[j][best];
            rem[j].erase(rem[j].begin() + (std::ptrdiff_t)best);
            real[j] = true;
            conflict = conflict || load[src[j] & 7u] > 0;
            load[src[j] & 7u]++;
          }
          conflicts += conflict ? 1 : 0;
          // lanes without a hop read a zero unit in a bank group no real lane uses
          // (there is one whenever such a lane exists: at most 7 real lanes)
          int freeg = 0;
          while (freeg < 7 && load[freeg] > 0) freeg++;
          const unsigned zero_unit = (unsigned)dim + (unsigned)((freeg - dim % 8 + 8) % 8);
          unsigned* out = sched.data() + (size_t)(rd0 + rd) * 32 + q * 8;
          for (int j = 0; j < 8; j++) out[j] = 16u * (real[j] ? src[j] : zero_unit);
        }
        for (int j = 0; j < 8; j++)
          if (!rem[j].empty()) return -1;
        rd0 += R;
      }
    }
  }
  return conflicts;
}

// Hop order of the position-ordered column kernel (k_hxv_fx_r): the two rows
// 2i, 2i+1 share a quarter warp, each reading the four 16-byte units of its
// source row, so a round is conflict free when their sources differ in
// parity.  Within each sign group the rows' hops are re-ordered so that
// even sources of one row meet odd sources of the other as often as the
// counts allow; the rest follow.  rhop: [width*dim] words, k-major; cnt,
// npos: per row (all in position order).  Exact sums: no result changes.
void fx_rhop_parity_order(int dim, int width, const int* cnt, const int* npos, unsigned* rhop) {
  std::vector<unsigned> A[2], B[2], oa, ob;
  for (int r = 0; r + 1 < dim; r += 2) {
    for (int grp = 0; grp < 2; grp++) {
      const int a0 = grp ? npos[r] : 0, a1 = grp ? cnt[r] : npos[r];
      const int b0 = grp ? npos[r + 1] : 0, b1 = grp ? cnt[r + 1] : npos[r + 1];
      for (int q = 0; q < 2; q++) A[q].clear(), B[q].clear();
      for (int h = a0; h < a1 && h < width; h++) {
        const unsigned w = rhop[(size_t)h * dim + r];
        A[(w & 0xFFFFFFu) & 1u].push_back(w);
      }
      for (int h = b0; h < b1 && h < width; h++) {
        const unsigned w = rhop[(size_t)h * dim + r + 1];
        B[(w & 0xFFFFFFu) & 1u].push_back(w);
      }
      oa.clear();
      ob.clear();
      size_t i0 = 0, i1 = 0;  // even of A with odd of B, then odd of A with even of B
      for (; i0 < A[0].size() && i0 < B[1].size(); i0++) oa.push_back(A[0][i0]), ob.push_back(B[1][i0]);
      for (; i1 < A[1].size() && i1 < B[0].size(); i1++) oa.push_back(A[1][i1]), ob.push_back(B[0][i1]);
      for (size_t i = i0; i < A[0].size(); i++) oa.push_back(A[0][i]);
      for (size_t i = i1; i < A[1].size(); i++) oa.push_back(A[1][i]);
      for (size_t i = i0; i < B[1].size(); i++) ob.push_back(B[1][i]);
      for (size_t i = i1; i < B[0].size(); i++) ob.push_back(B[0][i]);
      for (int h = a0; h < a1 && h < width; h++) rhop[(size_t)h * dim + r] = oa[h - a0];
      for (int h = b0; h < b1 && h < width; h++) rhop[(size_t)h * dim + r + 1] = ob[h - b0];
    }
  }
}

static bool hxv1_ok(const SectorView& sv, const FxView& fv, int m) {
  return m == 1 && fv.up_npos && fv.dw_npos && (int64_t)sv.dimup * sv.dimdw >= FX1_MIN_DIM &&
         (size_t)sv.dimup * sizeof(i64) <= 200 * 1024;
}

template <int K>
static void launch_hxv1_k(const SectorView& sv, const FxView& fv, const i64* X, i64* Y, cudaStream_t st) {
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_hxv1_up<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(k_hxv1_up2<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, FX1_SMEM_MAX);
    attr = true;
  }
  count_launch_external();
  count_launch_external();
  const bool paired = fv.up_sched && fv.up_wround && fv.up_wgrp && fx_pair_fits(sv.dimup);
  if (paired)
    k_hxv1_up2<K><<<(sv.dimdw + 1) / 2, FX1_UP2_THREADS, (size_t)(sv.dimup + FX1_ZERO_UNITS) * 16, st>>>(sv, fv, X,
                                                                                                     Y);
  else
    k_hxv1_up<K><<<sv.dimdw, 1024, (size_t)sv.dimup * sizeof(i64), st>>>(sv, fv, X, Y);
  if (paired && sv.dimup % 2 == 0) {  // row pairs: 16-byte streams of the neighbour columns
    const int64_t fit = FX1_CHUNK_BYTES / ((int64_t)sv.dimdw * sizeof(i64));
    int rows = (int)std::max<int64_t>(FX1_DW2_ROWS, fit / FX1_DW2_ROWS * FX1_DW2_ROWS);
    rows = std::min(rows, (sv.dimup + FX1_DW2_ROWS - 1) / FX1_DW2_ROWS * FX1_DW2_ROWS);
    const int nck = (sv.dimup + rows - 1) / rows;
    k_hxv1_dw2<K><<<nck * sv.dimdw, FX1_DW2_ROWS / 2, (size_t)sv.wdw * 9 + 16, st>>>(sv, fv, rows, X, Y);
    return;
  }
  int rows = (int)std::max<int64_t>(256, FX1_CHUNK_BYTES / ((int64_t)sv.dimdw * sizeof(i64)));
  rows = std::min(rows, sv.dimup);
  const int nck = (sv.dimup + rows - 1) / rows;
  k_hxv1_dw<K><<<nck * sv.dimdw, 256, (size_t)sv.wdw * 9 + 16, st>>>(sv, fv, rows, X, Y);
}

void launch_hxv_fx(const SectorView& sv, const FxView& fv, int m, const i64* X, i64* Y, cudaStream_t st) {
  if (hxv1_ok(sv, fv, m)) {  // one vector of a large sector: the two-kernel staged form
    switch (fv.K) {
      case 1: launch_hxv1_k<1>(sv, fv, X, Y, st); break;
      case 2: launch_hxv1_k<2>(sv, fv, X, Y, st); break;
      case 3: launch_hxv1_k<3>(sv, fv, X, Y, st); break;
      default: launch_hxv1_k<4>(sv, fv, X, Y, st); break;
    }
    return;
  }
  count_launch_external();
  dim3 blk;
  int ns;
  slab_shape(m, blk, ns);
  const int64_t D = (int64_t)sv.dimup * sv.dimdw;
  const dim3 grd(nblk_fx(D, blk.y, 152 * 32), ns, 1);
  switch (fv.K) {
    case 1: k_hxv_fx<1><<<grd, blk, 0, st>>>(sv, fv, m, X, Y); break;
    case 2: k_hxv_fx<2><<<grd, blk, 0, st>>>(sv, fv, m, X, Y); break;
    case 3: k_hxv_fx<3><<<grd, blk, 0, st>>>(sv, fv, m, X, Y); break;
    default: k_hxv_fx<4><<<grd, blk, 0, st>>>(sv, fv, m, X, Y); break;
  }
}

// ---------------------------------------------------------------------------
// exact dot products
// ---------------------------------------------------------------------------
__global__ void k_fx_dot(int64_t rows, int m, const i64* X, const i64* Y, i64* partial) {
  extern __shared__ i128 shq[];
  const int CW = blockDim.x, RB = blockDim.y;
  const int c = blockIdx.y * CW + threadIdx.x;
  const int64_t sb = (int64_t)blockIdx.y * rows * CW + threadIdx.x;
  i128 s = 0;
  if (c < m)
    for (int64_t i = (int64_t)blockIdx.x * RB + threadIdx.y; i < rows; i += (int64_t)gridDim.x * RB)
      s += (i128)X[sb + i * CW] * Y[sb + i * CW];
  shq[threadIdx.y * CW + threadIdx.x] = s;
  __syncthreads();
  for (int h = RB / 2; h > 0; h >>= 1) {
    if (threadIdx.y < h) shq[threadIdx.y * CW + threadIdx.x] += shq[(threadIdx.y + h) * CW + threadIdx.x];
    __syncthreads();
  }
  if (threadIdx.y == 0 && c < m) {
    const i128 v = shq[threadIdx.x];
    partial[2 * ((int64_t)blockIdx.x * m + c)] = (i64)(u64)v;
    partial[2 * ((int64_t)blockIdx.x * m + c) + 1] = (i64)(v >> 64);
  }
}
void launch_fx_dot(const ColBatch& b, const i64* X, const i64* Y, int sx, int sy, i64* partial, int nblk,
                   double* out_col, cudaStream_t st) {
  count_launch_external();
  dim3 blk;
  int ns;
  slab_shape(b.m, blk, ns);
  dim3 grd(nblk, ns, 1);
  k_fx_dot<<<grd, blk, sizeof(i128) * 256, st>>>(b.rows, b.m, X, Y, partial);
  launch_fx_partial_reduce(b.m, nblk, partial, sx + sy, out_col, st);
}

// ---------------------------------------------------------------------------
// element updates
// ---------------------------------------------------------------------------
__global__ void k_fx_coef(int nch, const double* x, double scale, int C, i64* cfx) {
  for (int ch = blockIdx.x * blockDim.x + threadIdx.x; ch < nch; ch += gridDim.x * blockDim.x)
    cfx[ch] = __double2ll_rn(ldexp(scale * x[ch], C));
}
void launch_fx_coef(int nch, const double* x, double scale, int C, i64* cfx, cudaStream_t st) {
  count_launch_external();
  k_fx_coef<<<nblk_fx(nch, 128), 128, 0, st>>>(nch, x, scale, C, cfx);
}

__global__ void k_fx_update(int64_t rows, int m, const int* col2ch, const ChainMeta* meta, int sh,
                            const i64* afx, const i64* bfx, int use_b, const i64* X, const i64* Xp,
                            const i64* Y, i64* Wo) {
  const int CW = blockDim.x, RB = blockDim.y;
  const int c = blockIdx.y * CW + threadIdx.x;
  if (c >= m) return;
  const int ch = col2ch[c];
  if (!meta[ch].active) return;
  const i64 a = afx[ch], b = use_b ? bfx[ch] : 0;
  const int64_t sb = (int64_t)blockIdx.y * rows * CW + threadIdx.x;
  for (int64_t i = (int64_t)blockIdx.x * RB + threadIdx.y; i < rows; i += (int64_t)gridDim.x * RB) {
    const int64_t g = sb + i * CW;
    i128 p = (i128)a * X[g];
    if (use_b) p += (i128)b * Xp[g];
    Wo[g] = Y[g] - rshift_round(p, sh);
  }
}
void launch_fx_update(const ColBatch& b, const FxScales& s, const i64* afx, const i64* bfx, bool use_b,
                      const i64* X, const i64* Xp, const i64* Y, i64* W, cudaStream_t st) {
  count_launch_external();
  dim3 blk;
  int ns;
  slab_shape(b.m, blk, ns);
  const dim3 grd(nblk_fx(b.rows, blk.y), ns, 1);
  k_fx_update<<<grd, blk, 0, st>>>(b.rows, b.m, b.col2ch, b.meta, s.C + s.F - s.G, afx, bfx, use_b ? 1 : 0, X,
                                   Xp, Y, W);
}

// per-chain multiplier m = round(f * 2^E) < 2^61 and shift E + si - so
__global__ void k_fx_mult(int nch, const double* f, int si, int so, i64* mul, i64* sh) {
  for (int ch = blockIdx.x * blockDim.x + threadIdx.x; ch < nch; ch += gridDim.x * blockDim.x) {
    const double x = f[ch];
    if (x == 0.0 || !isfinite(x)) { mul[ch] = 0; sh[ch] = 0; continue; }
    int e;
    frexp(fabs(x), &e);       // |x| in [2^(e-1), 2^e)
    int E = 60 - e;           // |x| * 2^E < 2^60
    int shift = E + si - so;
    if (shift > 120) { E -= shift - 120; shift = 120; }
    if (shift < 0) { E -= shift; shift = 0; }
    mul[ch] = __double2ll_rn(ldexp(x, E));
    sh[ch] = shift;
  }
}
// slab-tiled: block (W columns x RB rows), slab from blockIdx.y, so no
// per-element division
__global__ void k_fx_apply(int64_t rows, int m, const int* col2ch, const ChainMeta* meta, const i64* mul,
                           const i64* sh, int zero_inactive, const i64* Xi, i64* Xo) {
  const int CW = blockDim.x, RB = blockDim.y;
  const int c = blockIdx.y * CW + threadIdx.x;
  if (c >= m) return;
  const int ch = col2ch[c];
  const bool act = meta[ch].active;
  if (!act && !zero_inactive) return;
  const i64 mu = mul[ch];
  const int s = (int)sh[ch];
  const int64_t sb = (int64_t)blockIdx.y * rows * CW + threadIdx.x;
  for (int64_t i = (int64_t)blockIdx.x * RB + threadIdx.y; i < rows; i += (int64_t)gridDim.x * RB) {
    const int64_t g = sb + i * CW;
    Xo[g] = act ? rshift_round((i128)mu * Xi[g], s) : 0;
  }
}
// The same on 8-column slabs with 16-byte accesses (columns 2tx, 2tx+1 of
// slab blockIdx.y); a column that is not written (retired with
// zero_inactive == 0, or a pad column) keeps its value.
__global__ void __launch_bounds__(256) k_fx_apply8(int64_t rows, int m, const int* col2ch, const ChainMeta* meta,
                                                   const i64* mul, const i64* sh, int zero_inactive, const i64* Xi,
                                                   i64* Xo) {
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int c0 = blockIdx.y * FX_SLAB + 2 * tx;
  i64 mu[2] = {0, 0};
  int sv[2] = {0, 0};
  bool wr[2] = {false, false};
#pragma unroll
  for (int j = 0; j < 2; j++) {
    const int c = c0 + j;
    if (c < m) {
      const int ch = col2ch[c];
      const bool act = meta[ch].active != 0;
      wr[j] = act || zero_inactive;
      if (act) { mu[j] = mul[ch]; sv[j] = (int)sh[ch]; }
    }
  }
  if (!wr[0] && !wr[1]) return;
  const bool s63a = sv[0] >= 1 && sv[0] <= 63, s63b = sv[1] >= 1 && sv[1] <= 63;
  const int64_t sb = (int64_t)blockIdx.y * rows * (FX_SLAB / 2) + tx;
  const longlong2* I2 = (const longlong2*)Xi + sb;
  longlong2* O2 = (longlong2*)Xo + sb;
  const int64_t stride = (int64_t)gridDim.x * blockDim.y;
  constexpr int U = 4;  // rows in flight per thread
  for (int64_t i0 = (int64_t)blockIdx.x * blockDim.y + ty; i0 < rows; i0 += U * stride) {
    longlong2 v[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int64_t i = i0 + u * stride;
      v[u] = i < rows ? I2[i * 4] : make_longlong2(0ll, 0ll);
    }
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int64_t i = i0 + u * stride;
      if (i >= rows) break;
      const i64 o0 = s63a ? rshift_round63((i128)mu[0] * v[u].x, sv[0]) : rshift_round((i128)mu[0] * v[u].x, sv[0]);
      const i64 o1 = s63b ? rshift_round63((i128)mu[1] * v[u].y, sv[1]) : rshift_round((i128)mu[1] * v[u].y, sv[1]);
      if (wr[0] && wr[1]) {
        O2[i * 4] = make_longlong2(o0, o1);
      } else {
        i64* o = (i64*)(O2 + i * 4);
        if (wr[0]) o[0] = o0;
        if (wr[1]) o[1] = o1;
      }
    }
  }
}

static void launch_apply(const ColBatch& b, const i64* mul, const i64* sh, int zero_inactive, const i64* Xi,
                         i64* Xo, cudaStream_t st) {
  dim3 blk;
  int ns;
  slab_shape(b.m, blk, ns);
  if (fx_slab_w(b.m) == FX_SLAB) {
    const dim3 b8(FX_SLAB / 2, 64, 1);
    const int64_t nrb = (b.rows + b8.y - 1) / b8.y;
    const int gx = (int)std::max<int64_t>(1, std::min<int64_t>(nrb, 152 * 8));
    k_fx_apply8<<<dim3(gx, ns, 1), b8, 0, st>>>(b.rows, b.m, b.col2ch, b.meta, mul, sh, zero_inactive, Xi, Xo);
    return;
  }
  const int64_t nrb = (b.rows + blk.y - 1) / blk.y;
  const int gx = (int)std::max<int64_t>(1, std::min<int64_t>(nrb, 152 * 16));
  dim3 grd(gx, ns, 1);
  k_fx_apply<<<grd, blk, 0, st>>>(b.rows, b.m, b.col2ch, b.meta, mul, sh, zero_inactive, Xi, Xo);
}
void launch_fx_normalize(const ColBatch& b, const FxScales& s, const double* invbeta, const i64* W,
                         i64* X, i64* scratch, cudaStream_t st) {
  count_launch_external();
  count_launch_external();
  k_fx_mult<<<nblk_fx(b.nch, 128), 128, 0, st>>>(b.nch, invbeta, s.G, s.F, scratch, scratch + b.nch);
  launch_apply(b, scratch, scratch + b.nch, 1, W, X, st);
}
void launch_fx_rescale(const ColBatch& b, const double* f, int si, int so, const i64* Xi, i64* Xo,
                       i64* scratch, cudaStream_t st) {
  count_launch_external();
  count_launch_external();
  k_fx_mult<<<nblk_fx(b.nch, 128), 128, 0, st>>>(b.nch, f, si, so, scratch, scratch + b.nch);
  launch_apply(b, scratch, scratch + b.nch, 0, Xi, Xo, st);
}

__global__ void k_fx_psi_accum(int64_t n, const double* s, int k, const i64* X, i64* psi) {
  const i64 sfx = __double2ll_rn(ldexp(s[k], 61));  // |s| <= 1
  for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < n;
       g += (int64_t)gridDim.x * blockDim.x)
    psi[g] += rshift_round((i128)sfx * X[g], 61);
}
void launch_fx_psi_accum(int64_t n, const double* s, int k, const i64* X, i64* psi, cudaStream_t st) {
  count_launch_external();
  k_fx_psi_accum<<<nblk_fx(n, 256), 256, 0, st>>>(n, s, k, X, psi);
}

__global__ void k_fx_from_double(int64_t n, const double* x, int F, i64* X) {
  for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < n;
       g += (int64_t)gridDim.x * blockDim.x)
    X[g] = __double2ll_rn(ldexp(x[g], F));
}
void launch_fx_from_double(int64_t n, const double* x, int F, i64* X, cudaStream_t st) {
  count_launch_external();
  k_fx_from_double<<<nblk_fx(n, 256), 256, 0, st>>>(n, x, F, X);
}
__global__ void k_fx_to_double(int64_t n, const i64* X, int F, double* x) {
  for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < n;
       g += (int64_t)gridDim.x * blockDim.x)
    x[g] = ldexp((double)X[g], -F);
}
void launch_fx_to_double(int64_t n, const i64* X, int F, double* x, cudaStream_t st) {
  count_launch_external();
  k_fx_to_double<<<nblk_fx(n, 256), 256, 0, st>>>(n, X, F, x);
}


// sum of int128 partials over `rows` rows per column -> double (scale
// 2^-sexp): one warp per column, lanes stride the rows, then an exact
// shuffle tree (the sum is exact, so the order does not matter)
__global__ void k_fx_partial_reduce(int m, int rows, const i64* partial, int sexp, double* out) {
  const int lane = threadIdx.x & 31;
  const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int c = wid; c < m; c += nw) {
    i128 s = 0;
    for (int b = lane; b < rows; b += 32) {
      const u64 lo = (u64)partial[2 * ((int64_t)b * m + c)];
      const i64 hi = partial[2 * ((int64_t)b * m + c) + 1];
      s += (i128)(((unsigned __int128)(u64)hi << 64) | lo);
    }
    u64 lo = (u64)s;
    i64 hi = (i64)(s >> 64);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      const u64 lo2 = __shfl_xor_sync(0xffffffffu, lo, off);
      const i64 hi2 = __shfl_xor_sync(0xffffffffu, hi, off);
      const u64 sl = lo + lo2;
      hi = hi + hi2 + (sl < lo ? 1 : 0);
      lo = sl;
    }
    if (lane == 0) out[c] = i128_to_double((i128)(((unsigned __int128)(u64)hi << 64) | lo), sexp);
  }
}

void launch_fx_partial_reduce(int m, int rows, const i64* partial, int sexp, double* out, cudaStream_t st) {
  count_launch_external();
  k_fx_partial_reduce<<<nblk_fx((int64_t)m * 32, 256), 256, 0, st>>>(m, rows, partial, sexp, out);
}

// W = Y - (afx*X + bfx*Xp) >> sh in place of Y, with the exact int128 partial
// of beta^2 = <W, W> per (block, column); retired chains are left untouched.
__global__ void k_fx_update_dot(int64_t rows, int m, const int* col2ch, const ChainMeta* meta, int sh,
                                const i64* afx, const i64* bfx, int use_b, const i64* X, const i64* Xp,
                                i64* YW, i64* partial) {
  extern __shared__ i128 shq[];
  const int CW = blockDim.x, RB = blockDim.y;
  const int c = blockIdx.y * CW + threadIdx.x;
  i128 s = 0;
  if (c < m) {
    const int ch = col2ch[c];
    if (meta[ch].active) {
      const i64 a = afx[ch], b = use_b ? bfx[ch] : 0;
      const int64_t sb = (int64_t)blockIdx.y * rows * CW + threadIdx.x;
      for (int64_t i = (int64_t)blockIdx.x * RB + threadIdx.y; i < rows; i += (int64_t)gridDim.x * RB) {
        const int64_t g = sb + i * CW;
        i128 p = (i128)a * X[g];
        if (use_b) p += (i128)b * Xp[g];
        const i64 w = YW[g] - rshift_round(p, sh);
        YW[g] = w;
        s += (i128)w * w;
      }
    }
  }
  shq[threadIdx.y * CW + threadIdx.x] = s;
  __syncthreads();
  for (int h = RB / 2; h > 0; h >>= 1) {
    if (threadIdx.y < h) shq[threadIdx.y * CW + threadIdx.x] += shq[(threadIdx.y + h) * CW + threadIdx.x];
    __syncthreads();
  }
  if (threadIdx.y == 0 && c < m) {
    const i128 v = shq[threadIdx.x];
    partial[2 * ((int64_t)blockIdx.x * m + c)] = (i64)(u64)v;
    partial[2 * ((int64_t)blockIdx.x * m + c) + 1] = (i64)(v >> 64);
  }
}
// The same on 8-column slabs with 16-byte accesses: thread (tx, ty) owns
// columns 2tx, 2tx+1 of slab blockIdx.y and rows ty, ty + 64, ... of its
// block's stride; a warp moves 8 rows x 64 bytes per access.  Retired chains
// and pad columns get zero coefficients (W = YW, untouched) and no beta^2
// contribution.
#define FXU_RB 64
__global__ void __launch_bounds__(256) k_fx_update_dot8(int64_t rows, int m, const int* col2ch,
                                                        const ChainMeta* meta, int sh, const i64* afx,
                                                        const i64* bfx, int use_b, const i64* X, const i64* Xp,
                                                        i64* YW, i64* partial) {
  __shared__ i128 red[FXU_RB][FX_SLAB];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int c0 = blockIdx.y * FX_SLAB + 2 * tx;
  i64 a[2] = {0, 0}, bb[2] = {0, 0};
  bool act[2] = {false, false};
#pragma unroll
  for (int j = 0; j < 2; j++) {
    const int c = c0 + j;
    if (c < m) {
      const int ch = col2ch[c];
      act[j] = meta[ch].active != 0;
      if (act[j]) { a[j] = afx[ch]; bb[j] = use_b ? bfx[ch] : 0; }
    }
  }
  const int64_t sb = (int64_t)blockIdx.y * rows * (FX_SLAB / 2) + tx;  // longlong2 units
  const longlong2* X2 = (const longlong2*)X + sb;
  const longlong2* P2 = (const longlong2*)Xp + sb;
  longlong2* Y2 = (longlong2*)YW + sb;
  i128 s0 = 0, s1 = 0;
  const int64_t stride = (int64_t)gridDim.x * FXU_RB;
  for (int64_t i = (int64_t)blockIdx.x * FXU_RB + ty; i < rows; i += 2 * stride) {
    const int64_t i2 = i + stride;
    const bool two = i2 < rows;
    const longlong2 xa = X2[i * 4], ya = Y2[i * 4];
    const longlong2 pa = use_b ? P2[i * 4] : make_longlong2(0, 0);
    longlong2 xb = make_longlong2(0, 0), yb = make_longlong2(0, 0), pb = make_longlong2(0, 0);
    if (two) {
      xb = X2[i2 * 4];
      yb = Y2[i2 * 4];
      if (use_b) pb = P2[i2 * 4];
    }
    const i64 w0 = ya.x - rshift_round((i128)a[0] * xa.x + (i128)bb[0] * pa.x, sh);
    const i64 w1 = ya.y - rshift_round((i128)a[1] * xa.y + (i128)bb[1] * pa.y, sh);
    Y2[i * 4] = make_longlong2(w0, w1);
    s0 += (i128)w0 * w0;
    s1 += (i128)w1 * w1;
    if (two) {
      const i64 v0 = yb.x - rshift_round((i128)a[0] * xb.x + (i128)bb[0] * pb.x, sh);
      const i64 v1 = yb.y - rshift_round((i128)a[1] * xb.y + (i128)bb[1] * pb.y, sh);
      Y2[i2 * 4] = make_longlong2(v0, v1);
      s0 += (i128)v0 * v0;
      s1 += (i128)v1 * v1;
    }
  }
  red[ty][2 * tx] = act[0] ? s0 : (i128)0;
  red[ty][2 * tx + 1] = act[1] ? s1 : (i128)0;
  __syncthreads();
  for (int h = FXU_RB / 2; h > 0; h >>= 1) {
    if (ty < h) {
      red[ty][2 * tx] += red[ty + h][2 * tx];
      red[ty][2 * tx + 1] += red[ty + h][2 * tx + 1];
    }
    __syncthreads();
  }
  if (ty == 0) {
#pragma unroll
    for (int j = 0; j < 2; j++) {
      const int c = c0 + j;
      if (c < m) {
        const i128 v = red[0][2 * tx + j];
        partial[2 * ((int64_t)blockIdx.x * m + c)] = (i64)(u64)v;
        partial[2 * ((int64_t)blockIdx.x * m + c) + 1] = (i64)(v >> 64);
      }
    }
  }
}

void launch_fx_update_dot(const ColBatch& b, const FxScales& s, const i64* afx, const i64* bfx, bool use_b,
                          const i64* X, const i64* Xp, i64* YW, i64* partial, int nblk, double* out_col,
                          cudaStream_t st) {
  count_launch_external();
  dim3 blk;
  int ns;
  slab_shape(b.m, blk, ns);
  dim3 grd(nblk, ns, 1);
  if (fx_slab_w(b.m) == FX_SLAB)
    k_fx_update_dot8<<<grd, dim3(FX_SLAB / 2, FXU_RB, 1), 0, st>>>(b.rows, b.m, b.col2ch, b.meta,
                                                                    s.C + s.F - s.G, afx, bfx, use_b ? 1 : 0, X,
                                                                    Xp, YW, partial);
  else
    k_fx_update_dot<<<grd, blk, sizeof(i128) * 256, st>>>(b.rows, b.m, b.col2ch, b.meta, s.C + s.F - s.G, afx,
                                                          bfx, use_b ? 1 : 0, X, Xp, YW, partial);
  launch_fx_partial_reduce(b.m, nblk, partial, 2 * s.G, out_col, st);
}


// start vector in fixed point: R_i = round(v_i * 2^40) with v_i the
// splitmix64 value of (seed, sector, index) in [-1, 1)
__global__ void k_fx_start_raw(int64_t n, uint64_t seed, int isector, i64* R) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    uint64_t z = seed + 0xD1B54A32D192ED03ull * (uint64_t)isector + (uint64_t)i + 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z = z ^ (z >> 31);
    const double v = (double)(z >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0;
    R[i] = __double2ll_rn(ldexp(v, 40));
  }
}
void launch_fx_start_raw(int64_t n, uint64_t seed, int isector, i64* R, cudaStream_t st) {
  count_launch_external();
  k_fx_start_raw<<<nblk_fx(n, 256), 256, 0, st>>>(n, seed, isector, R);
}


// ---------------------------------------------------------------------------
// Packed hop words and the warp-per-row H x v for column batches.
// ---------------------------------------------------------------------------
__global__ void k_fx_pack(int64_t n, const int* src, const double2* amp, const double* classes, int K,
                          unsigned* hop) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const double a = amp[t].x;
    const double mag = fabs(a);
    unsigned cls = 0;
    for (int k = 0; k < K; k++)
      if (classes[k] == mag) cls = (unsigned)k;
    hop[t] = ((unsigned)src[t] & 0xFFFFFFu) | (cls << 24) | (a < 0.0 ? 0x80000000u : 0u);
  }
}
void launch_fx_pack(int dim, int width, const int* src, const double2* amp, const double* classes, int K,
                    unsigned* hop, cudaStream_t st) {
  count_launch_external();
  const int64_t n = (int64_t)dim * width;
  if (n == 0) return;
  k_fx_pack<<<nblk_fx(n, 256), 256, 0, st>>>(n, src, amp, classes, K, hop);
}

// In-place partition of each row's hop words, positive amplitudes first;
// npos[row] = their count.  The fixed-point sums are exact, so the order of
// a row's hops does not change any result.
__global__ void k_fx_sign_sort(int dim, int width, const int* cnt, unsigned* hop, int* npos) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= dim) return;
  int i = 0, j = cnt[r] - 1;
  while (i <= j) {
    const unsigned a = hop[r + (int64_t)i * dim];
    if (!(a >> 31)) { i++; continue; }
    const unsigned b = hop[r + (int64_t)j * dim];
    hop[r + (int64_t)i * dim] = b;
    hop[r + (int64_t)j * dim] = a;
    j--;
  }
  npos[r] = i;
}
void launch_fx_sign_sort(int dim, int width, const int* cnt, unsigned* hop, int* npos, cudaStream_t st) {
  if (dim == 0) return;
  count_launch_external();
  k_fx_sign_sort<<<(dim + 127) / 128, 128, 0, st>>>(dim, width, cnt, hop, npos);
}

__global__ void k_fx_perm_tables(int dim, int width, const int* perm, const int* pinv, const unsigned* hop,
                                 const int* cnt, const int* npos, const int* words, const i64* e1, unsigned* phop,
                                 unsigned* rhop, int* pcnt, int* pnpos, int* pword, i64* pe1) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= dim) return;
  const int r = perm[i];
  pcnt[i] = cnt[r];
  pnpos[i] = npos[r];
  pword[i] = words[r];
  pe1[i] = e1[r];
  for (int h = 0; h < width; h++) {  // source as its first swizzled 16-byte unit (see fxs_unit)
    const unsigned hw = hop[(int64_t)h * dim + r];
    const unsigned src = hw & 0xFFFFFFu;
    phop[(int64_t)h * dim + i] = (src * 4u + ((src >> 1) & 3u)) | (hw & 0xFF000000u);
    rhop[(int64_t)h * dim + i] = (h < cnt[r] ? (unsigned)pinv[src] : 0u) | (hw & 0xFF000000u);
  }
}
void launch_fx_perm_tables(int dim, int width, const int* perm, const int* pinv, const unsigned* hop,
                           const int* cnt, const int* npos, const int* words, const i64* e1, unsigned* phop,
                           unsigned* rhop, int* pcnt, int* pnpos, int* pword, i64* pe1, cudaStream_t st) {
  if (dim == 0) return;
  count_launch_external();
  k_fx_perm_tables<<<(dim + 127) / 128, 128, 0, st>>>(dim, width, perm, pinv, hop, cnt, npos, words, e1, phop,
                                                      rhop, pcnt, pnpos, pword, pe1);
}

// accumulate one hop's source row into the class accumulators; the class and
// sign are warp-uniform, so the branches do not diverge.  xr points at the
// source row's first column within slab 0; coff[q] adds lane column q's slab
// offset.
template <int K, int NCQ>
__device__ __forceinline__ void hop_row(i64 (&S)[K][NCQ], unsigned hw, const i64* __restrict__ xr,
                                        const int64_t (&coff)[NCQ], int lim) {
  const int cls = (K == 1) ? 0 : (int)((hw >> 24) & 3u);
  const bool neg = hw >> 31;
#pragma unroll
  for (int k = 0; k < K; k++) {
    if (k != cls) continue;
    if (neg) {
#pragma unroll
      for (int q = 0; q < NCQ; q++)
        if (32 * q < lim) S[k][q] -= xr[coff[q]];
    } else {
#pragma unroll
      for (int q = 0; q < NCQ; q++)
        if (32 * q < lim) S[k][q] += xr[coff[q]];
    }
  }
}

// Column-batch H x v, warp form: one warp per row and 128 columns (4 per
// lane) per CTA column slice (blockIdx.y), hop word decoded once per row and
// slice.  Rows of 8-column slabs: lane column c of row r sits at
// r*8 + (c/8)*8*D + c%8.
// MODE 1: diagonal + up hops, rows in idw-major order (a column block's up
//         neighbours are the rows in flight: L2 resident).
// MODE 2: down hops added into Y, rows in iup-major order (a slab's down
//         neighbours stay in L2); with apart != nullptr it also forms the
//         exact int128 partials of alpha = <X, Y> per (row block, column).
#define FXW_NCQ 4
template <int K, int MODE>
__global__ void __launch_bounds__(256) k_hxv_fx_w(SectorView sv, FxView fv, int m, const i64* __restrict__ X,
                                                  i64* __restrict__ Y, i64* __restrict__ apart) {
  constexpr int NCQ = FXW_NCQ, W = FX_SLAB;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int wid = blockIdx.x * (blockDim.x >> 5) + warp;
  const int nw = gridDim.x * (blockDim.x >> 5);
  const int c0 = blockIdx.y * 32 * NCQ;
  const int lim = m - c0 - lane;  // column c0 + lane + 32q exists while 32q < lim
  const int DU = sv.dimup, DD = sv.dimdw;
  const int D = DU * DD;
  int64_t coff[NCQ];
#pragma unroll
  for (int q = 0; q < NCQ; q++) {
    const int c = c0 + lane + 32 * q;
    coff[q] = (int64_t)(c / W) * W * D + (c % W);
  }
  i128 adot[NCQ];
#pragma unroll
  for (int q = 0; q < NCQ; q++) adot[q] = 0;
  for (int rr = wid; rr < D; rr += nw) {
    int idw, iup;
    if (MODE == 2) { iup = rr / DD; idw = rr - iup * DD; }
    else { idw = rr / DU; iup = rr - idw * DU; }
    const int r = iup + idw * DU;
    i64 dfx = 0;
    if (MODE != 2)
      dfx = fv.up_e1[iup] + fv.dw_e1[idw] + mixed_fx(fv, (unsigned)sv.up_words[iup], (unsigned)sv.dw_words[idw]);
    const int nu = (MODE == 2) ? 0 : sv.up_cnt[iup];
    const int nd = (MODE == 1) ? 0 : sv.dw_cnt[idw];
    const int colbase = idw * DU;
    i64 S[K][NCQ];
#pragma unroll
    for (int k = 0; k < K; k++)
#pragma unroll
      for (int q = 0; q < NCQ; q++) S[k][q] = 0;
    for (int h = 0, o = iup; h < nu; h++, o += DU) {
      const unsigned hw = fv.up_hop[o];
      hop_row<K, NCQ>(S, hw, X + (int64_t)(colbase + (int)(hw & 0xFFFFFFu)) * W, coff, lim);
    }
    for (int h = 0, o = idw; h < nd; h++, o += DD) {
      const unsigned hw = fv.dw_hop[o];
      hop_row<K, NCQ>(S, hw, X + (int64_t)(iup + (int)(hw & 0xFFFFFFu) * DU) * W, coff, lim);
    }
    const i64* xo = X + (int64_t)r * W;
    i64* yo = Y + (int64_t)r * W;
#pragma unroll
    for (int q = 0; q < NCQ; q++) {
      if (32 * q < lim) {
        i128 p = 0;
        if (MODE != 2) p = (i128)dfx * xo[coff[q]];
#pragma unroll
        for (int k = 0; k < K; k++) p += (i128)fv.afx[k] * S[k][q];
        i64 y = rshift_round(p, fv.shift);
        if (MODE == 2) {
          y += yo[coff[q]];
          if (apart) adot[q] += (i128)xo[coff[q]] * y;
        }
        yo[coff[q]] = y;
      }
    }
  }
  if (MODE == 2 && apart) {  // block reduction of the alpha partials per column
    __shared__ i128 red[8][32 * FXW_NCQ];
#pragma unroll
    for (int q = 0; q < NCQ; q++) red[warp][lane + 32 * q] = adot[q];
    __syncthreads();
    for (int t = threadIdx.x; t < 32 * NCQ; t += blockDim.x) {
      i128 sum = 0;
      for (int w = 0; w < (int)(blockDim.x >> 5); w++) sum += red[w][t];
      const int c = c0 + t;
      if (c < m) {
        const int64_t o2 = 2 * ((int64_t)blockIdx.x * m + c);
        apart[o2] = (i64)(u64)sum;
        apart[o2 + 1] = (i64)(sum >> 64);
      }
    }
  }
}

// grid.x row blocks of the warp form (its alpha partial rows)
int hxv_fx_w_rowblocks(int64_t D) { return nblk_fx(D * 32, 256, 152 * 6); }

void launch_hxv_fx_w(const SectorView& sv, const FxView& fv, int m, const i64* X, i64* Y, i64* apart,
                     cudaStream_t st) {
  const int64_t D = (int64_t)sv.dimup * sv.dimdw;
  dim3 grd(hxv_fx_w_rowblocks(D), (m + 32 * FXW_NCQ - 1) / (32 * FXW_NCQ), 1);
#define VCA_W(KK)                                                              \
  do {                                                                         \
    count_launch_external();                                                   \
    count_launch_external();                                                   \
    k_hxv_fx_w<KK, 1><<<grd, 256, 0, st>>>(sv, fv, m, X, Y, nullptr);          \
    k_hxv_fx_w<KK, 2><<<grd, 256, 0, st>>>(sv, fv, m, X, Y, apart);            \
  } while (0)
  switch (fv.K) {
    case 1: VCA_W(1); break;
    case 2: VCA_W(2); break;
    case 3: VCA_W(3); break;
    default: VCA_W(4); break;
  }
#undef VCA_W
}

// Column-batch H x v, staged form, for sectors whose up-spin block of one
// slab fits shared memory.  One CTA per (slab cs, down configuration idw);
// the slab is the slow grid index, so the CTAs in flight all work in one
// slab (D*64 bytes, 47 MB for the 4x3 cluster's largest chain sectors: L2
// resident).  The CTA's rows are the DimUp rows idw*DimUp + iup, one
// contiguous block of X.  Three phases:
//  1. down hops: the hop list of idw is the same for every row of the CTA,
//     so the down part is a signed sum of whole blocks X[idw'] -- streamed
//     with coalesced 16-byte loads into a shared accumulator (exact int64
//     sums per class for K = 1, the exact int128 sum_k a_k S_k for K > 1);
//     the CTA's own block is copied into shared memory alongside.
//  2. up hops and diagonal: two lanes per row, four columns each (16-byte
//     units q and q+2 of the row), sixteen rows per warp taken in order of
//     their up-hop count (fv.up_perm) with their tables read in that order
//     (fv.up_p*); hop lists are sign sorted, so the inner loops are plain
//     64-bit adds or subtracts; every source row is a shared-memory read.
//     y = round((d x + sum_k a_k S_k) 2^-shift) overwrites the accumulator.
//  3. Y streams out with coalesced 16-byte stores; with apart != nullptr the
//     exact int128 alpha partials <X,Y> of the CTA's columns go to row idw.
// The 16-byte units of a staged row are XOR-swizzled by (row >> 1) & 3 so
// random rows spread over the banks.  Pad columns (>= m) of X are zero, so
// those of Y come out zero.
__device__ __forceinline__ int fxs_unit(int row, int j) { return row * 4 + (j ^ ((row >> 1) & 3)); }


template <int K>
__global__ void __launch_bounds__(512, 2) k_hxv_fx_s(SectorView sv, FxView fv, int m, const i64* __restrict__ X,
                                                     i64* __restrict__ Y, i64* __restrict__ apart) {
  extern __shared__ __align__(16) unsigned char fxs_smem[];
  constexpr int W = FX_SLAB, RPW = 16;
  const int DU = sv.dimup, DD = sv.dimdw;
  const int64_t D = (int64_t)DU * DD;
  const int npair = DU * 4;                                 // 16-byte units per block
  longlong2* xs2 = (longlong2*)fxs_smem;                   // [DU][4] X block (swizzled)
  longlong2* ac2 = xs2 + npair;                            // [DU][4] down sums, then y
  longlong2* ah2 = ac2 + npair;                            // [DU][4] high words (K > 1 only)
  int64_t* doff = (int64_t*)(ah2 + (K > 1 ? npair : 0));   // idw's down hops: element offsets
  unsigned char* dcl = (unsigned char*)(doff + sv.wdw);    // and classes
  const int cs = blockIdx.x / DD;
  const int idw = blockIdx.x - cs * DD;
  const int c0 = cs * W;
  const long long* Xs = (const long long*)X + (int64_t)cs * D * W;  // this slab
  long long* Ys = (long long*)Y + (int64_t)cs * D * W;
  const int64_t rowbase = (int64_t)idw * DU;
  const int nd = sv.dw_cnt[idw];
  const int ndp = fv.dw_npos[idw];
  for (int h = threadIdx.x; h < nd; h += blockDim.x) {
    const unsigned hw = fv.dw_hop[idw + h * DD];
    doff[h] = (int64_t)(hw & 0xFFFFFFu) * DU * W;
    dcl[h] = (unsigned char)((hw >> 24) & 3u);
  }
  __syncthreads();
  // ---- phase 1: own block to shared memory, down blocks summed -----------
  // each thread sums P1 units t, t + blockDim, ... per hop list pass
  {
    constexpr int FXS_P1 = (K == 1) ? 4 : 2;
    const longlong2* xb = (const longlong2*)Xs;
    const longlong2* own = xb + rowbase * (W / 2);
    for (int t0 = threadIdx.x; t0 < npair; t0 += FXS_P1 * blockDim.x) {
      u64 S[K][FXS_P1][2];
#pragma unroll
      for (int k = 0; k < K; k++)
#pragma unroll
        for (int e = 0; e < FXS_P1; e++) S[k][e][0] = S[k][e][1] = 0;
      const bool full = t0 + (FXS_P1 - 1) * (int)blockDim.x < npair;
      for (int h = 0; h < nd; h++) {
        const longlong2* src = xb + (doff[h] >> 1) + t0;
        const int cls = (K == 1) ? 0 : (int)dcl[h];
        longlong2 v[FXS_P1];
#pragma unroll
        for (int e = 0; e < FXS_P1; e++)
          v[e] = (full || t0 + e * (int)blockDim.x < npair) ? __ldcg(src + e * blockDim.x) : make_longlong2(0, 0);
        if (h < ndp) {
#pragma unroll
          for (int k = 0; k < K; k++)
            if (k == cls)
#pragma unroll
              for (int e = 0; e < FXS_P1; e++) { S[k][e][0] += (u64)v[e].x; S[k][e][1] += (u64)v[e].y; }
        } else {
#pragma unroll
          for (int k = 0; k < K; k++)
            if (k == cls)
#pragma unroll
              for (int e = 0; e < FXS_P1; e++) { S[k][e][0] -= (u64)v[e].x; S[k][e][1] -= (u64)v[e].y; }
        }
      }
#pragma unroll
      for (int e = 0; e < FXS_P1; e++) {
        const int t = t0 + e * blockDim.x;
        if (t >= npair) break;
        const int su = fxs_unit(t >> 2, t & 3);
        xs2[su] = __ldcg(own + t);
        if (K == 1) {
          ac2[su] = make_longlong2((long long)S[0][e][0], (long long)S[0][e][1]);
        } else {
          i128 p0 = 0, p1 = 0;
#pragma unroll
          for (int k = 0; k < K; k++) {
            p0 += (i128)fv.afx[k] * (i64)S[k][e][0];
            p1 += (i128)fv.afx[k] * (i64)S[k][e][1];
          }
          ac2[su] = make_longlong2((long long)(u64)p0, (long long)(u64)p1);
          ah2[su] = make_longlong2((long long)(p0 >> 64), (long long)(p1 >> 64));
        }
      }
    }
  }
  __syncthreads();
  // ---- phase 2: up hops and diagonal, y into the accumulator -------------
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  {
    const int sub = lane >> 1, q = lane & 1;  // units q and q+2: columns 2q,2q+1,2q+4,2q+5
    const i64 e1d = fv.dw_e1[idw];
    const unsigned wdw = (unsigned)sv.dw_words[idw];
    for (int i = warp * RPW + sub; i < DU; i += nwarp * RPW) {
      const int iup = fv.up_perm[i];
      u64 S[K][4];
#pragma unroll
      for (int k = 0; k < K; k++)
#pragma unroll
        for (int j = 0; j < 4; j++) S[k][j] = 0;
      const int nu = fv.up_pcnt[i];
      const int nup = fv.up_pnpos[i];
      // table entries hold fxs_unit(src, 0); units q and q+2 are that ^ q and ^ (q|2)
      int h = 0, o = i;
#pragma unroll 2
      for (; h < nup; h++, o += DU) {
        const unsigned hw = fv.up_phop[o];
        const int ua = (int)(hw & 0xFFFFFFu) ^ q;
        const longlong2 a = xs2[ua], b2 = xs2[ua ^ 2];
        const int cls = (K == 1) ? 0 : (int)((hw >> 24) & 3u);
#pragma unroll
        for (int k = 0; k < K; k++)
          if (k == cls) { S[k][0] += a.x; S[k][1] += a.y; S[k][2] += b2.x; S[k][3] += b2.y; }
      }
#pragma unroll 2
      for (; h < nu; h++, o += DU) {
        const unsigned hw = fv.up_phop[o];
        const int ua = (int)(hw & 0xFFFFFFu) ^ q;
        const longlong2 a = xs2[ua], b2 = xs2[ua ^ 2];
        const int cls = (K == 1) ? 0 : (int)((hw >> 24) & 3u);
#pragma unroll
        for (int k = 0; k < K; k++)
          if (k == cls) { S[k][0] -= a.x; S[k][1] -= a.y; S[k][2] -= b2.x; S[k][3] -= b2.y; }
      }
      const int ua = fxs_unit(iup, q), ub = fxs_unit(iup, q + 2);
      const longlong2 xa = xs2[ua], xb = xs2[ub];
      const i64 x0[4] = {xa.x, xa.y, xb.x, xb.y};
      const longlong2 da = ac2[ua], db = ac2[ub];
      const i64 dlo[4] = {da.x, da.y, db.x, db.y};
      i64 dhi[4] = {0, 0, 0, 0};
      if (K > 1) {
        const longlong2 ha = ah2[ua], hb = ah2[ub];
        dhi[0] = ha.x; dhi[1] = ha.y; dhi[2] = hb.x; dhi[3] = hb.y;
      }
      const i64 dfx = fv.up_pe1[i] + e1d + mixed_fx(fv, (unsigned)fv.up_pword[i], wdw);
      i64 y[4];
#pragma unroll
      for (int j = 0; j < 4; j++) {
        i128 p = (i128)dfx * x0[j];
        if (K == 1) {
          p += (i128)fv.afx[0] * (i64)(S[0][j] + (u64)dlo[j]);
        } else {
#pragma unroll
          for (int k = 0; k < K; k++) p += (i128)fv.afx[k] * (i64)S[k][j];
          p += (i128)(((unsigned __int128)(u64)dhi[j] << 64) | (u64)dlo[j]);
        }
        y[j] = rshift_round(p, fv.shift);
      }
      ac2[ua] = make_longlong2(y[0], y[1]);
      ac2[ub] = make_longlong2(y[2], y[3]);
    }
  }
  __syncthreads();
  // ---- phase 3: Y out, alpha partials -------------------------------------
  {
    longlong2* yb = (longlong2*)Ys + rowbase * (W / 2);
    i128 ad0 = 0, ad1 = 0;  // columns 2u, 2u+1 with u = threadIdx.x & 3
    for (int t = threadIdx.x; t < npair; t += blockDim.x) {
      const int su = fxs_unit(t >> 2, t & 3);
      const longlong2 yv = ac2[su];
      __stcs(yb + t, yv);
      if (apart) {
        const longlong2 xv = xs2[su];
        ad0 += (i128)xv.x * yv.x;
        ad1 += (i128)xv.y * yv.y;
      }
    }
    if (apart) {
      __shared__ i128 red[16][W];
      const int u = lane & 3;
      i128 adv[2] = {ad0, ad1};
#pragma unroll
      for (int j = 0; j < 2; j++) {
        u64 lo = (u64)adv[j];
        i64 hi = (i64)(adv[j] >> 64);
#pragma unroll
        for (int off = 4; off < 32; off <<= 1) {  // lanes holding the same columns
          const u64 lo2 = __shfl_xor_sync(0xffffffffu, lo, off);
          const i64 hi2 = __shfl_xor_sync(0xffffffffu, hi, off);
          const u64 sl = lo + lo2;
          hi = hi + hi2 + (sl < lo ? 1 : 0);
          lo = sl;
        }
        if (lane < 4) red[warp][2 * u + j] = ((i128)hi << 64) | (i128)lo;
      }
      __syncthreads();
      if ((int)threadIdx.x < W && c0 + (int)threadIdx.x < m) {
        i128 sum = 0;
        for (int w = 0; w < nwarp; w++) sum += red[w][threadIdx.x];
        const int64_t o2 = 2 * ((int64_t)idw * m + c0 + threadIdx.x);
        apart[o2] = (i64)(u64)sum;
        apart[o2 + 1] = (i64)(sum >> 64);
      }
    }
  }
}

// Column-batch H x v, position-ordered form, for chain batches whose rows
// of the fast spin role are stored in up_perm order (row p + idw*DimUp holds
// up configuration up_perm[p]; fv.rows_permuted == 1).  One CTA per (slab
// cs, down configuration idw), 256 threads.  A lane owns 16-byte unit u
// (columns 2u, 2u+1) of rows p and p+8 of its warp's group of sixteen
// consecutive positions, so one mapping serves all three parts:
//  * down hops: rows p of the neighbour blocks X[idw'] (the hop list of idw
//    is the same for every row) -- coalesced 512-byte loads, summed in
//    registers;
//  * up hops: sources are positions (fv.up_rhop) in the shared-memory copy
//    of the CTA's own block; the sixteen rows of a warp have nearly equal
//    hop counts (decreasing order), and hop lists are sign sorted;
//  * Y rows and the exact int128 alpha partials of unit u -- coalesced
//    stores, partials in registers.
// Only the own-block copy needs a barrier; shared memory is one block
// (DimUp*64 bytes), so four CTAs share an SM on the 4x3 chain sectors.
#define FXR_THREADS 256

// ---- bulk copy of the own block (cp.async.bulk, mbarrier completion) ----
// A bounded wait that runs out adds 1 to g_fx_wait_fail, which the solve and
// the timed H x v turn into VCA_ERR_TIMEOUT; g_fx_stage_extra_tx (a test
// hook, 0 otherwise) raises the bytes the barrier expects above those
// copied, so that the wait runs out without any fault.
__device__ int g_fx_wait_fail = 0;
__device__ int g_fx_stage_extra_tx = 0;
#define FXB_WAIT_NS 1000000000ull
__device__ __forceinline__ uint64_t fxb_time() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ bool fxb_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ bool fxb_wait_bounded(uint32_t bar, uint32_t parity) {
  const uint64_t t0 = fxb_time();
  while (!fxb_try_wait(bar, parity))
    if (fxb_time() - t0 > FXB_WAIT_NS) return false;
  return true;
}
// thread 0: init the barrier, expect the bytes, start the copy
__device__ __forceinline__ void fxb_start(uint32_t bar, uint32_t dst, const void* src, uint32_t bytes) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(1u) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  const uint32_t expect = bytes + (uint32_t)g_fx_stage_extra_tx;
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(expect) : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}
template <int K, bool SH63, bool APART>
__global__ void __launch_bounds__(FXR_THREADS, 4) k_hxv_fx_r(SectorView sv, FxView fv, int m,
                                                              const i64* __restrict__ X, i64* __restrict__ Y,
                                                              i64* __restrict__ apart) {
  extern __shared__ __align__(16) unsigned char fxr_smem[];
  constexpr int W = FX_SLAB;
  const int DU = sv.dimup, DD = sv.dimdw;
  const int64_t D = (int64_t)DU * DD;
  longlong2* xs2 = (longlong2*)fxr_smem;                // [DU][4] own block, position order
  unsigned long long* sbar = (unsigned long long*)(xs2 + (size_t)DU * 4);  // its copy's mbarrier (16-byte slot)
  int* doff = (int*)(sbar + 2);                        // down hops: offsets in 16-byte units
  unsigned char* dcl = (unsigned char*)(doff + sv.wdw);
  const int cs = blockIdx.x / DD;
  const int idw = blockIdx.x - cs * DD;
  const int c0 = cs * W;
  const int64_t rowbase = (int64_t)idw * DU;
  const longlong2* own = (const longlong2*)X + (int64_t)cs * D * (W / 2) + rowbase * 4;
  longlong2* yown = (longlong2*)Y + (int64_t)cs * D * (W / 2) + rowbase * 4;
  const int nd = sv.dw_cnt[idw];
  const int ndp = fv.dw_npos[idw];
  // the own block (DU x 64 contiguous bytes) by one bulk copy, the down-hop
  // table meanwhile; thread 0 waits (bounded) and the CTA follows its outcome
  __shared__ int stage_ok;
  const uint32_t bar_s = (uint32_t)__cvta_generic_to_shared(sbar);
  if (threadIdx.x == 0)
    fxb_start(bar_s, (uint32_t)__cvta_generic_to_shared(xs2), own, (uint32_t)DU * 64u);
  for (int h = threadIdx.x; h < nd; h += blockDim.x) {
    const unsigned hw = fv.dw_hop[idw + h * DD];
    doff[h] = ((int)(hw & 0xFFFFFFu) - idw) * DU * 4;  // neighbour block relative to own (|.| < D*4 < 2^31)
    dcl[h] = (unsigned char)((hw >> 24) & 3u);
  }
  if (threadIdx.x == 0) {
    const bool ok = fxb_wait_bounded(bar_s, 0);
    if (!ok) {
      atomicAdd(&g_fx_wait_fail, 1);
      fxb_wait_bounded(bar_s, 0);  // the copy's bytes in flight, again bounded
    }
    stage_ok = ok ? 1 : 0;
  }
  __syncthreads();
  if (!stage_ok) return;  // uniform: no later barrier is reached by part of the CTA
  for (int it = 0; it < (1 << 16) && !fxb_try_wait(bar_s, 0); it++) {
  }  // the phase is complete: this thread's acquire of the copied bytes
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  const int u = lane & 3, rsub = lane >> 2;
  const i64 e1d = fv.dw_e1[idw];
  const unsigned wdw = (unsigned)sv.dw_words[idw];
  i128 ad0 = 0, ad1 = 0;
  for (int pb = warp * 16; pb < DU; pb += nwarp * 16) {
    const int pr0 = pb + rsub, pr1 = pb + 8 + rsub;
    const bool ok0 = pr0 < DU, ok1 = pr1 < DU;
    u64 S[K][2][2];
#pragma unroll
    for (int k = 0; k < K; k++) S[k][0][0] = S[k][0][1] = S[k][1][0] = S[k][1][1] = 0;
    // down hops: rows pr0, pr1 of the neighbour blocks
    // (a row past the block end reads row 0 of the same neighbour block, in
    // bounds, and is never stored)
    const longlong2* a0 = own + (ok0 ? pr0 : 0) * 4 + u;
    const longlong2* a1 = own + (ok1 ? pr1 : 0) * 4 + u;
    int h = 0;
#pragma unroll 2
    for (; h < ndp; h++) {  // hop lists are sign sorted: positive amplitudes first
      const int o = doff[h];
      const longlong2 v0 = __ldcg(a0 + o), v1 = __ldcg(a1 + o);
      const int cls = (K == 1) ? 0 : (int)dcl[h];
#pragma unroll
      for (int k = 0; k < K; k++)
        if (k == cls) {
          S[k][0][0] += (u64)v0.x; S[k][0][1] += (u64)v0.y; S[k][1][0] += (u64)v1.x; S[k][1][1] += (u64)v1.y;
        }
    }
#pragma unroll 2
    for (; h < nd; h++) {
      const int o = doff[h];
      const longlong2 v0 = __ldcg(a0 + o), v1 = __ldcg(a1 + o);
      const int cls = (K == 1) ? 0 : (int)dcl[h];
#pragma unroll
      for (int k = 0; k < K; k++)
        if (k == cls) {
          S[k][0][0] -= (u64)v0.x; S[k][0][1] -= (u64)v0.y; S[k][1][0] -= (u64)v1.x; S[k][1][1] -= (u64)v1.y;
        }
    }
    // up hops from the shared block, then the diagonal, Y and alpha
#pragma unroll
    for (int j = 0; j < 2; j++) {
      const int p = j ? pr1 : pr0;
      if (p >= DU) continue;
      const int nu = fv.up_pcnt[p];
      const int nup = fv.up_pnpos[p];
      int h = 0, o = p;
#pragma unroll 2
      for (; h < nup; h++, o += DU) {
        const unsigned hw = fv.up_rhop[o];
        const longlong2 v = xs2[(int)(hw & 0xFFFFFFu) * 4 + u];
        const int cls = (K == 1) ? 0 : (int)((hw >> 24) & 3u);
#pragma unroll
        for (int k = 0; k < K; k++)
          if (k == cls) { S[k][j][0] += (u64)v.x; S[k][j][1] += (u64)v.y; }
      }
#pragma unroll 2
      for (; h < nu; h++, o += DU) {
        const unsigned hw = fv.up_rhop[o];
        const longlong2 v = xs2[(int)(hw & 0xFFFFFFu) * 4 + u];
        const int cls = (K == 1) ? 0 : (int)((hw >> 24) & 3u);
#pragma unroll
        for (int k = 0; k < K; k++)
          if (k == cls) { S[k][j][0] -= (u64)v.x; S[k][j][1] -= (u64)v.y; }
      }
      const longlong2 x = xs2[p * 4 + u];
      const i64 dfx = fv.up_pe1[p] + e1d + mixed_fx(fv, (unsigned)fv.up_pword[p], wdw);
      i128 q0 = (i128)dfx * x.x, q1 = (i128)dfx * x.y;
#pragma unroll
      for (int k = 0; k < K; k++) {
        q0 += (i128)fv.afx[k] * (i64)S[k][j][0];
        q1 += (i128)fv.afx[k] * (i64)S[k][j][1];
      }
      const i64 y0 = SH63 ? rshift_round63(q0, fv.shift) : rshift_round(q0, fv.shift);
      const i64 y1 = SH63 ? rshift_round63(q1, fv.shift) : rshift_round(q1, fv.shift);
      __stcs(yown + p * 4 + u, make_longlong2(y0, y1));
      if (APART) {
        if (c0 + 2 * u < m) ad0 += (i128)x.x * y0;
        if (c0 + 2 * u + 1 < m) ad1 += (i128)x.y * y1;
      }
    }
  }
  if (APART) {
    __shared__ i128 red[FXR_THREADS / 32][W];
    i128 adv[2] = {ad0, ad1};
#pragma unroll
    for (int j = 0; j < 2; j++) {
      u64 lo = (u64)adv[j];
      i64 hi = (i64)(adv[j] >> 64);
#pragma unroll
      for (int off = 4; off < 32; off <<= 1) {  // lanes holding the same columns
        const u64 lo2 = __shfl_xor_sync(0xffffffffu, lo, off);
        const i64 hi2 = __shfl_xor_sync(0xffffffffu, hi, off);
        const u64 sl = lo + lo2;
        hi = hi + hi2 + (sl < lo ? 1 : 0);
        lo = sl;
      }
      if (lane < 4) red[warp][2 * u + j] = ((i128)hi << 64) | (i128)lo;
    }
    __syncthreads();
    if ((int)threadIdx.x < W && c0 + (int)threadIdx.x < m) {
      i128 sum = 0;
      for (int w = 0; w < nwarp; w++) sum += red[w][threadIdx.x];
      const int64_t o2 = 2 * ((int64_t)idw * m + c0 + threadIdx.x);
      apart[o2] = (i64)(u64)sum;
      apart[o2 + 1] = (i64)(sum >> 64);
    }
  }
}

#define FXR_SMEM_MAX (200 * 1024)
static size_t hxv_fx_r_smem(const SectorView& sv) {
  return (size_t)sv.dimup * FX_SLAB * sizeof(i64) + 16 + (size_t)sv.wdw * 5 + 16;
}

int fx_take_wait_failures() {
  int v = 0;
  if (cudaMemcpyFromSymbol(&v, g_fx_wait_fail, sizeof(int)) != cudaSuccess) return -1;
  if (v) {
    const int z = 0;
    cudaMemcpyToSymbol(g_fx_wait_fail, &z, sizeof(int));
  }
  return v;
}
int fx_set_stage_extra_tx(int bytes) {
  return cudaMemcpyToSymbol(g_fx_stage_extra_tx, &bytes, sizeof(int)) == cudaSuccess ? 0 : -1;
}

bool hxv_fx_r_ok(const SectorView& sv, const FxView& fv, int m) {
  return fv.up_rhop && fv.up_pcnt && fv.dw_npos && fv.K <= 2 && m >= 16 && hxv_fx_r_smem(sv) <= FXR_SMEM_MAX &&
         (int64_t)sv.dimdw * ((m + FX_SLAB - 1) / FX_SLAB) < ((int64_t)1 << 31) &&
         (int64_t)sv.dimup * sv.dimdw * 4 < ((int64_t)1 << 31);
}

template <int K, bool SH63, bool APART>
static void launch_hxv_fx_r_t(const SectorView& sv, const FxView& fv, int m, const i64* X, i64* Y, i64* apart,
                              cudaStream_t st) {
  static bool attr_set = false;  // per instantiation, process-wide (every device is sm_103a)
  if (!attr_set) {
    cudaFuncSetAttribute(k_hxv_fx_r<K, SH63, APART>, cudaFuncAttributeMaxDynamicSharedMemorySize, FXR_SMEM_MAX);
    attr_set = true;
  }
  const int ns = (m + FX_SLAB - 1) / FX_SLAB;
  count_launch_external();
  k_hxv_fx_r<K, SH63, APART><<<sv.dimdw * ns, FXR_THREADS, hxv_fx_r_smem(sv), st>>>(sv, fv, m, X, Y, apart);
}
template <int K>
static void launch_hxv_fx_r_k(const SectorView& sv, const FxView& fv, int m, const i64* X, i64* Y, i64* apart,
                              cudaStream_t st) {
  const bool sh63 = fv.shift >= 1 && fv.shift <= 63;
  if (sh63 && apart) launch_hxv_fx_r_t<K, true, true>(sv, fv, m, X, Y, apart, st);
  else if (sh63) launch_hxv_fx_r_t<K, true, false>(sv, fv, m, X, Y, apart, st);
  else if (apart) launch_hxv_fx_r_t<K, false, true>(sv, fv, m, X, Y, apart, st);
  else launch_hxv_fx_r_t<K, false, false>(sv, fv, m, X, Y, apart, st);
}

#define FXS_THREADS 512
#define FXS_SMEM_MAX (220 * 1024)
static size_t hxv_fx_s_smem(const SectorView& sv, int K) {
  // X block, down sums (and their high words for K > 1), down hop table
  return (size_t)sv.dimup * FX_SLAB * sizeof(i64) * (K > 1 ? 3 : 2) + (size_t)sv.wdw * 9 + 16;
}

static bool hxv_fx_s_ok(const SectorView& sv, const FxView& fv, int m, bool warp_only) {
  return !warp_only && fv.up_perm && fv.up_phop && fv.dw_npos && m >= FX_SLAB &&
         hxv_fx_s_smem(sv, fv.K) <= FXS_SMEM_MAX &&
         (int64_t)sv.dimdw * ((m + FX_SLAB - 1) / FX_SLAB) < ((int64_t)1 << 31);
}

template <int K>
static void launch_hxv_fx_s_k(const SectorView& sv, const FxView& fv, int m, const i64* X, i64* Y, i64* apart,
                              cudaStream_t st) {
  static bool attr_set = false;  // per instantiation, process-wide (every device is sm_103a)
  if (!attr_set) {
    cudaFuncSetAttribute(k_hxv_fx_s<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, FXS_SMEM_MAX);
    attr_set = true;
  }
  const int ns = (m + FX_SLAB - 1) / FX_SLAB;
  count_launch_external();
  k_hxv_fx_s<K><<<sv.dimdw * ns, FXS_THREADS, hxv_fx_s_smem(sv, K), st>>>(sv, fv, m, X, Y, apart);
}

// ---------------------------------------------------------------------------
// Column batches of large sectors whose up block of one slab does not fit
// shared memory: the paired-column forms on 16-byte column pairs of the
// slabs.  Slab s holds columns 8s..8s+7 as rows of 64 bytes, so the four
// 16-byte pairs of a row are four interleaved single-vector problems that
// share the row's diagonal and the up role's bank schedule.
//  * up part (+ diagonal): one CTA per (down configuration, slab, pair),
//    pairs fastest so the four CTAs of one 64-byte row block run together
//    and read its lines once from DRAM; the block's DimUp units are staged
//    and the schedule walked as in k_hxv1_up2.
//  * down part: one CTA per (chunk of FXS_DW_ROWS rows, slab, group of
//    FXS_DW_GRP down configurations), chunk-major so the chunk's rows of
//    every down configuration (FXS_DW_ROWS * DimDw * 64 bytes) stay in L2;
//    four lanes per row, one pair each: a warp reads 512 contiguous bytes
//    of each neighbour block.
// Both halves round their own int128 sums, as the single-vector form does.
// ---------------------------------------------------------------------------
#define FXS_DW_ROWS 64
#define FXS_DW_GRP 8
template <int K>
__global__ void __launch_bounds__(FX1_UP2_THREADS, 1) k_hxv_slab_up2(SectorView sv, FxView fv, int nslab,
                                                                 const i64* __restrict__ X, i64* __restrict__ Y) {
  extern __shared__ __align__(16) unsigned char x1p_smem[];
  longlong2* xs = (longlong2*)x1p_smem;
  const int DU = sv.dimup, DD = sv.dimdw;
  const int pr = blockIdx.x & 3;
  const int rest = blockIdx.x >> 2;
  const int sl = rest % nslab, idw = rest / nslab;
  if (idw >= DD) return;
  const int64_t base = ((int64_t)sl * DU * DD + (int64_t)idw * DU) * 4 + pr;  // 16-byte units
  const longlong2* X2 = (const longlong2*)X + base;
  longlong2* Y2 = (longlong2*)Y + base;
  constexpr int U = 8;
  for (int t0 = threadIdx.x; t0 < DU; t0 += U * FX1_UP2_THREADS) {
    longlong2 a[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int t = t0 + u * FX1_UP2_THREADS;
      a[u] = t < DU ? __ldcg(X2 + (int64_t)t * 4) : make_longlong2(0ll, 0ll);
    }
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int t = t0 + u * FX1_UP2_THREADS;
      if (t < DU) xs[t] = a[u];
    }
  }
  if (threadIdx.x < FX1_ZERO_UNITS) xs[DU + threadIdx.x] = make_longlong2(0ll, 0ll);
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int nw = (DU + 31) >> 5;
  const i64 e1d = fv.dw_e1[idw];
  const unsigned wd = (unsigned)sv.dw_words[idw];
  for (int w = threadIdx.x >> 5; w < nw; w += FX1_UP2_THREADS / 32) {
    const int iup = w * 32 + lane;
    const bool row = iup < DU;
    const i64 eu = row ? fv.up_e1[iup] : 0;
    const unsigned wu = row ? (unsigned)sv.up_words[iup] : 0u;
    u64 A[K], B[K];
    up2_rounds<K>(fv, w, lane, DU, x1p_smem, A, B);
    if (!row) continue;
    const longlong2 xi = xs[iup];
    const i64 d = eu + e1d + mixed_fx(fv, wu, wd);
    i128 p0 = (i128)d * xi.x, p1 = (i128)d * xi.y;
#pragma unroll
    for (int k = 0; k < K; k++) p0 += (i128)fv.afx[k] * (i64)A[k], p1 += (i128)fv.afx[k] * (i64)B[k];
    const bool sh63 = fv.shift >= 1 && fv.shift <= 63;
    __stcg(Y2 + (int64_t)iup * 4, make_longlong2((long long)rshift_round_u(p0, fv.shift, sh63),
                                                 (long long)rshift_round_u(p1, fv.shift, sh63)));
  }
}

template <int K>
__global__ void __launch_bounds__(FXS_DW_ROWS * 4) k_hxv_slab_dw2(SectorView sv, FxView fv, int nslab,
                                                              const i64* __restrict__ X, i64* __restrict__ Y) {
  const int DU = sv.dimup, DD = sv.dimdw;
  const int ngrp = (DD + FXS_DW_GRP - 1) / FXS_DW_GRP;
  const int grp = blockIdx.x % ngrp;
  const int t2 = blockIdx.x / ngrp;
  const int sl = t2 % nslab, ck = t2 / nslab;
  const int pr = threadIdx.x & 3;
  const int iup = ck * FXS_DW_ROWS + (threadIdx.x >> 2);
  if (iup >= DU) return;
  const int64_t D = (int64_t)DU * DD;
  const longlong2* X2 = (const longlong2*)X + ((int64_t)sl * D + iup) * 4 + pr;
  longlong2* Y2 = (longlong2*)Y + ((int64_t)sl * D + iup) * 4 + pr;
  const int64_t bstride = (int64_t)DU * 4;  // one down configuration, in 16-byte units
  for (int j = 0; j < FXS_DW_GRP; j++) {
    const int idw = grp * FXS_DW_GRP + j;
    if (idw >= DD) break;
    const int nd = sv.dw_cnt[idw], ndp = fv.dw_npos[idw];
    const int64_t own = (int64_t)idw * bstride;
    const longlong2 y = __ldcg(Y2 + own);
    u64 A[K], B[K];
#pragma unroll
    for (int k = 0; k < K; k++) A[k] = B[k] = 0;
    int h = 0;
#pragma unroll 4
    for (; h < ndp; h++) {
      const unsigned hw = __ldg(fv.dw_hop + idw + (int64_t)h * DD);
      const longlong2 v = __ldcg(X2 + (int64_t)(hw & 0xFFFFFFu) * bstride);
      const int cls = (K == 1) ? 0 : (int)((hw >> 24) & 3u);
#pragma unroll
      for (int k = 0; k < K; k++)
        if (k == cls) A[k] += (u64)v.x, B[k] += (u64)v.y;
    }
#pragma unroll 4
    for (; h < nd; h++) {
      const unsigned hw = __ldg(fv.dw_hop + idw + (int64_t)h * DD);
      const longlong2 v = __ldcg(X2 + (int64_t)(hw & 0xFFFFFFu) * bstride);
      const int cls = (K == 1) ? 0 : (int)((hw >> 24) & 3u);
#pragma unroll
      for (int k = 0; k < K; k++)
        if (k == cls) A[k] -= (u64)v.x, B[k] -= (u64)v.y;
    }
    i128 pa = 0, pb = 0;
#pragma unroll
    for (int k = 0; k < K; k++) pa += (i128)fv.afx[k] * (i64)A[k], pb += (i128)fv.afx[k] * (i64)B[k];
    const bool sh63 = fv.shift >= 1 && fv.shift <= 63;
    __stcg(Y2 + own, make_longlong2((long long)((i64)y.x + rshift_round_u(pa, fv.shift, sh63)),
                                    (long long)((i64)y.y + rshift_round_u(pb, fv.shift, sh63))));
  }
}

#define FXS_DOT_ROWS (152 * 4)  // alpha partial rows of the slab-pair form
static bool hxv_fx_slab2_ok(const SectorView& sv, const FxView& fv, int m, bool warp_only) {
  return !warp_only && !fv.rows_permuted && fv.up_sched && fv.up_wround && fv.up_wgrp && fv.dw_npos &&
         fx_pair_fits(sv.dimup) && m >= FX_SLAB && m % FX_SLAB == 0 &&
         (int64_t)sv.dimup * sv.dimdw >= FX1_MIN_DIM;
}

template <int K>
static void launch_hxv_slab_k(const SectorView& sv, const FxView& fv, int m, const i64* X, i64* Y, i64* apart,
                              cudaStream_t st) {
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_hxv_slab_up2<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, FX1_SMEM_MAX);
    attr = true;
  }
  const int nslab = m / FX_SLAB;
  const int DU = sv.dimup, DD = sv.dimdw;
  count_launch_external();
  count_launch_external();
  k_hxv_slab_up2<K><<<DD * nslab * 4, FX1_UP2_THREADS, (size_t)(DU + FX1_ZERO_UNITS) * 16, st>>>(sv, fv, nslab, X, Y);
  const int nck = (DU + FXS_DW_ROWS - 1) / FXS_DW_ROWS, ngrp = (DD + FXS_DW_GRP - 1) / FXS_DW_GRP;
  k_hxv_slab_dw2<K><<<nck * nslab * ngrp, FXS_DW_ROWS * 4, 0, st>>>(sv, fv, nslab, X, Y);
  if (apart) {  // exact int128 <X, Y> partials, FXS_DOT_ROWS rows of m
    count_launch_external();
    dim3 blk;
    int ns;
    slab_shape(m, blk, ns);
    k_fx_dot<<<dim3(FXS_DOT_ROWS, ns, 1), blk, sizeof(i128) * 256, st>>>((int64_t)DU * DD, m, X, Y, apart);
  }
}

int hxv_fx_cols_rows(const SectorView& sv, const FxView& fv, int m, bool warp_only) {
  if (fv.rows_permuted || hxv_fx_s_ok(sv, fv, m, warp_only)) return sv.dimdw;
  if (hxv_fx_slab2_ok(sv, fv, m, warp_only)) return FXS_DOT_ROWS;
  return hxv_fx_w_rowblocks((int64_t)sv.dimup * sv.dimdw);
}

void launch_hxv_fx_cols(const SectorView& sv, const FxView& fv, int m, const i64* X, i64* Y, i64* apart,
                        bool warp_only, cudaStream_t st) {
  if (fv.rows_permuted) {  // callers set it only where hxv_fx_r_ok holds
    if (fv.K == 1) launch_hxv_fx_r_k<1>(sv, fv, m, X, Y, apart, st);
    else launch_hxv_fx_r_k<2>(sv, fv, m, X, Y, apart, st);
    return;
  }
  if (hxv_fx_s_ok(sv, fv, m, warp_only)) {
    switch (fv.K) {
      case 1: launch_hxv_fx_s_k<1>(sv, fv, m, X, Y, apart, st); break;
      case 2: launch_hxv_fx_s_k<2>(sv, fv, m, X, Y, apart, st); break;
      case 3: launch_hxv_fx_s_k<3>(sv, fv, m, X, Y, apart, st); break;
      default: launch_hxv_fx_s_k<4>(sv, fv, m, X, Y, apart, st); break;
    }
    return;
  }
  if (hxv_fx_slab2_ok(sv, fv, m, warp_only)) {
    switch (fv.K) {
      case 1: launch_hxv_slab_k<1>(sv, fv, m, X, Y, apart, st); break;
      case 2: launch_hxv_slab_k<2>(sv, fv, m, X, Y, apart, st); break;
      case 3: launch_hxv_slab_k<3>(sv, fv, m, X, Y, apart, st); break;
      default: launch_hxv_slab_k<4>(sv, fv, m, X, Y, apart, st); break;
    }
    return;
  }
  launch_hxv_fx_w(sv, fv, m, X, Y, apart, st);
}

}  // namespace vca
