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

// 16-byte asynchronous global -> shared copies (sm_80+ cp.async): a CTA
// issues its whole tile before waiting once, so many loads are in flight.
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

static void col_shape_fx(int m, dim3& blk) {
  int cw = 1;
  while (cw < m && cw < 32) cw <<= 1;
  blk = dim3(cw, 256 / cw, 1);
}

// round-half-up arithmetic shift of an int128 by s >= 0
__device__ __forceinline__ i64 rshift_round(i128 p, int s) {
  if (s <= 0) return (i64)p;
  p += ((i128)1) << (s - 1);
  return (i64)(p >> s);
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

template <int K>
__global__ void k_hxv_fx(SectorView sv, FxView fv, int m, const i64* __restrict__ X, i64* __restrict__ Y) {
  const int64_t D = (int64_t)sv.dimup * sv.dimdw;
  const int CW = blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.y + threadIdx.y; i < D;
       i += (int64_t)gridDim.x * blockDim.y) {
    const int idw = (int)(i / sv.dimup);
    const int iup = (int)(i - (int64_t)idw * sv.dimup);
    const i64 dfx = fv.up_e1[iup] + fv.dw_e1[idw] +
                    mixed_fx(fv, (unsigned)sv.up_words[iup], (unsigned)sv.dw_words[idw]);
    const int nu = sv.up_cnt[iup], nd = sv.dw_cnt[idw];
    const int64_t colbase = (int64_t)idw * sv.dimup;
    for (int c = threadIdx.x; c < m; c += CW) {
      i64 S[K];
#pragma unroll
      for (int k = 0; k < K; k++) S[k] = 0;
      for (int h = 0; h < nu; h++) {
        const int64_t o = (int64_t)h * sv.dimup + iup;
        acc_hop<K>(S, fv.up_code[o], X[(colbase + sv.up_src[o]) * m + c]);
      }
      for (int h = 0; h < nd; h++) {
        const int64_t o = (int64_t)h * sv.dimdw + idw;
        acc_hop<K>(S, fv.dw_code[o], X[((int64_t)iup + (int64_t)sv.dw_src[o] * sv.dimup) * m + c]);
      }
      i128 p = (i128)dfx * X[i * m + c];
#pragma unroll
      for (int k = 0; k < K; k++) p += (i128)fv.afx[k] * S[k];
      Y[i * m + c] = rshift_round(p, fv.shift);
    }
  }
}


void launch_hxv_fx(const SectorView& sv, const FxView& fv, int m, const i64* X, i64* Y, cudaStream_t st) {
  count_launch_external();
  dim3 blk;
  col_shape_fx(m, blk);
  const int64_t D = (int64_t)sv.dimup * sv.dimdw;
  const int nb = nblk_fx(D, blk.y, 152 * 32);
  switch (fv.K) {
    case 1: k_hxv_fx<1><<<nb, blk, 0, st>>>(sv, fv, m, X, Y); break;
    case 2: k_hxv_fx<2><<<nb, blk, 0, st>>>(sv, fv, m, X, Y); break;
    case 3: k_hxv_fx<3><<<nb, blk, 0, st>>>(sv, fv, m, X, Y); break;
    default: k_hxv_fx<4><<<nb, blk, 0, st>>>(sv, fv, m, X, Y); break;
  }
}

// ---------------------------------------------------------------------------
// exact dot products
// ---------------------------------------------------------------------------
__global__ void k_fx_dot(int64_t rows, int m, const i64* X, const i64* Y, i64* partial) {
  extern __shared__ i128 shq[];
  const int CW = blockDim.x, RB = blockDim.y;
  const int c = blockIdx.y * CW + threadIdx.x;
  i128 s = 0;
  if (c < m)
    for (int64_t i = (int64_t)blockIdx.x * RB + threadIdx.y; i < rows; i += (int64_t)gridDim.x * RB)
      s += (i128)X[i * m + c] * Y[i * m + c];
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
__global__ void k_fx_dot_reduce(int m, int nblk, const i64* partial, int scale_exp, double* out) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < m; c += gridDim.x * blockDim.x) {
    i128 s = 0;
    for (int b = 0; b < nblk; b++) {
      const u64 lo = (u64)partial[2 * ((int64_t)b * m + c)];
      const i64 hi = partial[2 * ((int64_t)b * m + c) + 1];
      s += (i128)(((unsigned __int128)(u64)hi << 64) | lo);
    }
    out[c] = i128_to_double(s, scale_exp);
  }
}
void launch_fx_dot(const ColBatch& b, const i64* X, const i64* Y, int sx, int sy, i64* partial, int nblk,
                   double* out_col, cudaStream_t st) {
  count_launch_external();
  count_launch_external();
  dim3 blk;
  col_shape_fx(b.m, blk);
  dim3 grd(nblk, (b.m + blk.x - 1) / blk.x, 1);
  k_fx_dot<<<grd, blk, sizeof(i128) * 256, st>>>(b.rows, b.m, X, Y, partial);
  k_fx_dot_reduce<<<nblk_fx(b.m, 128), 128, 0, st>>>(b.m, nblk, partial, sx + sy, out_col);
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
                            const i64* Y, i64* W) {
  const int64_t n = rows * m;
  for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < n;
       g += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(g % m);
    const int ch = col2ch[c];
    if (!meta[ch].active) continue;
    i128 p = (i128)afx[ch] * X[g];
    if (use_b) p += (i128)bfx[ch] * Xp[g];
    W[g] = Y[g] - rshift_round(p, sh);
  }
}
void launch_fx_update(const ColBatch& b, const FxScales& s, const i64* afx, const i64* bfx, bool use_b,
                      const i64* X, const i64* Xp, const i64* Y, i64* W, cudaStream_t st) {
  count_launch_external();
  const int64_t n = b.rows * b.m;
  k_fx_update<<<nblk_fx(n, 256), 256, 0, st>>>(b.rows, b.m, b.col2ch, b.meta, s.C + s.F - s.G, afx, bfx,
                                                use_b ? 1 : 0, X, Xp, Y, W);
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
// column-tiled: block (CW columns x RB rows), column from blockIdx.y, so no
// per-element division by m
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
  for (int64_t i = (int64_t)blockIdx.x * RB + threadIdx.y; i < rows; i += (int64_t)gridDim.x * RB) {
    const int64_t g = i * m + c;
    Xo[g] = act ? rshift_round((i128)mu * Xi[g], s) : 0;
  }
}
static void launch_apply(const ColBatch& b, const i64* mul, const i64* sh, int zero_inactive, const i64* Xi,
                         i64* Xo, cudaStream_t st) {
  dim3 blk;
  col_shape_fx(b.m, blk);
  const int64_t nrb = (b.rows + blk.y - 1) / blk.y;
  const int gx = (int)std::max<int64_t>(1, std::min<int64_t>(nrb, 152 * 16));
  dim3 grd(gx, (b.m + blk.x - 1) / blk.x, 1);
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


// ---------------------------------------------------------------------------
// Two-pass H x v on column batches (fixed point).
//
// Pass A (up hops + diagonal): one CTA per (idw, column chunk); the block
// X[:, idw, chunk] (DimUp x CW int64, <= 200 KB) is staged in shared memory,
// so every up hop is a shared-memory load and X is read from DRAM once.
// Pass B (down hops): one CTA per (iup, column chunk); X[iup, :, chunk]
// (DimDw x CW) is staged likewise, Y is completed in place and the exact
// int128 partial of alpha = <X, Y> is written per (iup, column).
// DRAM per column element: A reads X, writes Y (16 B); B reads X, Y and
// writes Y (24 B).
// ---------------------------------------------------------------------------
template <int K>
__global__ void __launch_bounds__(256) k_hxv_fx_a(SectorView sv, FxView fv, int m, int cw,
                                                  const i64* __restrict__ X, i64* __restrict__ Y) {
  extern __shared__ i64 xs[];  // [DimUp][cw]
  const int nchunk = (m + cw - 1) / cw;
  const int idw = blockIdx.x / nchunk;
  const int c0 = (blockIdx.x % nchunk) * cw;
  const int ncol = min(cw, m - c0);
  const int DU = sv.dimup;
  const int64_t base = (int64_t)idw * DU;
  if ((m & 1) == 0 && (ncol & 1) == 0 && (cw & 1) == 0) {
    // pairs of int64 = 16 B; row starts (base+r)*m + c0 are even -> aligned
    const int hp = cw >> 1, hn = ncol >> 1;
    for (int t = threadIdx.x; t < DU * hp; t += blockDim.x) {
      const int r = t / hp, q = t - r * hp;
      if (q < hn) cp_async16(xs + r * cw + 2 * q, X + (base + r) * m + c0 + 2 * q);
      else { xs[r * cw + 2 * q] = 0; xs[r * cw + 2 * q + 1] = 0; }
    }
    cp_async_wait_all();
  } else {
    for (int t = threadIdx.x; t < DU * cw; t += blockDim.x) {
      const int r = t / cw, cc = t - r * cw;
      xs[t] = (cc < ncol) ? X[(base + r) * m + c0 + cc] : 0;
    }
  }
  __syncthreads();
  const i64 edw = fv.dw_e1[idw];
  const unsigned wd = (unsigned)sv.dw_words[idw];
  for (int t = threadIdx.x; t < DU * cw; t += blockDim.x) {
    const int r = t / cw, cc = t - r * cw;
    if (cc >= ncol) continue;
    const i64 dfx = fv.up_e1[r] + edw + mixed_fx(fv, (unsigned)sv.up_words[r], wd);
    i64 S[K];
#pragma unroll
    for (int k = 0; k < K; k++) S[k] = 0;
    const int nu = sv.up_cnt[r];
    for (int h = 0; h < nu; h++) {
      const int64_t o = (int64_t)h * DU + r;
      acc_hop<K>(S, fv.up_code[o], xs[sv.up_src[o] * cw + cc]);
    }
    i128 p = (i128)dfx * xs[t];
#pragma unroll
    for (int k = 0; k < K; k++) p += (i128)fv.afx[k] * S[k];
    Y[(base + r) * m + c0 + cc] = rshift_round(p, fv.shift);
  }
}

template <int K>
__global__ void __launch_bounds__(256) k_hxv_fx_b(SectorView sv, FxView fv, int m, int cw,
                                                  const i64* __restrict__ X, i64* __restrict__ Y,
                                                  i64* __restrict__ apart) {
  extern __shared__ i64 xs[];  // [DimDw][cw]
  __shared__ i128 red[256];
  const int nchunk = (m + cw - 1) / cw;
  const int iup = blockIdx.x / nchunk;
  const int c0 = (blockIdx.x % nchunk) * cw;
  const int ncol = min(cw, m - c0);
  const int DU = sv.dimup, DD = sv.dimdw;
  if ((m & 1) == 0 && (ncol & 1) == 0 && (cw & 1) == 0) {
    const int hp = cw >> 1, hn = ncol >> 1;
    for (int t = threadIdx.x; t < DD * hp; t += blockDim.x) {
      const int r = t / hp, q = t - r * hp;
      if (q < hn) cp_async16(xs + r * cw + 2 * q, X + ((int64_t)iup + (int64_t)r * DU) * m + c0 + 2 * q);
      else { xs[r * cw + 2 * q] = 0; xs[r * cw + 2 * q + 1] = 0; }
    }
    cp_async_wait_all();
  } else {
    for (int t = threadIdx.x; t < DD * cw; t += blockDim.x) {
      const int r = t / cw, cc = t - r * cw;
      xs[t] = (cc < ncol) ? X[((int64_t)iup + (int64_t)r * DU) * m + c0 + cc] : 0;
    }
  }
  __syncthreads();
  // thread t always handles column t % cw (blockDim is a multiple of cw)
  i128 adot = 0;
  for (int t = threadIdx.x; t < DD * cw; t += blockDim.x) {
    const int r = t / cw, cc = t - r * cw;
    if (cc >= ncol) continue;
    i64 S[K];
#pragma unroll
    for (int k = 0; k < K; k++) S[k] = 0;
    const int nd = sv.dw_cnt[r];
    for (int h = 0; h < nd; h++) {
      const int64_t o = (int64_t)h * DD + r;
      acc_hop<K>(S, fv.dw_code[o], xs[sv.dw_src[o] * cw + cc]);
    }
    i128 p = 0;
#pragma unroll
    for (int k = 0; k < K; k++) p += (i128)fv.afx[k] * S[k];
    const int64_t g = ((int64_t)iup + (int64_t)r * DU) * m + c0 + cc;
    const i64 y = Y[g] + rshift_round(p, fv.shift);
    Y[g] = y;
    adot += (i128)xs[t] * y;
  }
  red[threadIdx.x] = adot;
  __syncthreads();
  if ((int)threadIdx.x < cw) {
    i128 s = 0;
    for (int q = threadIdx.x; q < (int)blockDim.x; q += cw) s += red[q];
    if ((int)threadIdx.x < ncol) {
      const int64_t o = 2 * ((int64_t)iup * m + c0 + threadIdx.x);
      apart[o] = (i64)(u64)s;
      apart[o + 1] = (i64)(s >> 64);
    }
  }
}

// sum of int128 partials over `rows` rows per column -> double (scale 2^-sexp)
__global__ void k_fx_partial_reduce(int m, int rows, const i64* partial, int sexp, double* out) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < m; c += gridDim.x * blockDim.x) {
    i128 s = 0;
    for (int b = 0; b < rows; b++) {
      const u64 lo = (u64)partial[2 * ((int64_t)b * m + c)];
      const i64 hi = partial[2 * ((int64_t)b * m + c) + 1];
      s += (i128)(((unsigned __int128)(u64)hi << 64) | lo);
    }
    out[c] = i128_to_double(s, sexp);
  }
}

int hxv_fx_chunk(int rows, int m) {
  const int budget = 100 * 1024 / 8;  // int64 slots: <= 100 KB so two CTAs share an SM
  int cw = 32;
  while (cw > 1 && (cw >= 2 * m || rows * cw > budget)) cw >>= 1;
  if (rows * cw > budget) return 0;  // a single column does not fit
  return cw;
}

bool launch_hxv_fx2(const SectorView& sv, const FxView& fv, int m, const i64* X, i64* Y, i64* apart,
                    cudaStream_t st) {
  const int cwa = hxv_fx_chunk(sv.dimup, m), cwb = hxv_fx_chunk(sv.dimdw, m);
  if (!cwa || !cwb) return false;
  const size_t sha = (size_t)sv.dimup * cwa * sizeof(i64), shb = (size_t)sv.dimdw * cwb * sizeof(i64);
  const int ga = sv.dimdw * ((m + cwa - 1) / cwa), gb = sv.dimup * ((m + cwb - 1) / cwb);
  count_launch_external();
  count_launch_external();
#define VCA_FX2(KK)                                                                                  \
  {                                                                                                  \
    static bool attr = false;                                                                        \
    if (!attr) {                                                                                     \
      cudaFuncSetAttribute(k_hxv_fx_a<KK>, cudaFuncAttributeMaxDynamicSharedMemorySize, 104 * 1024); \
      cudaFuncSetAttribute(k_hxv_fx_b<KK>, cudaFuncAttributeMaxDynamicSharedMemorySize, 104 * 1024); \
      attr = true;                                                                                   \
    }                                                                                                \
  }                                                                                                  \
  k_hxv_fx_a<KK><<<ga, 256, sha, st>>>(sv, fv, m, cwa, X, Y);                                        \
  k_hxv_fx_b<KK><<<gb, 256, shb, st>>>(sv, fv, m, cwb, X, Y, apart);
  switch (fv.K) {
    case 1: VCA_FX2(1) break;
    case 2: VCA_FX2(2) break;
    case 3: VCA_FX2(3) break;
    default: VCA_FX2(4) break;
  }
#undef VCA_FX2
  return true;
}

void launch_fx_partial_reduce(int m, int rows, const i64* partial, int sexp, double* out, cudaStream_t st) {
  count_launch_external();
  k_fx_partial_reduce<<<nblk_fx(m, 128), 128, 0, st>>>(m, rows, partial, sexp, out);
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
      for (int64_t i = (int64_t)blockIdx.x * RB + threadIdx.y; i < rows; i += (int64_t)gridDim.x * RB) {
        const int64_t g = i * m + c;
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
void launch_fx_update_dot(const ColBatch& b, const FxScales& s, const i64* afx, const i64* bfx, bool use_b,
                          const i64* X, const i64* Xp, i64* YW, i64* partial, int nblk, double* out_col,
                          cudaStream_t st) {
  count_launch_external();
  dim3 blk;
  col_shape_fx(b.m, blk);
  dim3 grd(nblk, (b.m + blk.x - 1) / blk.x, 1);
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

// accumulate one hop's source row into the class accumulators; the class and
// sign are warp-uniform, so the branches do not diverge
template <int K, int NCQ>
__device__ __forceinline__ void hop_row(i64 (&S)[K][NCQ], unsigned hw, const i64* __restrict__ xr, int lim) {
  const int cls = (K == 1) ? 0 : (int)((hw >> 24) & 3u);
  const bool neg = hw >> 31;
#pragma unroll
  for (int k = 0; k < K; k++) {
    if (k != cls) continue;
    if (neg) {
#pragma unroll
      for (int q = 0; q < NCQ; q++)
        if (32 * q < lim) S[k][q] -= xr[32 * q];
    } else {
#pragma unroll
      for (int q = 0; q < NCQ; q++)
        if (32 * q < lim) S[k][q] += xr[32 * q];
    }
  }
}

// MODE 0: full product (rows in idw-major order).
// MODE 1: diagonal + up hops only, rows in idw-major order: a column block's
//         up neighbours are the rows being processed, so they stay in L2.
// MODE 2: down hops added into Y, rows in iup-major order: a slab's down
//         neighbours stay in L2.  Modes 1 + 2 read X from DRAM about once each.
template <int K, int NCQ, int MODE>
__global__ void __launch_bounds__(256) k_hxv_fx_w(SectorView sv, FxView fv, int m, const i64* __restrict__ X,
                                                  i64* __restrict__ Y) {
  const int lane = threadIdx.x & 31;
  const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  const int DU = sv.dimup, DD = sv.dimdw;
  const int D = DU * DD;
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
    for (int c0 = 0; c0 < m; c0 += 32 * NCQ) {
      const int lim = m - c0 - lane;  // column lane + 32q exists while 32q < lim
      i64 S[K][NCQ];
#pragma unroll
      for (int k = 0; k < K; k++)
#pragma unroll
        for (int q = 0; q < NCQ; q++) S[k][q] = 0;
      for (int h = 0, o = iup; h < nu; h++, o += DU) {
        const unsigned hw = fv.up_hop[o];
        hop_row<K, NCQ>(S, hw, X + (int64_t)(colbase + (int)(hw & 0xFFFFFFu)) * m + c0 + lane, lim);
      }
      for (int h = 0, o = idw; h < nd; h++, o += DD) {
        const unsigned hw = fv.dw_hop[o];
        hop_row<K, NCQ>(S, hw, X + (int64_t)(iup + (int)(hw & 0xFFFFFFu) * DU) * m + c0 + lane, lim);
      }
      const i64* xo = X + (int64_t)r * m + c0 + lane;
      i64* yo = Y + (int64_t)r * m + c0 + lane;
#pragma unroll
      for (int q = 0; q < NCQ; q++) {
        if (32 * q < lim) {
          i128 p = 0;
          if (MODE != 2) p = (i128)dfx * xo[32 * q];
#pragma unroll
          for (int k = 0; k < K; k++) p += (i128)fv.afx[k] * S[k][q];
          const i64 y = rshift_round(p, fv.shift);
          yo[32 * q] = (MODE == 2) ? yo[32 * q] + y : y;
        }
      }
    }
  }
}

void launch_hxv_fx_w(const SectorView& sv, const FxView& fv, int m, const i64* X, i64* Y, cudaStream_t st) {
  const int64_t D = (int64_t)sv.dimup * sv.dimdw;
  const int blocks = nblk_fx(D * 32, 256, 152 * 8);
  // columns per pass: 32*NCQ, NCQ limited so K*NCQ int64 accumulators stay in registers
#define VCA_W(KK, NQ)                                                   \
  do {                                                                  \
    count_launch_external();                                            \
    count_launch_external();                                            \
    k_hxv_fx_w<KK, NQ, 1><<<blocks, 256, 0, st>>>(sv, fv, m, X, Y);     \
    k_hxv_fx_w<KK, NQ, 2><<<blocks, 256, 0, st>>>(sv, fv, m, X, Y);     \
  } while (0)
  const int ncq = (m + 31) / 32;
  switch (fv.K) {
    case 1:
      if (ncq <= 4) VCA_W(1, 4);
      else if (ncq <= 8) VCA_W(1, 8);
      else VCA_W(1, 16);
      break;
    case 2:
      if (ncq <= 4) VCA_W(2, 4);
      else VCA_W(2, 8);
      break;
    case 3: VCA_W(3, 4); break;
    default: VCA_W(4, 4); break;
  }
#undef VCA_W
}
}  // namespace vca
