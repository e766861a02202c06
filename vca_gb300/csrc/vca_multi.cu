// vca_multi.cu -- all sectors' ground-state Lanczos in one batched loop
// (fixed-point path).
//
// The reference diagonalises the (N_up, N_dw) sectors one after the other
// (VCA_DIAG.f90:83-249).  Most sectors are small, so a sector-at-a-time GPU
// loop is launch bound.  Here the vectors of every sector of a group are
// packed back to back and cut into tiles of MS_TILE elements; each Lanczos
// phase is one launch over all tiles (a tile -> sector work table), the
// per-sector scalars are reduced by one thread per sector, and the
// convergence test of every sector is one warp per sector.  The arithmetic is
// the same fixed-point arithmetic as the single-sector kernels, and every
// reduction is an exact int128 sum, so each sector gets bitwise the same
// alpha/beta sequence as when it runs alone.
#include "vca_multi.cuh"
#include "vca_tri.cuh"

namespace vca {

void count_launch_external();

typedef __int128 i128;
typedef unsigned long long u64;

__device__ __forceinline__ i64 ms_rshift(i128 p, int s) {
  if (s <= 0) return (i64)p;
  p += ((i128)1) << (s - 1);
  return (i64)(p >> s);
}
__device__ __forceinline__ double ms_i128_to_double(i128 v, int scale_exp) {
  const bool neg = v < 0;
  unsigned __int128 u = neg ? (unsigned __int128)(-v) : (unsigned __int128)v;
  const u64 hi = (u64)(u >> 64), lo = (u64)u;
  double d = (double)hi * 18446744073709551616.0 + (double)lo;
  d = ldexp(d, -scale_exp);
  return neg ? -d : d;
}
__device__ __forceinline__ uint64_t ms_splitmix64(uint64_t x) {
  uint64_t z = x + 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__device__ __forceinline__ i64 ms_mixed(const FxView& f, unsigned u, unsigned d) {
  i64 s = f.c0fx;
  for (int o = 0; o < f.norb; o++) s += f.Ufx[o] * (i64)__popc(u & d & f.omask[o]);
  int c = 0;
  for (int o = 0; o < f.norb; o++)
    for (int q = o + 1; q < f.norb; q++)
      c += __popc(u & f.omask[o] & (d >> (q - o))) + __popc(u & f.omask[q] & (d << (q - o)));
  return s + f.Ustfx * (i64)c;
}

// block reduction of an int128 per-thread value into tpart[t] (2 x int64)
__device__ __forceinline__ void ms_block_store(i128 v, i64* tpart, int t) {
  __shared__ i128 red[256];
  red[threadIdx.x] = v;
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    tpart[2 * t] = (i64)(u64)red[0];
    tpart[2 * t + 1] = (i64)(red[0] >> 64);
  }
  __syncthreads();
}
__device__ __forceinline__ i128 ms_sum_parts(const i64* tpart, int t0, int n) {
  i128 s = 0;
  for (int t = t0; t < t0 + n; t++)
    s += (i128)(((unsigned __int128)(u64)tpart[2 * t + 1] << 64) | (u64)tpart[2 * t]);
  return s;
}

// the same sum spread over the lanes of a warp (exact, any order), the
// total returned to every lane
__device__ __forceinline__ i128 ms_sum_parts_warp(const i64* tpart, int t0, int n) {
  const int lane = threadIdx.x & 31;
  i128 s = 0;
  for (int t = t0 + lane; t < t0 + n; t += 32)
    s += (i128)(((unsigned __int128)(u64)tpart[2 * t + 1] << 64) | (u64)tpart[2 * t]);
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
  return ((i128)hi << 64) | (i128)lo;
}

// start vector: R_i = round(v_i * 2^40) with v_i the splitmix64 value of the
// single-sector path; tpart = sum R^2
__global__ void k_ms_start_raw(const MsSector* secs, const int* tsec, const int64_t* tstart, int ntiles,
                               uint64_t seed, i64* R, i64* tpart) {
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const MsSector& S = secs[tsec[t]];
    const int64_t i0 = tstart[t], i1 = min(i0 + (int64_t)MS_TILE, S.D);
    i128 acc = 0;
    for (int64_t i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
      const uint64_t z = ms_splitmix64(seed + 0xD1B54A32D192ED03ull * (uint64_t)S.isector + (uint64_t)i);
      const double v = (double)(z >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0;
      const i64 r = __double2ll_rn(ldexp(v, 40));
      R[S.off + i] = r;
      acc += (i128)r * r;
    }
    ms_block_store(acc, tpart, t);
  }
}

// per-sector multiplier f * 2^(so - si) as (mul, shift) (k_fx_mult restated)
__device__ __forceinline__ void ms_mult(double x, int si, int so, i64& mul, int& sh) {
  if (x == 0.0 || !isfinite(x)) { mul = 0; sh = 0; return; }
  int e;
  frexp(fabs(x), &e);
  int E = 60 - e;
  int shift = E + si - so;
  if (shift > 120) { E -= shift - 120; shift = 120; }
  if (shift < 0) { E -= shift; shift = 0; }
  mul = __double2ll_rn(ldexp(x, E));
  sh = shift;
}

__global__ void k_ms_start_norm(int nsec, const MsSector* secs, const i64* tpart, int F, ChainMeta* meta,
                                i64* mul, int* msh) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < nsec; s += gridDim.x * blockDim.x) {
    const double n2 = ms_i128_to_double(ms_sum_parts(tpart, secs[s].tile0, secs[s].ntile), 80);
    double invn = 0.0;
    if (n2 > 0.0) invn = 1.0 / sqrt(n2);
    else { meta[s].active = 0; meta[s].len = 0; }
    i64 m;
    int sh;
    ms_mult(invn, 40, F, m, sh);
    mul[s] = m;
    msh[s] = sh;
  }
}

__global__ void k_ms_apply(const MsSector* secs, const int* tsec, const int64_t* tstart, int ntiles,
                           const ChainMeta* meta, const i64* mul, const int* msh, int zero_inactive,
                           const i64* Xi, i64* Xo) {
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int s = tsec[t];
    const MsSector& S = secs[s];
    const int64_t i0 = tstart[t], i1 = min(i0 + (int64_t)MS_TILE, S.D);
    const bool act = meta[s].active;
    if (!act && !zero_inactive) continue;
    const i64 m = mul[s];
    const int sh = msh[s];
    for (int64_t i = i0 + threadIdx.x; i < i1; i += blockDim.x)
      Xo[S.off + i] = act ? ms_rshift((i128)m * Xi[S.off + i], sh) : 0;
  }
}

// H x v (single column, fixed point) + exact alpha partial per tile
template <int K>
__global__ void __launch_bounds__(256) k_ms_hxv(const MsSector* secs, const int* tsec, const int64_t* tstart,
                                                int ntiles, const ChainMeta* meta, const i64* __restrict__ X,
                                                i64* __restrict__ Y, i64* tpart) {
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int s = tsec[t];
    i128 adot = 0;
    if (meta[s].active) {
      const MsSector& S = secs[s];
      const SectorView& sv = S.sv;
      const FxView& fv = S.fv;
      const i64* Xs = X + S.off;
      const int64_t i0 = tstart[t], i1 = min(i0 + (int64_t)MS_TILE, S.D);
      for (int64_t i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
        const int idw = (int)(i / sv.dimup);
        const int iup = (int)(i - (int64_t)idw * sv.dimup);
        const i64 dfx = fv.up_e1[iup] + fv.dw_e1[idw] +
                        ms_mixed(fv, (unsigned)sv.up_words[iup], (unsigned)sv.dw_words[idw]);
        i64 Sk[K];
#pragma unroll
        for (int k = 0; k < K; k++) Sk[k] = 0;
        const int nu = sv.up_cnt[iup], nd = sv.dw_cnt[idw];
        const int64_t colbase = (int64_t)idw * sv.dimup;
        for (int h = 0; h < nu; h++) {
          const int64_t o = (int64_t)h * sv.dimup + iup;
          const signed char code = fv.up_code[o];
          const i64 v = Xs[colbase + sv.up_src[o]];
          const i64 sv_ = (code < 0) ? -v : v;
#pragma unroll
          for (int k = 0; k < K; k++) Sk[k] += (K == 1 || (code & 3) == k) ? sv_ : 0;
        }
        for (int h = 0; h < nd; h++) {
          const int64_t o = (int64_t)h * sv.dimdw + idw;
          const signed char code = fv.dw_code[o];
          const i64 v = Xs[(int64_t)iup + (int64_t)sv.dw_src[o] * sv.dimup];
          const i64 sv_ = (code < 0) ? -v : v;
#pragma unroll
          for (int k = 0; k < K; k++) Sk[k] += (K == 1 || (code & 3) == k) ? sv_ : 0;
        }
        const i64 x = Xs[i];
        i128 p = (i128)dfx * x;
#pragma unroll
        for (int k = 0; k < K; k++) p += (i128)fv.afx[k] * Sk[k];
        const i64 y = ms_rshift(p, fv.shift);
        Y[S.off + i] = y;
        adot += (i128)x * y;
      }
    }
    ms_block_store(adot, tpart, t);
  }
}

// one warp per sector
__global__ void k_ms_alpha(int nsec, const MsSector* secs, const ChainMeta* meta, const i64* tpart, int sexp,
                           int C, const double* bnow, double* alpha, i64* afx, i64* bfx) {
  const int lane = threadIdx.x & 31;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < nsec; s += nw) {
    if (!meta[s].active) continue;
    const i128 v = ms_sum_parts_warp(tpart, secs[s].tile0, secs[s].ntile);
    if (lane == 0) {
      const double a = 0.0 + ms_i128_to_double(v, sexp);
      alpha[s] = a;
      afx[s] = __double2ll_rn(ldexp(1.0 * a, C));
      bfx[s] = __double2ll_rn(ldexp(1.0 * bnow[s], C));
    }
  }
}

__global__ void k_ms_update(const MsSector* secs, const int* tsec, const int64_t* tstart, int ntiles,
                            const ChainMeta* meta, int sh, const i64* afx, const i64* bfx, int use_b,
                            const i64* X, const i64* Xp, i64* YW, i64* tpart) {
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int s = tsec[t];
    i128 acc = 0;
    if (meta[s].active) {
      const MsSector& S = secs[s];
      const int64_t i0 = tstart[t], i1 = min(i0 + (int64_t)MS_TILE, S.D);
      const i64 a = afx[s], b = use_b ? bfx[s] : 0;
      for (int64_t i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
        const int64_t g = S.off + i;
        i128 p = (i128)a * X[g];
        if (use_b) p += (i128)b * Xp[g];
        const i64 w = YW[g] - ms_rshift(p, sh);
        YW[g] = w;
        acc += (i128)w * w;
      }
    }
    ms_block_store(acc, tpart, t);
  }
}

// beta^2 -> sp_lanc_tridiag bookkeeping (as k_lanczos_record) + normalisation multiplier
__global__ void k_ms_record(int nsec, const MsSector* secs, ChainMeta* meta, const i64* tpart, int sexp, int k,
                            const double* alpha, double* A, double* Bt, int ld, double tol, double* bnow,
                            int G, int F, i64* mul, int* msh) {
  const int lane = threadIdx.x & 31;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < nsec; s += nw) {
    ChainMeta mt = meta[s];
    if (!mt.active) continue;
    const i128 v = ms_sum_parts_warp(tpart, secs[s].tile0, secs[s].ntile);
    if (lane != 0) continue;
    const double b2 = 0.0 + ms_i128_to_double(v, sexp);
    const double a = alpha[s];
    const double b = sqrt(fmax(b2, 0.0));
    A[(int64_t)s * ld + (k - 1)] = a;
    mt.len = k;
    double invb;
    if (b < tol) {
      mt.active = 0;
      invb = 0.0;
    } else {
      if (k < mt.nlanc) Bt[(int64_t)s * ld + k] = b;
      if (k >= mt.nlanc) mt.active = 0;
      invb = 1.0 / b;
    }
    bnow[s] = b;
    meta[s] = mt;
    i64 m;
    int sh;
    ms_mult(invb, G, F, m, sh);
    mul[s] = m;
    msh[s] = sh;
  }
}

// convergence test of every unfinished sector, one warp per sector
__global__ void k_ms_check(int nsec, ChainMeta* meta, const double* A, const double* Bt, int ld,
                           const double* bnow, double* svec, double* theta, double* resid, int* state,
                           int* mconv, double tol, int* undone) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int s = warp; s < nsec; s += nw) {
    if (state[s]) continue;
    const ChainMeta mt = meta[s];
    const int kk = mt.len;
    if (kk < 1) {  // zero start vector: report as finished without a value
      if (lane == 0) { state[s] = 2; theta[s] = INFINITY; mconv[s] = 0; }
      continue;
    }
    warp_tri_lowest(A + (int64_t)s * ld, Bt + (int64_t)s * ld, kk, bnow[s], theta + s,
                    svec + (int64_t)s * 5 * ld, resid + s);
    __syncwarp();
    if (lane == 0) {
      const double th = theta[s];
      if (!mt.active || resid[s] <= tol * fmax(1.0, fabs(th))) {
        state[s] = 1;
        mconv[s] = kk;
        meta[s].active = 0;
      } else {
        atomicAdd(undone, 1);
      }
    }
  }
}

void ms_launch_start(const MsGroup& gp, uint64_t seed, int F, i64* R, i64* X, i64* tpart, ChainMeta* meta,
                     i64* mul, int* msh, cudaStream_t st) {
  count_launch_external();
  count_launch_external();
  count_launch_external();
  const int nb = std::min(gp.ntiles, 152 * 8);
  k_ms_start_raw<<<nb, 256, 0, st>>>(gp.secs, gp.tsec, gp.tstart, gp.ntiles, seed, R, tpart);
  k_ms_start_norm<<<(gp.nsec + 127) / 128, 128, 0, st>>>(gp.nsec, gp.secs, tpart, F, meta, mul, msh);
  k_ms_apply<<<nb, 256, 0, st>>>(gp.secs, gp.tsec, gp.tstart, gp.ntiles, meta, mul, msh, 1, R, X);
}

void ms_launch_step(const MsGroup& gp, const FxScales& fs, int K, int k, double tol, MsBufs& b, cudaStream_t st) {
  const int nb = std::min(gp.ntiles, 152 * 8);
  const int sb = (gp.nsec * 32 + 127) / 128;  // one warp per sector
  for (int q = 0; q < 5; q++) count_launch_external();
  switch (K) {
    case 1: k_ms_hxv<1><<<nb, 256, 0, st>>>(gp.secs, gp.tsec, gp.tstart, gp.ntiles, b.meta, b.X, b.YW, b.tpart); break;
    case 2: k_ms_hxv<2><<<nb, 256, 0, st>>>(gp.secs, gp.tsec, gp.tstart, gp.ntiles, b.meta, b.X, b.YW, b.tpart); break;
    case 3: k_ms_hxv<3><<<nb, 256, 0, st>>>(gp.secs, gp.tsec, gp.tstart, gp.ntiles, b.meta, b.X, b.YW, b.tpart); break;
    default: k_ms_hxv<4><<<nb, 256, 0, st>>>(gp.secs, gp.tsec, gp.tstart, gp.ntiles, b.meta, b.X, b.YW, b.tpart); break;
  }
  k_ms_alpha<<<sb, 128, 0, st>>>(gp.nsec, gp.secs, b.meta, b.tpart, fs.F + fs.G, fs.C, b.bnow, b.alpha, b.afx, b.bfx);
  k_ms_update<<<nb, 256, 0, st>>>(gp.secs, gp.tsec, gp.tstart, gp.ntiles, b.meta, fs.C + fs.F - fs.G, b.afx,
                                  b.bfx, k > 1 ? 1 : 0, b.X, b.Xp, b.YW, b.tpart);
  k_ms_record<<<sb, 128, 0, st>>>(gp.nsec, gp.secs, b.meta, b.tpart, 2 * fs.G, k, b.alpha, b.A, b.Bt, b.ld, tol,
                                  b.bnow, fs.G, fs.F, b.mul, b.msh);
  // X_next into the old Xp buffer (retired sectors get zeros)
  k_ms_apply<<<nb, 256, 0, st>>>(gp.secs, gp.tsec, gp.tstart, gp.ntiles, b.meta, b.mul, b.msh, 1, b.YW, b.Xp);
  i64* t = b.Xp;
  b.Xp = b.X;
  b.X = t;
}

void ms_launch_check(const MsGroup& gp, MsBufs& b, double tol, cudaStream_t st) {
  count_launch_external();
  const int warps = gp.nsec;
  const int threads = 128;
  const int blocks = std::max(1, (warps * 32 + threads - 1) / threads);
  k_ms_check<<<blocks, threads, 0, st>>>(gp.nsec, b.meta, b.A, b.Bt, b.ld, b.bnow, b.svec, b.theta, b.resid,
                                         b.state, b.mconv, tol, b.undone);
}


// ===========================================================================
// The same batched ground-state search in FP64, real (T = double) or complex
// (T = double2) vectors, for the Hamiltonians the fixed-point path does not
// take (more than 4 hopping magnitudes, complex amplitudes).  The recurrence,
// start vectors and stopping rule are those of the single-sector FP64
// Lanczos (y = H x - beta x_prev, alpha = <x, y>, y -= alpha x, beta = |y|,
// x_next = y / beta); tile partial sums are reduced in a fixed order, so the
// run is deterministic.
// ===========================================================================
namespace {
__device__ __forceinline__ double m64_re(double a, double b) { return a * b; }
__device__ __forceinline__ double m64_re(double2 a, double2 b) { return a.x * b.x + a.y * b.y; }
__device__ __forceinline__ double m64_axpy(double y, double s, double x) { return fma(-s, x, y); }
__device__ __forceinline__ double2 m64_axpy(double2 y, double s, double2 x) {
  return make_double2(fma(-s, x.x, y.x), fma(-s, x.y, y.y));
}
__device__ __forceinline__ double m64_scale(double x, double f) { return x * f; }
__device__ __forceinline__ double2 m64_scale(double2 x, double f) { return make_double2(x.x * f, x.y * f); }
__device__ __forceinline__ void m64_set(double& x, double v) { x = v; }
__device__ __forceinline__ void m64_set(double2& x, double v) { x = make_double2(v, 0.0); }
__device__ __forceinline__ double m64_cfma(double2 a, double x, double acc) { return fma(a.x, x, acc); }
__device__ __forceinline__ double2 m64_cfma(double2 a, double2 x, double2 acc) {
  acc.x = fma(a.x, x.x, acc.x);
  acc.x = fma(-a.y, x.y, acc.x);
  acc.y = fma(a.x, x.y, acc.y);
  acc.y = fma(a.y, x.x, acc.y);
  return acc;
}
__device__ __forceinline__ double m64_diag(double d_re, double, double x) { return d_re * x; }
__device__ __forceinline__ double2 m64_diag(double d_re, double d_im, double2 x) {
  return make_double2(d_re * x.x - d_im * x.y, d_re * x.y + d_im * x.x);
}

// fixed-order block reduction of one double per thread into tpart[t]
__device__ __forceinline__ void m64_block_store(double v, double* tpart, int t) {
  __shared__ double red[256];
  red[threadIdx.x] = v;
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) tpart[t] = red[0];
  __syncthreads();
}
// fixed-order warp sum of the tile partials of one sector
__device__ __forceinline__ double m64_sum_tiles(const double* tpart, int t0, int n) {
  const int lane = threadIdx.x & 31;
  double s = 0.0;
  for (int t = t0 + lane; t < t0 + n; t += 32) s += tpart[t];
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
  return s;
}
}  // namespace

// start vector (the values of the single-sector path) and its |x|^2 partials
template <typename T>
__global__ void k_m64_start(const MsSector* secs, const int* tsec, const int64_t* tstart, int ntiles, uint64_t seed,
                            T* X, double* tpart) {
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const MsSector& S = secs[tsec[t]];
    const int64_t i0 = tstart[t], i1 = min(i0 + (int64_t)MS_TILE, S.D);
    double acc = 0.0;
    for (int64_t i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
      const uint64_t z = ms_splitmix64(seed + 0xD1B54A32D192ED03ull * (uint64_t)S.isector + (uint64_t)i);
      const double v = (double)(z >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0;
      m64_set(X[S.off + i], v);
      acc += v * v;
    }
    m64_block_store(acc, tpart, t);
  }
}
// per sector: 1/|x| (0 and retired when the start vector vanishes)
__global__ void k_m64_norm(int nsec, const MsSector* secs, const double* tpart, ChainMeta* meta, double* invn) {
  const int lane = threadIdx.x & 31;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < nsec; s += nw) {
    const double n2 = m64_sum_tiles(tpart, secs[s].tile0, secs[s].ntile);
    if (lane == 0) {
      if (n2 > 0.0) {
        invn[s] = 1.0 / sqrt(n2);
      } else {
        invn[s] = 0.0;
        meta[s].active = 0;
        meta[s].len = 0;
      }
    }
  }
}
// Xo = f[sector] Xi (f = 0 for retired sectors)
template <typename T>
__global__ void k_m64_scale(const MsSector* secs, const int* tsec, const int64_t* tstart, int ntiles, const double* f,
                            const T* Xi, T* Xo) {
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int s = tsec[t];
    const MsSector& S = secs[s];
    const int64_t i0 = tstart[t], i1 = min(i0 + (int64_t)MS_TILE, S.D);
    const double fs = f[s];
    for (int64_t i = i0 + threadIdx.x; i < i1; i += blockDim.x) Xo[S.off + i] = m64_scale(Xi[S.off + i], fs);
  }
}
// y = H x - beta x_prev and the <x, y> partials (the stored H x v of
// VCA_HAMILTONIAN_SPARSE_HxV.f90:152-200, one element per thread)
template <typename T>
__global__ void __launch_bounds__(256) k_m64_hxv(const MsSector* secs, const int* tsec, const int64_t* tstart,
                                                 int ntiles, MixedDiag md, const ChainMeta* meta,
                                                 const double* bnow, int use_b, const T* __restrict__ X,
                                                 const T* __restrict__ Xp, T* __restrict__ Y, double* tpart) {
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int s = tsec[t];
    double acc = 0.0;
    if (meta[s].active) {
      const MsSector& S = secs[s];
      const SectorView& sv = S.sv;
      const int64_t Dsec = (int64_t)sv.dimup * sv.dimdw;
      const int64_t i0 = tstart[t], i1 = min(i0 + (int64_t)MS_TILE, S.D);
      const double b = use_b ? bnow[s] : 0.0;
      for (int64_t i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
        // a [re; im] task (ncomp 2) applies the real H to each half
        const int64_t cb = (i >= Dsec) ? Dsec : 0;
        const T* x = X + S.off + cb;
        const int64_t ii = i - cb;
        const int idw = (int)(ii / sv.dimup);
        const int iup = (int)(ii - (int64_t)idw * sv.dimup);
        const double dre = sv.up_e1[iup].x + sv.dw_e1[idw].x +
                           mixed_diag(md, (unsigned)sv.up_words[iup], (unsigned)sv.dw_words[idw]);
        const double dim_ = sv.up_e1[iup].y + sv.dw_e1[idw].y;
        const T xi = x[ii];
        T y = m64_diag(dre, dim_, xi);
        const int nu = sv.up_cnt[iup], nd = sv.dw_cnt[idw];
        const int64_t colbase = (int64_t)idw * sv.dimup;
        for (int k = 0; k < nu; k++) {
          const int src = sv.up_src[(int64_t)k * sv.dimup + iup];
          y = m64_cfma(sv.up_amp[(int64_t)k * sv.dimup + iup], x[colbase + src], y);
        }
        for (int k = 0; k < nd; k++) {
          const int src = sv.dw_src[(int64_t)k * sv.dimdw + idw];
          y = m64_cfma(sv.dw_amp[(int64_t)k * sv.dimdw + idw], x[(int64_t)iup + (int64_t)src * sv.dimup], y);
        }
        if (use_b) y = m64_axpy(y, b, Xp[S.off + i]);
        Y[S.off + i] = y;
        acc += m64_re(xi, y);
      }
    }
    m64_block_store(acc, tpart, t);
  }
}
__global__ void k_m64_alpha(int nsec, const MsSector* secs, const ChainMeta* meta, const double* tpart,
                            double* alpha) {
  const int lane = threadIdx.x & 31;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < nsec; s += nw) {
    if (!meta[s].active) continue;
    const double a = m64_sum_tiles(tpart, secs[s].tile0, secs[s].ntile);
    if (lane == 0) alpha[s] = a;
  }
}
// y -= alpha x and the |y|^2 partials
template <typename T>
__global__ void k_m64_update(const MsSector* secs, const int* tsec, const int64_t* tstart, int ntiles,
                             const ChainMeta* meta, const double* alpha, const T* X, T* Y, double* tpart) {
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int s = tsec[t];
    double acc = 0.0;
    if (meta[s].active) {
      const MsSector& S = secs[s];
      const int64_t i0 = tstart[t], i1 = min(i0 + (int64_t)MS_TILE, S.D);
      const double a = alpha[s];
      for (int64_t i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
        const T y = m64_axpy(Y[S.off + i], a, X[S.off + i]);
        Y[S.off + i] = y;
        acc += m64_re(y, y);
      }
    }
    m64_block_store(acc, tpart, t);
  }
}
// beta -> the sp_lanc_tridiag bookkeeping (as k_lanczos_record) and 1/beta
__global__ void k_m64_record(int nsec, const MsSector* secs, ChainMeta* meta, const double* tpart, int k,
                             const double* alpha, double* A, double* Bt, int ld, double tol, double* bnow,
                             double* invb) {
  const int lane = threadIdx.x & 31;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < nsec; s += nw) {
    ChainMeta mt = meta[s];
    if (!mt.active) {
      if (lane == 0) invb[s] = 0.0;
      continue;
    }
    const double b2 = m64_sum_tiles(tpart, secs[s].tile0, secs[s].ntile);
    if (lane != 0) continue;
    const double b = sqrt(fmax(b2, 0.0));
    A[(int64_t)s * ld + (k - 1)] = alpha[s];
    mt.len = k;
    double ib;
    if (b < tol) {
      mt.active = 0;
      ib = 0.0;
    } else {
      if (k < mt.nlanc) Bt[(int64_t)s * ld + k] = b;
      if (k >= mt.nlanc) mt.active = 0;
      ib = 1.0 / b;
    }
    bnow[s] = b;
    invb[s] = ib;
    meta[s] = mt;
  }
}

template <typename T>
static void m64_start_t(const MsGroup& gp, uint64_t seed, Ms64Bufs& b, cudaStream_t st) {
  for (int q = 0; q < 3; q++) count_launch_external();
  const int nb = std::min(gp.ntiles, 152 * 8);
  const int sb = (gp.nsec * 32 + 127) / 128;
  k_m64_start<T><<<nb, 256, 0, st>>>(gp.secs, gp.tsec, gp.tstart, gp.ntiles, seed, (T*)b.X, b.tpart);
  k_m64_norm<<<sb, 128, 0, st>>>(gp.nsec, gp.secs, b.tpart, b.meta, b.invb);
  k_m64_scale<T><<<nb, 256, 0, st>>>(gp.secs, gp.tsec, gp.tstart, gp.ntiles, b.invb, (const T*)b.X, (T*)b.X);
}
template <typename T>
static void m64_step_t(const MsGroup& gp, const MixedDiag& md, int k, double tol, Ms64Bufs& b, cudaStream_t st) {
  for (int q = 0; q < 5; q++) count_launch_external();
  const int nb = std::min(gp.ntiles, 152 * 8);
  const int sb = (gp.nsec * 32 + 127) / 128;
  k_m64_hxv<T><<<nb, 256, 0, st>>>(gp.secs, gp.tsec, gp.tstart, gp.ntiles, md, b.meta, b.bnow, k > 1 ? 1 : 0,
                                   (const T*)b.X, (const T*)b.Xp, (T*)b.Y, b.tpart);
  k_m64_alpha<<<sb, 128, 0, st>>>(gp.nsec, gp.secs, b.meta, b.tpart, b.alpha);
  k_m64_update<T><<<nb, 256, 0, st>>>(gp.secs, gp.tsec, gp.tstart, gp.ntiles, b.meta, b.alpha, (const T*)b.X,
                                      (T*)b.Y, b.tpart);
  k_m64_record<<<sb, 128, 0, st>>>(gp.nsec, gp.secs, b.meta, b.tpart, k, b.alpha, b.A, b.Bt, b.ld, tol, b.bnow,
                                   b.invb);
  // x_next = y / beta into the old x_prev buffer (retired sectors get zeros)
  k_m64_scale<T><<<nb, 256, 0, st>>>(gp.secs, gp.tsec, gp.tstart, gp.ntiles, b.invb, (const T*)b.Y, (T*)b.Xp);
  void* t = b.Xp;
  b.Xp = b.X;
  b.X = t;
}

void m64_launch_start(const MsGroup& gp, bool cplx, uint64_t seed, Ms64Bufs& b, cudaStream_t st) {
  if (cplx) m64_start_t<double2>(gp, seed, b, st);
  else m64_start_t<double>(gp, seed, b, st);
}
void m64_launch_step(const MsGroup& gp, bool cplx, const MixedDiag& md, int k, double tol, Ms64Bufs& b,
                     cudaStream_t st) {
  if (cplx) m64_step_t<double2>(gp, md, k, tol, b, st);
  else m64_step_t<double>(gp, md, k, tol, b, st);
}
void m64_launch_check(const MsGroup& gp, Ms64Bufs& b, double tol, cudaStream_t st) {
  count_launch_external();
  const int threads = 128;
  const int blocks = std::max(1, (gp.nsec * 32 + threads - 1) / threads);
  k_ms_check<<<blocks, threads, 0, st>>>(gp.nsec, b.meta, b.A, b.Bt, b.ld, b.bnow, b.svec, b.theta, b.resid,
                                         b.state, b.mconv, tol, b.undone);
}

// ---- multi-task helpers of the batched form --------------------------------
__global__ void k_mt_norm(int nsec, const MsSector* secs, const double* tpart, ChainMeta* meta, double* n2,
                          double* invn) {
  const int lane = threadIdx.x & 31;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < nsec; s += nw) {
    const double v = m64_sum_tiles(tpart, secs[s].tile0, secs[s].ntile);
    if (lane == 0) {
      n2[s] = v;
      if (v > 0.0) {
        invn[s] = 1.0 / sqrt(v);
      } else {
        invn[s] = 0.0;
        meta[s].active = 0;
        meta[s].len = 0;
      }
    }
  }
}
template <typename T>
__global__ void k_m64_psi(const MsSector* secs, const int* tsec, const int64_t* tstart, int ntiles,
                          const double* svec, int ld5, const int* mconv, int k, const T* X, T* psi) {
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int s = tsec[t];
    if (k > mconv[s]) continue;
    const MsSector& S = secs[s];
    const int64_t i0 = tstart[t], i1 = min(i0 + (int64_t)MS_TILE, S.D);
    const double w = svec[(int64_t)s * ld5 + (k - 1)];
    for (int64_t i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
      T p = psi[S.off + i];
      p = m64_axpy(p, -w, X[S.off + i]);
      psi[S.off + i] = p;
    }
  }
}
template <typename T>
__global__ void k_m64_sqnorm(const MsSector* secs, const int* tsec, const int64_t* tstart, int ntiles, const T* X,
                             double* tpart) {
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const MsSector& S = secs[tsec[t]];
    const int64_t i0 = tstart[t], i1 = min(i0 + (int64_t)MS_TILE, S.D);
    double acc = 0.0;
    for (int64_t i = i0 + threadIdx.x; i < i1; i += blockDim.x) acc += m64_re(X[S.off + i], X[S.off + i]);
    m64_block_store(acc, tpart, t);
  }
}

void mt_launch_norm(const MsGroup& gp, const double* tpart, ChainMeta* meta, double* n2, double* invn,
                    cudaStream_t st) {
  count_launch_external();
  k_mt_norm<<<(gp.nsec * 32 + 127) / 128, 128, 0, st>>>(gp.nsec, gp.secs, tpart, meta, n2, invn);
}
void m64_launch_scale(const MsGroup& gp, bool cplx, const double* f, const void* Xi, void* Xo, cudaStream_t st) {
  count_launch_external();
  const int nb = std::min(gp.ntiles, 152 * 8);
  if (cplx)
    k_m64_scale<double2><<<nb, 256, 0, st>>>(gp.secs, gp.tsec, gp.tstart, gp.ntiles, f, (const double2*)Xi,
                                            (double2*)Xo);
  else
    k_m64_scale<double><<<nb, 256, 0, st>>>(gp.secs, gp.tsec, gp.tstart, gp.ntiles, f, (const double*)Xi,
                                           (double*)Xo);
}
void m64_launch_psi(const MsGroup& gp, bool cplx, const double* svec, int ld5, const int* mconv, int k,
                    const void* X, void* psi, cudaStream_t st) {
  count_launch_external();
  const int nb = std::min(gp.ntiles, 152 * 8);
  if (cplx)
    k_m64_psi<double2><<<nb, 256, 0, st>>>(gp.secs, gp.tsec, gp.tstart, gp.ntiles, svec, ld5, mconv, k,
                                          (const double2*)X, (double2*)psi);
  else
    k_m64_psi<double><<<nb, 256, 0, st>>>(gp.secs, gp.tsec, gp.tstart, gp.ntiles, svec, ld5, mconv, k,
                                         (const double*)X, (double*)psi);
}
void m64_launch_sqnorm(const MsGroup& gp, bool cplx, const void* X, double* tpart, cudaStream_t st) {
  count_launch_external();
  const int nb = std::min(gp.ntiles, 152 * 8);
  if (cplx)
    k_m64_sqnorm<double2><<<nb, 256, 0, st>>>(gp.secs, gp.tsec, gp.tstart, gp.ntiles, (const double2*)X, tpart);
  else
    k_m64_sqnorm<double><<<nb, 256, 0, st>>>(gp.secs, gp.tsec, gp.tstart, gp.ntiles, (const double*)X, tpart);
}

}  // namespace vca
