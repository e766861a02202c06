// vca_batch.cu -- the Lanczos phases of multi-task column batches (the
// Green's-function chains of the batched form, vca_batch.cuh).
//
// The recurrence is the single-sector column batch's (lanczos_step:
// y = H x - beta x_prev, alpha = <x, y>, y -= alpha x, beta = |y|,
// x_next = y / beta; VCA_GF_NORMAL.f90:218-223 through sp_lanc_tridiag), the
// stored semantics of H x v (VCA_HAMILTONIAN_SPARSE_HxV.f90:152-200); only
// the tiling differs: one launch per phase covers every task of the group.
#include "vca_batch.cuh"

namespace vca {

void count_launch_external();

namespace {

__device__ __forceinline__ double bre(double a, double b) { return a * b; }
__device__ __forceinline__ double bre(double2 a, double2 b) { return a.x * b.x + a.y * b.y; }
__device__ __forceinline__ double bfma(double2 a, double x, double acc) { return fma(a.x, x, acc); }
__device__ __forceinline__ double2 bfma(double2 a, double2 x, double2 acc) {
  acc.x = fma(a.x, x.x, acc.x);
  acc.x = fma(-a.y, x.y, acc.x);
  acc.y = fma(a.x, x.y, acc.y);
  acc.y = fma(a.y, x.x, acc.y);
  return acc;
}
__device__ __forceinline__ double bdiag(double dre, double, double x) { return dre * x; }
__device__ __forceinline__ double2 bdiag(double dre, double dim, double2 x) {
  return make_double2(dre * x.x - dim * x.y, dre * x.y + dim * x.x);
}
__device__ __forceinline__ double baxpy(double y, double s, double x) { return fma(-s, x, y); }
__device__ __forceinline__ double2 baxpy(double2 y, double s, double2 x) {
  return make_double2(fma(-s, x.x, y.x), fma(-s, x.y, y.y));
}
__device__ __forceinline__ double bscale(double x, double f) { return x * f; }
__device__ __forceinline__ double2 bscale(double2 x, double f) { return make_double2(x.x * f, x.y * f); }

// the (tile, column) partial of the row lanes of each column, fixed order
__device__ __forceinline__ void tile_col_store(double v, double* tpart, int64_t idx, bool ok) {
  __shared__ double red[MC_BY_MAX][33];
  red[threadIdx.y][threadIdx.x] = v;
  __syncthreads();
  if (threadIdx.y == 0 && ok) {
    double s = 0.0;
    for (int y = 0; y < (int)blockDim.y; y++) s += red[y][threadIdx.x];
    tpart[idx] = s;
  }
  __syncthreads();
}

template <typename T>
__global__ void __launch_bounds__(512) k_mc_hxv(McGroup gp, MixedDiag md, const ChainMeta* meta, const double* bnow,
                                                int use_b, const T* __restrict__ X, const T* __restrict__ Xp,
                                                T* __restrict__ Y, double* tpart) {
  for (int tile = blockIdx.x; tile < gp.ntiles; tile += gridDim.x) {
    const McTask tk = gp.tasks[gp.tile_task[tile]];
    const SectorView& sv = tk.sv;
    const int64_t r0 = gp.tile_row0[tile], r1 = gp.tile_row1[tile];
    const T* x = X + tk.xoff;
    for (int cb = 0; cb < tk.m; cb += 32) {
      const int c = cb + threadIdx.x;
      const bool ok = c < tk.m;
      const int ch = ok ? gp.col_chain[tk.col0 + c] : 0;
      const double b = (ok && use_b) ? bnow[ch] : 0.0;
      double acc = 0.0;
      for (int64_t i = r0 + threadIdx.y; i < r1; i += blockDim.y) {
        const int idw = (int)(i / sv.dimup);
        const int iup = (int)(i - (int64_t)idw * sv.dimup);
        if (!ok) continue;
        const double dre = sv.up_e1[iup].x + sv.dw_e1[idw].x +
                           mixed_diag(md, (unsigned)sv.up_words[iup], (unsigned)sv.dw_words[idw]);
        const double dim_ = sv.up_e1[iup].y + sv.dw_e1[idw].y;
        const T xi = x[i * tk.m + c];
        T y = bdiag(dre, dim_, xi);
        const int nu = sv.up_cnt[iup], nd = sv.dw_cnt[idw];
        const int64_t colbase = (int64_t)idw * sv.dimup;
        for (int k = 0; k < nu; k++) {
          const int s = sv.up_src[(int64_t)k * sv.dimup + iup];
          y = bfma(sv.up_amp[(int64_t)k * sv.dimup + iup], x[(colbase + s) * tk.m + c], y);
        }
        for (int k = 0; k < nd; k++) {
          const int s = sv.dw_src[(int64_t)k * sv.dimdw + idw];
          y = bfma(sv.dw_amp[(int64_t)k * sv.dimdw + idw], x[((int64_t)iup + (int64_t)s * sv.dimup) * tk.m + c], y);
        }
        if (use_b) y = baxpy(y, b, Xp[tk.xoff + i * tk.m + c]);
        Y[tk.xoff + i * tk.m + c] = y;
        acc += bre(xi, y);
      }
      if (ok && !meta[ch].active) acc = 0.0;
      tile_col_store(acc, tpart, tk.part0 + (int64_t)c * tk.ntile + (tile - tk.tile0), ok);
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(512) k_mc_update(McGroup gp, const ChainMeta* meta, const double* alpha,
                                                   const T* __restrict__ X, T* __restrict__ Y, double* tpart) {
  for (int tile = blockIdx.x; tile < gp.ntiles; tile += gridDim.x) {
    const McTask tk = gp.tasks[gp.tile_task[tile]];
    const int64_t r0 = gp.tile_row0[tile], r1 = gp.tile_row1[tile];
    for (int cb = 0; cb < tk.m; cb += 32) {
      const int c = cb + threadIdx.x;
      const bool ok = c < tk.m;
      const int ch = ok ? gp.col_chain[tk.col0 + c] : 0;
      const bool act = ok && meta[ch].active;
      const double a = act ? alpha[ch] : 0.0;
      double acc = 0.0;
      if (act)
        for (int64_t i = r0 + threadIdx.y; i < r1; i += blockDim.y) {
          const int64_t e = tk.xoff + i * tk.m + c;
          const T y = baxpy(Y[e], a, X[e]);
          Y[e] = y;
          acc += bre(y, y);
        }
      tile_col_store(acc, tpart, tk.part0 + (int64_t)c * tk.ntile + (tile - tk.tile0), ok);
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(512) k_mc_scale(McGroup gp, const ChainMeta* meta, const double* f,
                                                  const T* __restrict__ Xi, T* __restrict__ Xo) {
  for (int tile = blockIdx.x; tile < gp.ntiles; tile += gridDim.x) {
    const McTask tk = gp.tasks[gp.tile_task[tile]];
    const int64_t r0 = gp.tile_row0[tile], r1 = gp.tile_row1[tile];
    for (int cb = 0; cb < tk.m; cb += 32) {
      const int c = cb + threadIdx.x;
      if (c >= tk.m) continue;
      const int ch = gp.col_chain[tk.col0 + c];
      const double a = meta[ch].active ? f[ch] : 0.0;  // retired chains get zero columns
      for (int64_t i = r0 + threadIdx.y; i < r1; i += blockDim.y) {
        const int64_t e = tk.xoff + i * tk.m + c;
        Xo[e] = bscale(Xi[e], a);
      }
    }
  }
}

// one warp per chain: its columns in order, lanes over the task's tiles, then
// a fixed xor tree
__global__ void k_mc_reduce(McGroup gp, const double* tpart, double* out) {
  const int lane = threadIdx.x & 31;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int ch = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; ch < gp.nch; ch += nw) {
    const McChain cc = gp.chains[ch];
    const McTask tk = gp.tasks[cc.task];
    double s = 0.0;
    for (int q = 0; q < cc.ncol; q++) {
      const int c = cc.col0 + q;
      const double* pc = tpart + tk.part0 + (int64_t)c * tk.ntile;  // the column's tiles, contiguous
      for (int t = lane; t < tk.ntile; t += 32) s += pc[t];
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    if (lane == 0) out[ch] = s;
  }
}

inline int nblk_tiles(int ntiles) { return ntiles < 152 * 8 ? ntiles : 152 * 8; }

}  // namespace

void mc_launch_reduce(const McGroup& gp, const double* tpart, double* out, cudaStream_t st) {
  count_launch_external();
  k_mc_reduce<<<(gp.nch * 32 + 127) / 128, 128, 0, st>>>(gp, tpart, out);
}
void mc_launch_hxv(const McGroup& gp, bool cplx, const MixedDiag& md, const ChainMeta* meta, const double* bnow,
                   int use_b, const void* X, const void* Xp, void* Y, double* tpart, cudaStream_t st) {
  count_launch_external();
  const dim3 blk(32, gp.by);
  if (cplx)
    k_mc_hxv<double2><<<nblk_tiles(gp.ntiles), blk, 0, st>>>(gp, md, meta, bnow, use_b, (const double2*)X,
                                                             (const double2*)Xp, (double2*)Y, tpart);
  else
    k_mc_hxv<double><<<nblk_tiles(gp.ntiles), blk, 0, st>>>(gp, md, meta, bnow, use_b, (const double*)X,
                                                            (const double*)Xp, (double*)Y, tpart);
}
void mc_launch_update(const McGroup& gp, bool cplx, const ChainMeta* meta, const double* alpha, const void* X,
                      void* Y, double* tpart, cudaStream_t st) {
  count_launch_external();
  const dim3 blk(32, gp.by);
  if (cplx)
    k_mc_update<double2><<<nblk_tiles(gp.ntiles), blk, 0, st>>>(gp, meta, alpha, (const double2*)X, (double2*)Y,
                                                                tpart);
  else
    k_mc_update<double><<<nblk_tiles(gp.ntiles), blk, 0, st>>>(gp, meta, alpha, (const double*)X, (double*)Y, tpart);
}
void mc_launch_scale(const McGroup& gp, bool cplx, const ChainMeta* meta, const double* f, const void* Xi, void* Xo,
                     cudaStream_t st) {
  count_launch_external();
  const dim3 blk(32, gp.by);
  if (cplx)
    k_mc_scale<double2><<<nblk_tiles(gp.ntiles), blk, 0, st>>>(gp, meta, f, (const double2*)Xi, (double2*)Xo);
  else
    k_mc_scale<double><<<nblk_tiles(gp.ntiles), blk, 0, st>>>(gp, meta, f, (const double*)Xi, (double*)Xo);
}

}  // namespace vca
