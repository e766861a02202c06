// vca_kernels.cu -- sm_103a kernels of the cluster-ED -> Lanczos GF -> Omega
// path (GB300).  Every grid is bounded by its buffers: grid-stride loops over
// explicit 64-bit extents, no device-side waits.
#include "vca_kernels.cuh"
#include "vca_fx.cuh"
#include "vca_tri.cuh"
#include "vca_multi.cuh"
#include "vca_batch.cuh"

#include <cmath>
#include <atomic>
#include <cstdio>

namespace vca {

static std::atomic<long long> g_launches{0};
long long launch_count() { return g_launches.load(); }
#define COUNT_LAUNCH() g_launches.fetch_add(1, std::memory_order_relaxed)
void count_launch_external() { COUNT_LAUNCH(); }

__constant__ int64_t c_binom[VCA_MAX_NS + 1][VCA_MAX_NS + 1];

static inline int nblocks(int64_t n, int threads, int cap = 152 * 16) {
  int64_t b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > cap) b = cap;
  return (int)b;
}

void set_binomials(int Ns, cudaStream_t st) {
  static Binom h;
  for (int n = 0; n <= VCA_MAX_NS; n++)
    for (int k = 0; k <= VCA_MAX_NS; k++) {
      if (k > n) { h.c[n][k] = 0; continue; }
      int64_t v = 1;
      for (int t = 1; t <= k; t++) v = v * (n + 1 - t) / t;
      h.c[n][k] = v;
    }
  (void)Ns;
  cudaMemcpyToSymbolAsync(c_binom, &h, sizeof(h), 0, cudaMemcpyHostToDevice, st);
}

// colex rank of a Fock word: sum_t C(pos_t, t) over set bits (ascending)
__device__ __forceinline__ int rank_word(unsigned w) {
  int64_t r = 0;
  int t = 1;
  while (w) {
    int p = __ffs(w) - 1;
    r += c_binom[p][t];
    t++;
    w &= w - 1;
  }
  return (int)r;
}

__device__ __forceinline__ double parity(unsigned x) { return (__popc(x) & 1) ? -1.0 : 1.0; }

// ---------------------------------------------------------------------------
// Fock maps: ascending words of popcount n (build_sector, VCA_SETUP.f90:660-695)
// ---------------------------------------------------------------------------
__global__ void k_build_words(int Ns, int n, int dim, int* words) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < dim; r += gridDim.x * blockDim.x) {
    int64_t rr = r;
    unsigned w = 0;
    for (int t = n; t >= 1; --t) {
      int p = Ns - 1;
      while (p >= t && c_binom[p][t] > rr) --p;  // largest p with C(p,t) <= rr
      w |= 1u << p;
      rr -= c_binom[p][t];
    }
    words[r] = (int)w;
  }
}
void launch_build_words(int Ns, int n, int dim, int* words, cudaStream_t st) {
  COUNT_LAUNCH();
  k_build_words<<<nblocks(dim, 256), 256, 0, st>>>(Ns, n, dim, words);
}

// ---------------------------------------------------------------------------
// Pull hop tables.  Row = target word w; a pair (i <- j) with amplitude A of
// c^dag_i c_j contributes when bit i is set and bit j clear in w; the source
// is ws = w - i + j and the element is A * sg1 * sg2 with the one-word sign
// convention of c/cdg (VCA_SETUP.f90:724-750): sg1 from bits of ws below j,
// sg2 from bits of (ws without j) below i.  Same elements as the stored
// spH0ups/spH0dws of VCA_HAMILTONIAN/stored/H_cluster_up.f90 (cluster :1-28,
// bath :30-55, hybridisation :57-86) enumerated by target instead of source.
// ---------------------------------------------------------------------------
__global__ void k_hop_count(int dim, const int* words, const HopPair* pairs, int npairs, int* cnt,
                            int* gmax) {
  int local_max = 0;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < dim; r += gridDim.x * blockDim.x) {
    unsigned w = (unsigned)words[r];
    int c = 0;
    for (int q = 0; q < npairs; q++) {
      HopPair p = pairs[q];
      if (((w >> p.i) & 1u) && !((w >> p.j) & 1u)) c++;
    }
    cnt[r] = c;
    local_max = max(local_max, c);
  }
  atomicMax(gmax, local_max);
}
int launch_hop_count(int Ns, int n, int dim, const int* words, const HopPair* d_pairs, int npairs,
                     int* cnt, int* d_scratch_max, cudaStream_t st) {
  COUNT_LAUNCH();
  (void)Ns;
  (void)n;
  cudaMemsetAsync(d_scratch_max, 0, sizeof(int), st);
  k_hop_count<<<nblocks(dim, 256), 256, 0, st>>>(dim, words, d_pairs, npairs, cnt, d_scratch_max);
  int h = 0;
  cudaMemcpyAsync(&h, d_scratch_max, sizeof(int), cudaMemcpyDeviceToHost, st);
  cudaStreamSynchronize(st);
  return h;
}

__global__ void k_hop_fill(int dim, int width, const int* words, const HopPair* pairs, int npairs,
                           int* src, double2* amp) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < dim; r += gridDim.x * blockDim.x) {
    unsigned w = (unsigned)words[r];
    int c = 0;
    for (int q = 0; q < npairs && c < width; q++) {
      HopPair p = pairs[q];
      if (!(((w >> p.i) & 1u) && !((w >> p.j) & 1u))) continue;
      unsigned ws = (w ^ (1u << p.i)) | (1u << p.j);
      double sg1 = parity(ws & ((1u << p.j) - 1u));
      unsigned k1 = ws & ~(1u << p.j);
      double sg2 = parity(k1 & ((1u << p.i) - 1u));
      double sg = sg1 * sg2;
      src[(int64_t)c * dim + r] = rank_word(ws);
      amp[(int64_t)c * dim + r] = make_double2(p.re * sg, p.im * sg);
      c++;
    }
    for (; c < width; c++) {  // padding never read (cnt[r] bounds the loop)
      src[(int64_t)c * dim + r] = 0;
      amp[(int64_t)c * dim + r] = make_double2(0.0, 0.0);
    }
  }
}
void launch_hop_fill(int Ns, int n, int dim, int width, const int* words, const HopPair* d_pairs,
                     int npairs, int* src, double2* amp, cudaStream_t st) {
  COUNT_LAUNCH();
  (void)Ns;
  (void)n;
  if (width == 0) return;
  k_hop_fill<<<nblocks(dim, 256), 256, 0, st>>>(dim, width, words, d_pairs, npairs, src, amp);
}

// one-body + same-spin energy of a word (H_cluster_local.f90:19-25,46-55,59-76,84-92)
__global__ void k_e1(int dim, const int* words, E1Params p, int with_const, double2* e1) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < dim; r += gridDim.x * blockDim.x) {
    unsigned w = (unsigned)words[r];
    double er = 0.0, ei = 0.0;
    unsigned x = w;
    while (x) {
      int b = __ffs(x) - 1;
      er += p.eps[b].x;
      ei += p.eps[b].y;
      x &= x - 1;
    }
    int same = 0;
    for (int o = 0; o < p.norb; o++)
      for (int q = o + 1; q < p.norb; q++) same += __popc(w & p.omask[o] & (w >> (q - o)));
    er += p.upar * same;
    if (with_const) { er += p.cst.x; ei += p.cst.y; }
    e1[r] = make_double2(er, ei);
  }
}
void launch_e1(int dim, const int* words, const E1Params& p, bool with_const, double2* e1,
               cudaStream_t st) {
  COUNT_LAUNCH();
  k_e1<<<nblocks(dim, 256), 256, 0, st>>>(dim, words, p, with_const ? 1 : 0, e1);
}

// ---------------------------------------------------------------------------
// H x v on a column batch: Y = d o X + H_up X + X H_dw^T per column, the
// stored product of VCA_HAMILTONIAN_SPARSE_HxV.f90:152-200 with the diagonal
// of H_cluster_local.f90 computed on the fly from the two words.
// Thread block = CW columns x RB rows; each thread walks its rows and its
// columns c = tx, tx+CW, ... (neighbour loads are contiguous across tx).
// ---------------------------------------------------------------------------
__global__ void k_hxv_real(SectorView sv, MixedDiag md, int m, const double* __restrict__ X,
                           double* __restrict__ Y) {
  const int64_t D = (int64_t)sv.dimup * sv.dimdw;
  const int CW = blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.y + threadIdx.y; i < D;
       i += (int64_t)gridDim.x * blockDim.y) {
    const int idw = (int)(i / sv.dimup);
    const int iup = (int)(i - (int64_t)idw * sv.dimup);
    const double d = sv.up_e1[iup].x + sv.dw_e1[idw].x +
                     mixed_diag(md, (unsigned)sv.up_words[iup], (unsigned)sv.dw_words[idw]);
    const int nu = sv.up_cnt[iup], nd = sv.dw_cnt[idw];
    const int64_t colbase = (int64_t)idw * sv.dimup;
    for (int c = threadIdx.x; c < m; c += CW) {
      double acc = d * X[i * m + c];
      for (int k = 0; k < nu; k++) {
        const int s = sv.up_src[(int64_t)k * sv.dimup + iup];
        acc = fma(sv.up_amp[(int64_t)k * sv.dimup + iup].x, X[(colbase + s) * m + c], acc);
      }
      for (int k = 0; k < nd; k++) {
        const int s = sv.dw_src[(int64_t)k * sv.dimdw + idw];
        acc = fma(sv.dw_amp[(int64_t)k * sv.dimdw + idw].x, X[((int64_t)iup + (int64_t)s * sv.dimup) * m + c], acc);
      }
      Y[i * m + c] = acc;
    }
  }
}

__device__ __forceinline__ double2 cfma(double2 a, double2 x, double2 acc) {
  acc.x = fma(a.x, x.x, acc.x);
  acc.x = fma(-a.y, x.y, acc.x);
  acc.y = fma(a.x, x.y, acc.y);
  acc.y = fma(a.y, x.x, acc.y);
  return acc;
}

__global__ void k_hxv_cplx(SectorView sv, MixedDiag md, int m, const double2* __restrict__ X,
                           double2* __restrict__ Y) {
  const int64_t D = (int64_t)sv.dimup * sv.dimdw;
  const int CW = blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.y + threadIdx.y; i < D;
       i += (int64_t)gridDim.x * blockDim.y) {
    const int idw = (int)(i / sv.dimup);
    const int iup = (int)(i - (int64_t)idw * sv.dimup);
    double2 d = make_double2(sv.up_e1[iup].x + sv.dw_e1[idw].x +
                                 mixed_diag(md, (unsigned)sv.up_words[iup], (unsigned)sv.dw_words[idw]),
                             sv.up_e1[iup].y + sv.dw_e1[idw].y);
    const int nu = sv.up_cnt[iup], nd = sv.dw_cnt[idw];
    const int64_t colbase = (int64_t)idw * sv.dimup;
    for (int c = threadIdx.x; c < m; c += CW) {
      double2 acc = cfma(d, X[i * m + c], make_double2(0.0, 0.0));
      for (int k = 0; k < nu; k++) {
        const int s = sv.up_src[(int64_t)k * sv.dimup + iup];
        acc = cfma(sv.up_amp[(int64_t)k * sv.dimup + iup], X[(colbase + s) * m + c], acc);
      }
      for (int k = 0; k < nd; k++) {
        const int s = sv.dw_src[(int64_t)k * sv.dimdw + idw];
        acc = cfma(sv.dw_amp[(int64_t)k * sv.dimdw + idw], X[((int64_t)iup + (int64_t)s * sv.dimup) * m + c], acc);
      }
      Y[i * m + c] = acc;
    }
  }
}

static void col_shape(int m, dim3& blk) {
  int cw = 1;
  while (cw < m && cw < 32) cw <<= 1;
  blk = dim3(cw, 256 / cw, 1);
}
void launch_hxv_real(const SectorView& sv, const MixedDiag& md, int m, const double* X, double* Y,
                     cudaStream_t st) {
  COUNT_LAUNCH();
  dim3 blk;
  col_shape(m, blk);
  int64_t D = (int64_t)sv.dimup * sv.dimdw;
  k_hxv_real<<<nblocks(D, blk.y, 152 * 32), blk, 0, st>>>(sv, md, m, X, Y);
}
void launch_hxv_cplx(const SectorView& sv, const MixedDiag& md, int m, const double2* X, double2* Y,
                     cudaStream_t st) {
  COUNT_LAUNCH();
  dim3 blk;
  col_shape(m, blk);
  int64_t D = (int64_t)sv.dimup * sv.dimdw;
  k_hxv_cplx<<<nblocks(D, blk.y, 152 * 32), blk, 0, st>>>(sv, md, m, X, Y);
}

// ---------------------------------------------------------------------------
// Column-batch vector operations.  Reductions are two-stage with a fixed
// grid: per-block partials, then a per-column sum in block order, so a
// repeated run reproduces the same bits.
// ---------------------------------------------------------------------------
template <bool CPLX>
__global__ void k_col_dot(int64_t rows, int m, const void* Xv, const void* Yv, double* partial) {
  extern __shared__ double sh[];
  const int CW = blockDim.x, RB = blockDim.y;
  const int c = blockIdx.y * CW + threadIdx.x;
  double s = 0.0;
  if (c < m) {
    for (int64_t i = (int64_t)blockIdx.x * RB + threadIdx.y; i < rows; i += (int64_t)gridDim.x * RB) {
      if (CPLX) {
        double2 x = ((const double2*)Xv)[i * m + c], y = ((const double2*)Yv)[i * m + c];
        s = fma(x.x, y.x, s);
        s = fma(x.y, y.y, s);
      } else {
        s = fma(((const double*)Xv)[i * m + c], ((const double*)Yv)[i * m + c], s);
      }
    }
  }
  sh[threadIdx.y * CW + threadIdx.x] = s;
  __syncthreads();
  for (int h = RB / 2; h > 0; h >>= 1) {
    if (threadIdx.y < h) sh[threadIdx.y * CW + threadIdx.x] += sh[(threadIdx.y + h) * CW + threadIdx.x];
    __syncthreads();
  }
  if (threadIdx.y == 0 && c < m) partial[(int64_t)blockIdx.x * m + c] = sh[threadIdx.x];
}
__global__ void k_col_reduce(int m, int nblk, const double* partial, double* out) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < m; c += gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int b = 0; b < nblk; b++) s += partial[(int64_t)b * m + c];
    out[c] = s;
  }
}
void launch_col_dot(const ColBatch& b, const void* X, const void* Y, double* partial, int nblk,
                    double* out_col, cudaStream_t st) {
  COUNT_LAUNCH();
  dim3 blk;
  col_shape(b.m, blk);
  dim3 grd(nblk, (b.m + blk.x - 1) / blk.x, 1);
  size_t shm = sizeof(double) * 256;
  if (b.cplx)
    k_col_dot<true><<<grd, blk, shm, st>>>(b.rows, b.m, X, Y, partial);
  else
    k_col_dot<false><<<grd, blk, shm, st>>>(b.rows, b.m, X, Y, partial);
  COUNT_LAUNCH();
  k_col_reduce<<<nblocks(b.m, 128), 128, 0, st>>>(b.m, nblk, partial, out_col);
}

template <bool CPLX>
__global__ void k_col_axpy(int64_t rows, int m, const int* col2ch, const ChainMeta* meta,
                           const double* coef, double sgn, const void* Xv, void* Yv) {
  const int64_t n = rows * m;
  for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < n;
       g += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(g % m);
    const int ch = col2ch[c];
    if (!meta[ch].active) continue;
    const double a = sgn * coef[ch];
    if (CPLX) {
      double2 x = ((const double2*)Xv)[g];
      double2& y = ((double2*)Yv)[g];
      y.x = fma(a, x.x, y.x);
      y.y = fma(a, x.y, y.y);
    } else {
      ((double*)Yv)[g] = fma(a, ((const double*)Xv)[g], ((double*)Yv)[g]);
    }
  }
}
void launch_col_axpy(const ColBatch& b, const double* coef, const void* X, void* Y, bool negate,
                     cudaStream_t st) {
  COUNT_LAUNCH();
  int64_t n = b.rows * b.m;
  if (b.cplx)
    k_col_axpy<true><<<nblocks(n, 256), 256, 0, st>>>(b.rows, b.m, b.col2ch, b.meta, coef,
                                                      negate ? -1.0 : 1.0, X, Y);
  else
    k_col_axpy<false><<<nblocks(n, 256), 256, 0, st>>>(b.rows, b.m, b.col2ch, b.meta, coef,
                                                       negate ? -1.0 : 1.0, X, Y);
}

template <bool CPLX>
__global__ void k_col_scale(int64_t rows, int m, const int* col2ch, const ChainMeta* meta,
                            const double* scale, const void* Yv, void* Xv) {
  const int64_t n = rows * m;
  for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < n;
       g += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(g % m);
    const int ch = col2ch[c];
    // retired chains get zero columns, so later products on them stay finite
    const double a = meta[ch].active ? scale[ch] : 0.0;
    if (CPLX) {
      double2 y = ((const double2*)Yv)[g];
      ((double2*)Xv)[g] = make_double2(a * y.x, a * y.y);
    } else {
      ((double*)Xv)[g] = a * ((const double*)Yv)[g];
    }
  }
}
void launch_col_scale(const ColBatch& b, const double* scale, const void* Y, void* X, cudaStream_t st) {
  COUNT_LAUNCH();
  int64_t n = b.rows * b.m;
  if (b.cplx)
    k_col_scale<true><<<nblocks(n, 256), 256, 0, st>>>(b.rows, b.m, b.col2ch, b.meta, scale, Y, X);
  else
    k_col_scale<false><<<nblocks(n, 256), 256, 0, st>>>(b.rows, b.m, b.col2ch, b.meta, scale, Y, X);
}

__global__ void k_chain_sum(int nch, const ChainMeta* meta, const double* in_col, double* out) {
  for (int ch = blockIdx.x * blockDim.x + threadIdx.x; ch < nch; ch += gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int q = 0; q < meta[ch].ncol; q++) s += in_col[meta[ch].col0 + q];
    out[ch] = s;
  }
}
void launch_chain_sum(const ColBatch& b, const double* in_col, double* out_ch, cudaStream_t st) {
  COUNT_LAUNCH();
  k_chain_sum<<<nblocks(b.nch, 128), 128, 0, st>>>(b.nch, b.meta, in_col, out_ch);
}

// sp_lanc_tridiag bookkeeping (SciFortran, restated): alpha_k stored, the
// chain stops when beta_{k+1} < tol, otherwise beta_{k+1} -> Bt[k] for k < nlanc.
__global__ void k_lanczos_record(int nch, ChainMeta* meta, int k, const double* alpha_ch,
                                 const double* beta2_ch, double* A, double* Bt, int ldab, double tol,
                                 double* invbeta, double* beta_now) {
  for (int ch = blockIdx.x * blockDim.x + threadIdx.x; ch < nch; ch += gridDim.x * blockDim.x) {
    ChainMeta mt = meta[ch];
    if (!mt.active) continue;
    const double a = alpha_ch[ch];
    const double b = sqrt(fmax(beta2_ch[ch], 0.0));
    A[(int64_t)ch * ldab + (k - 1)] = a;
    mt.len = k;
    if (b < tol) {
      mt.active = 0;
      invbeta[ch] = 0.0;
      beta_now[ch] = b;
    } else {
      if (k < mt.nlanc) Bt[(int64_t)ch * ldab + k] = b;
      if (k >= mt.nlanc) mt.active = 0;
      invbeta[ch] = 1.0 / b;
      beta_now[ch] = b;
    }
    meta[ch] = mt;
  }
}
void launch_lanczos_record(int nch, ChainMeta* meta, int k, const double* alpha_ch,
                           const double* beta2_ch, double* A, double* Bt, int ldab, double tol,
                           double* invbeta, double* beta_now, cudaStream_t st) {
  COUNT_LAUNCH();
  k_lanczos_record<<<nblocks(nch, 128), 128, 0, st>>>(nch, meta, k, alpha_ch, beta2_ch, A, Bt, ldab,
                                                      tol, invbeta, beta_now);
}

template <bool CPLX>
__global__ void k_psi_accum(int64_t n, const double* s, int k, const void* Xv, void* Pv) {
  const double a = s[k];
  for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < n;
       g += (int64_t)gridDim.x * blockDim.x) {
    if (CPLX) {
      double2 x = ((const double2*)Xv)[g];
      double2& p = ((double2*)Pv)[g];
      p.x = fma(a, x.x, p.x);
      p.y = fma(a, x.y, p.y);
    } else {
      ((double*)Pv)[g] = fma(a, ((const double*)Xv)[g], ((double*)Pv)[g]);
    }
  }
}
void launch_psi_accum(int64_t n, bool cplx, const double* s, int k, const void* X, void* psi,
                      cudaStream_t st) {
  COUNT_LAUNCH();
  if (cplx)
    k_psi_accum<true><<<nblocks(n, 256), 256, 0, st>>>(n, s, k, X, psi);
  else
    k_psi_accum<false><<<nblocks(n, 256), 256, 0, st>>>(n, s, k, X, psi);
}

// splitmix64 (Steele, Lea & Flood 2014) of (seed, sector, index) -> [-1, 1)
__device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
  uint64_t z = x + 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__global__ void k_start_vector(int64_t n, uint64_t seed, int isector, double* X) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    uint64_t z = splitmix64(seed + 0xD1B54A32D192ED03ull * (uint64_t)isector + (uint64_t)i);
    X[i] = (double)(z >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0;
  }
}
void launch_start_vector(int64_t n, uint64_t seed, int isector, double* X, cudaStream_t st) {
  COUNT_LAUNCH();
  k_start_vector<<<nblocks(n, 256), 256, 0, st>>>(n, seed, isector, X);
}
__global__ void k_fill(int64_t n, double v, double* X) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    X[i] = v;
}
void launch_fill(int64_t n, double v, double* X, cudaStream_t st) {
  COUNT_LAUNCH();
  k_fill<<<nblocks(n, 256), 256, 0, st>>>(n, v, X);
}

// ---------------------------------------------------------------------------
// Lowest eigenpair of the Lanczos T_k (one warp, vca_tri.cuh)
// ---------------------------------------------------------------------------
__global__ void k_tri_lowest(const double* A, const double* Bt, int k, double btail, double* theta_out,
                             double* s, double* resid) {
  warp_tri_lowest(A, Bt, k, btail, theta_out, s, resid);
}
void launch_tri_lowest(const double* A, const double* Bt, int k, double btail, double* theta,
                       double* s, double* resid, cudaStream_t st) {
  COUNT_LAUNCH();
  k_tri_lowest<<<1, 32, 0, st>>>(A, Bt, k, btail, theta, s, resid);
}

// ---------------------------------------------------------------------------
// Chain store: the tridiagonal (alpha, beta) of every Green's function chain,
// with its prefactor norm^2/zeta, sign (+1 particle, -1 hole), channel
// weight factor and ground-state energy.  G'(z) is evaluated from it as a
// continued fraction; poles and weights (add_to_lanczos_gf_normal,
// VCA_GF_NORMAL.f90:970-1033) are formed from it only when a caller asks for
// them.
// ---------------------------------------------------------------------------
__global__ void k_chain_store(int nch, const ChainMeta* meta, const double* A, const double* Bt, int ldab,
                              const double* norm2, const double2* wfac, const int* isign, double Ei,
                              double boltz, double zeta, ChainStore cs, int base) {
  const int ch = blockIdx.x;
  if (ch >= nch) return;
  const int n = meta[ch].len;
  const int64_t o = (int64_t)(base + ch) * cs.ld;
  for (int j = threadIdx.x; j < cs.ld; j += blockDim.x) {
    cs.A[o + j] = (j < n) ? A[(int64_t)ch * ldab + j] : 0.0;
    cs.B[o + j] = (j < n) ? Bt[(int64_t)ch * ldab + j] : 0.0;
  }
  if (threadIdx.x == 0) {
    cs.n[base + ch] = n;
    cs.pes[base + ch] = norm2[ch] * boltz / zeta;  // vnorm2*exp(-beta(Ei-Egs))/zeta
    cs.isign[base + ch] = isign[ch];
    cs.wfac[base + ch] = wfac[ch];
    cs.Ei[base + ch] = Ei;
  }
}
void launch_chain_store(int nch, const ChainMeta* meta, const double* A, const double* Bt, int ldab,
                        const double* norm2, const double2* wfac, const int* isign, double Ei, double boltz,
                        double zeta, const ChainStore& cs, int base, cudaStream_t st) {
  if (nch <= 0) return;
  COUNT_LAUNCH();
  k_chain_store<<<nch, 128, 0, st>>>(nch, meta, A, Bt, ldab, norm2, wfac, isign, Ei, boltz, zeta, cs, base);
}

// Chain tridiagonal -> poles and weights.  Implicit QL with Wilkinson shift
// (EISPACK tql2; the reference calls SciFortran eigh(d,e,Ev=Z) at
// VCA_GF_NORMAL.f90:1012) tracking only the first row of Z.  One thread per
// chain, one warp per block; work = 3*ld doubles per chain.  A chain whose
// QL needs more than max_iter sweeps for one eigenvalue is counted in *fail
// (its poles are then not to be used: the host turns the count into an error).
__global__ void k_chain_poles(int nch, ChainStore cs, double* work, double* poles, double2* weights,
                              int* nexc, int max_iter, int* fail) {
  const int ldab = cs.ld;
  for (int ch = blockIdx.x * blockDim.x + threadIdx.x; ch < nch; ch += gridDim.x * blockDim.x) {
    const int n = cs.n[ch];
    nexc[ch] = n;
    if (n <= 0) continue;
    double* d = work + (int64_t)ch * 3 * ldab;
    double* e = d + ldab;
    double* z = e + ldab;
    for (int i = 0; i < n; i++) {
      d[i] = cs.A[(int64_t)ch * ldab + i];
      e[i] = (i + 1 < n) ? cs.B[(int64_t)ch * ldab + i + 1] : 0.0;  // e[i] couples i,i+1
      z[i] = (i == 0) ? 1.0 : 0.0;
    }
    double f = 0.0, tst1 = 0.0;
    const double eps = 2.220446049250313e-16;
    bool failed = false;
    for (int l = 0; l < n; l++) {
      int iter = 0;
      double h = fabs(d[l]) + fabs(e[l]);
      if (tst1 < h) tst1 = h;
      int m = l;
      while (m < n - 1 && fabs(e[m]) > eps * tst1) m++;
      if (m > l) {
        do {
          if (++iter > max_iter) { failed = true; break; }
          double g = d[l];
          double p = (d[l + 1] - g) / (2.0 * e[l]);
          double r = hypot(p, 1.0);
          double sr = (p >= 0.0) ? r : -r;
          d[l] = e[l] / (p + sr);
          d[l + 1] = e[l] * (p + sr);
          double dl1 = d[l + 1];
          h = g - d[l];
          for (int i = l + 2; i < n; i++) d[i] -= h;
          f += h;
          p = d[m];
          double c = 1.0, c2 = 1.0, c3 = 1.0, el1 = e[l + 1], s = 0.0, s2 = 0.0;
          for (int i = m - 1; i >= l; i--) {
            c3 = c2;
            c2 = c;
            s2 = s;
            g = c * e[i];
            h = c * p;
            r = hypot(p, e[i]);
            e[i + 1] = s * r;
            s = e[i] / r;
            c = p / r;
            p = c * d[i] - s * g;
            d[i + 1] = h + s * (c * g + s * d[i]);
            double zi1 = z[i + 1], zi = z[i];
            z[i + 1] = s * zi + c * zi1;
            z[i] = c * zi - s * zi1;
          }
          p = -s * s2 * c3 * el1 * e[l] / dl1;
          e[l] = s * p;
          d[l] = c * p;
        } while (fabs(e[l]) > eps * tst1);
      }
      d[l] += f;
      e[l] = 0.0;
    }
    if (failed) atomicAdd(fail, 1);
    for (int ii = 1; ii < n; ii++) {  // ascending, as tql2
      int i = ii - 1, kk = i;
      double p = d[i];
      for (int j = ii; j < n; j++) if (d[j] < p) { kk = j; p = d[j]; }
      if (kk != i) {
        d[kk] = d[i];
        d[i] = p;
        double t = z[i];
        z[i] = z[kk];
        z[kk] = t;
      }
    }
    const double2 wf = cs.wfac[ch];
    const double pes = cs.pes[ch];
    const double Ei = cs.Ei[ch];
    const double sg = (double)cs.isign[ch];
    for (int j = 0; j < n; j++) {
      double w2 = z[j] * z[j] * pes;
      poles[(int64_t)ch * ldab + j] = sg * (d[j] - Ei);
      weights[(int64_t)ch * ldab + j] = make_double2(wf.x * w2, wf.y * w2);
    }
  }
}
void launch_chain_poles(int nch, const ChainStore& cs, double* work, double* poles, double2* weights, int* nexc,
                        int max_iter, int* fail, cudaStream_t st) {
  if (nch <= 0) return;
  COUNT_LAUNCH();
  k_chain_poles<<<nblocks(nch, 32), 32, 0, st>>>(nch, cs, work, poles, weights, nexc, max_iter, fail);
}

// ---------------------------------------------------------------------------
// Chain start vectors by gather: target row t, term (pos, coef): for c^dag
// the target spin word must hold pos and the source is w - pos; for c it must
// not and the source is w + pos.  sign = parity of source bits below pos
// (cdg/c, VCA_SETUP.f90:724-750) -- the same bits as in the target word.
// ---------------------------------------------------------------------------
template <bool GSC, bool COLC>
__global__ void k_chain_init(SectorView tgt, int src_dimup, const void* gsv, int nchain,
                             const ChainInit* ci, int m, void* Xv) {
  const int64_t D = (int64_t)tgt.dimup * tgt.dimdw;
  const int64_t n = D * nchain;
  const int W = fx_slab_w(m);  // slab-major batch
  for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < n;
       g += (int64_t)gridDim.x * blockDim.x) {
    const int ch = (int)(g % nchain);
    const int64_t i = g / nchain;
    const int idw = (int)(i / tgt.dimup);
    const int iup = (int)(i - (int64_t)idw * tgt.dimup);
    const ChainInit c = ci[ch];
    const unsigned w = (unsigned)(c.spin == 0 ? tgt.up_words[iup] : tgt.dw_words[idw]);
    double vr = 0.0, vi = 0.0;
    for (int q = 0; q < c.nterm; q++) {
      const int pos = c.t[q].pos;
      const bool occ = (w >> pos) & 1u;
      if (c.dag ? !occ : occ) continue;
      const unsigned ws = w ^ (1u << pos);
      const double sg = parity(ws & ((1u << pos) - 1u));
      const int rs = rank_word(ws);
      const int64_t si = (c.spin == 0) ? ((int64_t)rs + (int64_t)idw * src_dimup)
                                       : ((int64_t)iup + (int64_t)rs * src_dimup);
      double gr, gi;
      if (GSC) { double2 gv = ((const double2*)gsv)[si]; gr = gv.x; gi = gv.y; }
      else { gr = ((const double*)gsv)[si]; gi = 0.0; }
      // (coef * sg) * gs
      const double ar = c.t[q].re * sg, ai = c.t[q].im * sg;
      vr += ar * gr - ai * gi;
      vi += ar * gi + ai * gr;
    }
    if (COLC) {
      ((double2*)Xv)[i * m + c.col0] = make_double2(vr, vi);
    } else {
      ((double*)Xv)[i * m + c.col0] = vr;
      if (c.cplxcol) ((double*)Xv)[i * m + c.col0 + 1] = vi;
    }
  }
}
// The gather for the column tasks of the batched chains (vca_batch.cuh):
// column c of a task is part re/im of its chain's start vector.
template <typename T>
__global__ void __launch_bounds__(512) k_mc_chain_init(McGroup gp, T* X, double* tpart) {
  __shared__ double red[MC_BY_MAX][33];
  for (int tile = blockIdx.x; tile < gp.ntiles; tile += gridDim.x) {
    const McTask tk = gp.tasks[gp.tile_task[tile]];
    const SectorView& tgt = tk.sv;
    const int64_t r0 = gp.tile_row0[tile], r1 = gp.tile_row1[tile];
    for (int cb = 0; cb < tk.m; cb += 32) {
      const int c = cb + threadIdx.x;
      const bool ok = c < tk.m;
      double acc = 0.0;
      if (ok) {
        const int ch = gp.col_chain[tk.col0 + c];
        const int part = gp.col_part[tk.col0 + c];
        const MtChain op = gp.chains[ch].op;
        for (int64_t i = r0 + threadIdx.y; i < r1; i += blockDim.y) {
          const int idw = (int)(i / tgt.dimup);
          const int iup = (int)(i - (int64_t)idw * tgt.dimup);
          const unsigned w = (unsigned)(op.spin == 0 ? tgt.up_words[iup] : tgt.dw_words[idw]);
          double vr = 0.0, vi = 0.0;
          for (int q = 0; q < op.nterm; q++) {
            const int pos = op.pos[q];
            const bool occ = (w >> pos) & 1u;
            if (op.dag ? !occ : occ) continue;
            const unsigned ws = w ^ (1u << pos);
            const double sg = parity(ws & ((1u << pos) - 1u));
            const int rs = rank_word(ws);
            const int64_t si = (op.spin == 0) ? ((int64_t)rs + (int64_t)idw * op.src_dimup)
                                              : ((int64_t)iup + (int64_t)rs * op.src_dimup);
            double gr, gi = 0.0;
            if (sizeof(T) == sizeof(double2)) {
              const double2 gv = ((const double2*)op.gs)[si];
              gr = gv.x;
              gi = gv.y;
            } else {
              gr = ((const double*)op.gs)[si];
            }
            const double ar = op.cre[q] * sg, ai = op.cim[q] * sg;
            vr += ar * gr - ai * gi;
            vi += ar * gi + ai * gr;
          }
          const int64_t e = tk.xoff + i * tk.m + c;
          if (sizeof(T) == sizeof(double2)) {
            ((double2*)X)[e] = make_double2(vr, vi);
            acc += vr * vr + vi * vi;
          } else {
            const double v = part ? vi : vr;
            ((double*)X)[e] = v;
            acc += v * v;
          }
        }
      }
      red[threadIdx.y][threadIdx.x] = acc;
      __syncthreads();
      if (threadIdx.y == 0 && ok) {
        double sum = 0.0;
        for (int y = 0; y < (int)blockDim.y; y++) sum += red[y][threadIdx.x];
        tpart[tk.part0 + (int64_t)c * tk.ntile + (tile - tk.tile0)] = sum;
      }
      __syncthreads();
    }
  }
}
void mc_launch_chain_init(const McGroup& gp, bool cplx, void* X, double* tpart, cudaStream_t st) {
  COUNT_LAUNCH();
  const int nb = gp.ntiles < 152 * 8 ? gp.ntiles : 152 * 8;
  if (cplx) k_mc_chain_init<double2><<<nb, dim3(32, gp.by), 0, st>>>(gp, (double2*)X, tpart);
  else k_mc_chain_init<double><<<nb, dim3(32, gp.by), 0, st>>>(gp, (double*)X, tpart);
}

void launch_chain_init(const SectorView& tgt, int src_dimup, const void* gs, bool gs_cplx,
                       int nchain, const ChainInit* d_ci, int m, bool cols_cplx, void* X,
                       cudaStream_t st) {
  COUNT_LAUNCH();
  int64_t n = (int64_t)tgt.dimup * tgt.dimdw * nchain;
  int nb = nblocks(n, 256);
  if (cols_cplx) {
    if (gs_cplx) k_chain_init<true, true><<<nb, 256, 0, st>>>(tgt, src_dimup, gs, nchain, d_ci, m, X);
    else k_chain_init<false, true><<<nb, 256, 0, st>>>(tgt, src_dimup, gs, nchain, d_ci, m, X);
  } else {
    k_chain_init<false, false><<<nb, 256, 0, st>>>(tgt, src_dimup, gs, nchain, d_ci, m, X);
  }
}

// ---------------------------------------------------------------------------
// Cluster Green's function from poles (vca_gf_cluster_scalar,
// VCA_IO/gf_cluster.f90:23-49) and recombination (:50-62).
// ---------------------------------------------------------------------------
// Per (z, element) thread: sum over the element's chains of
// isign * pes * wfac / (zeta' - a0 - b1^2 / (zeta' - a1 - ...)), zeta' =
// isign*z + Ei: the continued fraction of the chain's tridiagonal, equal to
// the sum over its poles isign*(E_j - Ei) with weights wfac*pes*Z(1,j)^2.
__global__ void k_gf_eval(GfLayout g, int nz, const double2* z, double2* G) {
  const int64_t n = (int64_t)nz * g.nelem;
  const ChainStore& cs = g.cs;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int e = (int)(t % g.nelem);
    const int q = (int)(t / g.nelem);
    double ar = 0.0, ai = 0.0;
    for (int x = g.elem_ptr[e]; x < g.elem_ptr[e + 1]; x++) {
      const int ch = g.elem_chain[x];
      const int np = cs.n[ch];
      if (np <= 0) continue;
      const double sg = (double)cs.isign[ch];
      const double zr = sg * z[q].x + cs.Ei[ch], zi = sg * z[q].y;
      const double* A = cs.A + (int64_t)ch * cs.ld;
      const double* B = cs.B + (int64_t)ch * cs.ld;
      double tr = zr - A[np - 1], ti = zi;
      for (int k = np - 2; k >= 0; k--) {
        const double b2 = B[k + 1] * B[k + 1];
        const double inv = b2 / fma(tr, tr, ti * ti);  // b^2 / t = b^2 conj(t) / |t|^2
        tr = zr - A[k] - tr * inv;
        ti = zi + ti * inv;
      }
      const double inv = 1.0 / fma(tr, tr, ti * ti);
      const double cr = tr * inv, ci = -ti * inv;
      const double f = sg * cs.pes[ch];
      const double2 w = cs.wfac[ch];
      const double wr = w.x * f, wi = w.y * f;
      ar += wr * cr - wi * ci;
      ai += wr * ci + wi * cr;
    }
    G[t] = make_double2(ar, ai);
  }
}
void launch_gf_eval(const GfLayout& g, int nz, const double2* z, double2* G, cudaStream_t st) {
  COUNT_LAUNCH();
  int64_t n = (int64_t)nz * g.nelem;
  k_gf_eval<<<nblocks(n, 128), 128, 0, st>>>(g, nz, z, G);
}

// Pole tables as vca_gf_cluster_scalar sums them (VCA_IO/gf_cluster.f90:
// 30-45): per (z, element) thread, weight/(z - pole) over the element's
// states, channels and excitations in table order; poles and weights complex.
__global__ void k_gf_eval_poles(int nelem, const int64_t* ptr, const double2* poles, const double2* weights,
                                int nz, const double2* z, double2* G) {
  const int64_t n = (int64_t)nz * nelem;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int e = (int)(t % nelem);
    const int q = (int)(t / nelem);
    const double2 zq = z[q];
    double ar = 0.0, ai = 0.0;
    for (int64_t x = ptr[e]; x < ptr[e + 1]; x++) {
      const double dr = zq.x - poles[x].x, di = zq.y - poles[x].y;
      const double inv = 1.0 / fma(dr, dr, di * di);
      const double2 w = weights[x];
      ar += (w.x * dr + w.y * di) * inv;  // w conj(d) / |d|^2
      ai += (w.y * dr - w.x * di) * inv;
    }
    G[t] = make_double2(ar, ai);
  }
}
void launch_gf_eval_poles(int nelem, const int64_t* ptr, const double2* poles, const double2* weights, int nz,
                          const double2* z, double2* G, cudaStream_t st) {
  COUNT_LAUNCH();
  int64_t n = (int64_t)nz * nelem;
  k_gf_eval_poles<<<nblocks(n, 128), 128, 0, st>>>(nelem, ptr, poles, weights, nz, z, G);
}

__global__ void k_gf_assemble(ClusterDims cd, int nz, const double2* Graw, double2* Glso) {
  const int N = cd.N, NN = N * N;
  const int nel = cd.Nlat * cd.Nlat * cd.Nspin * cd.Norb * cd.Norb;
  const int64_t n = (int64_t)nz * NN;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int q = (int)(t / NN);
    const int ab = (int)(t % NN);
    const int a = ab % N, b = ab / N;
    // lso a = io + il*Norb + is*Norb*Nlat (VCA_AUX_FUNX.f90:261-262)
    const int io = a % cd.Norb, il = (a / cd.Norb) % cd.Nlat, is = a / (cd.Norb * cd.Nlat);
    const int jo = b % cd.Norb, jl = (b / cd.Norb) % cd.Nlat, js = b / (cd.Norb * cd.Nlat);
    double2 out = make_double2(0.0, 0.0);
    if (is == js) {
      auto E = [&](int i1, int j1, int o1, int p1) {
        return i1 + cd.Nlat * (j1 + cd.Nlat * (is + cd.Nspin * (o1 + cd.Norb * p1)));
      };
      const double2* G = Graw + (int64_t)q * nel;
      double2 g = G[E(il, jl, io, jo)];
      if (il == jl && io == jo) {
        out = g;
      } else {
        double2 gi = G[E(il, il, io, io)], gj = G[E(jl, jl, jo, jo)];
        double sr = gi.x + gj.x, si = gi.y + gj.y;
        // (1 - i*chan4)*(sr + i si) = (sr + chan4*si) + i(si - chan4*sr)
        const double c4 = (double)cd.chan4;
        out.x = 0.5 * (g.x - (sr + c4 * si));
        out.y = 0.5 * (g.y - (si - c4 * sr));
      }
    }
    Glso[t] = out;
  }
}
void launch_gf_assemble(const ClusterDims& cd, int nz, const double2* Graw, double2* Glso,
                        cudaStream_t st) {
  COUNT_LAUNCH();
  int64_t n = (int64_t)nz * cd.N * cd.N;
  k_gf_assemble<<<nblocks(n, 256), 256, 0, st>>>(cd, nz, Graw, Glso);
}

// complex helpers
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cdiv(double2 a, double2 b) {
  double den = b.x * b.x + b.y * b.y;
  return make_double2((a.x * b.x + a.y * b.y) / den, (a.y * b.x - a.x * b.y) / den);
}

__global__ void k_reduce_rows(int nrows, int ncols, const double* in, double scale, double* out) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < nrows; r += gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int c = 0; c < ncols; c++) s += in[(int64_t)r * ncols + c];
    out[r] = s * scale;
  }
}
void launch_reduce_rows(int nrows, int ncols, const double* in, double scale, double* out,
                        cudaStream_t st) {
  COUNT_LAUNCH();
  k_reduce_rows<<<nblocks(nrows, 128), 128, 0, st>>>(nrows, ncols, in, scale, out);
}

// Gauss-Legendre nodes/weights on (0,1): Newton on P_n from
// cos(pi (i+3/4)/(n+1/2)), ascending nodes.
// Gauss-Legendre nodes/weights on (0,1): Newton on P_n from the classical
// initial guess cos(pi(i+3/4)/(n+1/2)), P_n by the three-term recurrence
// with the reciprocals 1/j from a table (no division in the loop).  Newton
// converges quadratically from that guess; the loop ends once the step is at
// rounding level (at most 12 steps: near +-1 the step need not fall below
// 1e-16) and P_n is evaluated once more for the weight.
__global__ void k_recip_table(int n, double* inv) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j <= n; j += gridDim.x * blockDim.x)
    inv[j] = j ? 1.0 / (double)j : 0.0;
}
__device__ __forceinline__ void legendre_pair(int n, double z, const double* __restrict__ inv, double* pn,
                                              double* pn1) {
  double p1 = 1.0, p2 = 0.0;
  for (int j = 1; j <= n; j++) {
    const double p3 = p2;
    p2 = p1;
    p1 = ((2.0 * j - 1.0) * z * p2 - (j - 1.0) * p3) * inv[j];
  }
  *pn = p1;
  *pn1 = p2;
}
__global__ void k_gauss_legendre(int n, const double* inv, double* x, double* w) {
  const int half = (n + 1) / 2;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < half; i += gridDim.x * blockDim.x) {
    double z = cos(M_PI * (i + 0.75) / (n + 0.5)), p1, p2;
    for (int it = 0; it < 12; it++) {
      legendre_pair(n, z, inv, &p1, &p2);
      const double pp = n * (z * p1 - p2) / (z * z - 1.0);
      const double dz = p1 / pp;
      z -= dz;
      if (fabs(dz) <= 2.5e-16) break;
    }
    legendre_pair(n, z, inv, &p1, &p2);
    const double pp = n * (z * p1 - p2) / (z * z - 1.0);
    const double wt = 2.0 / ((1.0 - z * z) * pp * pp);
    x[i] = 0.5 * (1.0 - z);
    x[n - 1 - i] = 0.5 * (1.0 + z);
    w[i] = 0.5 * wt;
    w[n - 1 - i] = 0.5 * wt;
  }
}
void launch_gauss_legendre(int n, double* inv, double* x, double* w, cudaStream_t st) {
  COUNT_LAUNCH();
  k_recip_table<<<nblocks(n + 1, 256), 256, 0, st>>>(n, inv);
  COUNT_LAUNCH();
  k_gauss_legendre<<<nblocks((n + 1) / 2, 64), 64, 0, st>>>(n, inv, x, w);
}

// Delta_bath(z) = V [(z+xmu) - h]^{-1} V^dag (VCA_BATH_FUNCTIONS.f90:127-150);
// one thread per z, Gauss-Jordan with partial pivoting in `work`
// (2*Nb*Nb complex per z).  hb, V in lso layout (Nb x Nb, N x Nb).
__global__ void k_delta_bath(int nz, const double2* z, int N, int Nb, const double2* hb, const double2* V,
                             double xmu, double2* work, double2* out) {
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nz; q += gridDim.x * blockDim.x) {
    double2* M = work + (int64_t)q * 2 * Nb * Nb;
    double2* I = M + Nb * Nb;
    for (int i = 0; i < Nb; i++)
      for (int j = 0; j < Nb; j++) {
        double2 h = hb[i + j * Nb];
        M[i + j * Nb] = make_double2(-h.x, -h.y);
        I[i + j * Nb] = make_double2(i == j ? 1.0 : 0.0, 0.0);
      }
    for (int i = 0; i < Nb; i++) { M[i + i * Nb].x += z[q].x + xmu; M[i + i * Nb].y += z[q].y; }
    for (int k = 0; k < Nb; k++) {
      int p = k;
      double best = hypot(M[k + k * Nb].x, M[k + k * Nb].y);
      for (int i = k + 1; i < Nb; i++) {
        double mg = hypot(M[i + k * Nb].x, M[i + k * Nb].y);
        if (mg > best) { best = mg; p = i; }
      }
      if (p != k)
        for (int j = 0; j < Nb; j++) {
          double2 t = M[k + j * Nb]; M[k + j * Nb] = M[p + j * Nb]; M[p + j * Nb] = t;
          t = I[k + j * Nb]; I[k + j * Nb] = I[p + j * Nb]; I[p + j * Nb] = t;
        }
      double2 piv = M[k + k * Nb];
      for (int j = 0; j < Nb; j++) { M[k + j * Nb] = cdiv(M[k + j * Nb], piv); I[k + j * Nb] = cdiv(I[k + j * Nb], piv); }
      for (int i = 0; i < Nb; i++) {
        if (i == k) continue;
        double2 f = M[i + k * Nb];
        if (f.x == 0.0 && f.y == 0.0) continue;
        for (int j = 0; j < Nb; j++) {
          double2 t = cmul(f, M[k + j * Nb]);
          M[i + j * Nb].x -= t.x; M[i + j * Nb].y -= t.y;
          t = cmul(f, I[k + j * Nb]);
          I[i + j * Nb].x -= t.x; I[i + j * Nb].y -= t.y;
        }
      }
    }
    // out = V * I * V^dag
    for (int i = 0; i < N; i++)
      for (int j = 0; j < N; j++) {
        double2 s = make_double2(0.0, 0.0);
        for (int a = 0; a < Nb; a++) {
          double2 va = V[i + a * N];
          for (int b = 0; b < Nb; b++) {
            double2 vb = V[j + b * N];
            double2 t = cmul(va, I[a + b * Nb]);
            s.x += t.x * vb.x + t.y * vb.y;  // t * conj(vb)
            s.y += t.y * vb.x - t.x * vb.y;
          }
        }
        out[(int64_t)q * N * N + i + j * N] = s;
      }
  }
}
void launch_delta_bath(int nz, const double2* z, int N, int Nb, const double2* hb, const double2* V,
                       double xmu, double2* work, double2* out, cudaStream_t st) {
  COUNT_LAUNCH();
  k_delta_bath<<<nblocks(nz, 64), 64, 0, st>>>(nz, z, N, Nb, hb, V, xmu, work, out);
}


// ---------------------------------------------------------------------------
// small helpers
// ---------------------------------------------------------------------------
// chain start-vector norms: invnorm = 1/sqrt(norm2); a zero-norm chain is
// retired with no excitations (the reference would divide by zero).
__global__ void k_chain_norm_init(int nch, ChainMeta* meta, const double* norm2, double* invnorm) {
  for (int ch = blockIdx.x * blockDim.x + threadIdx.x; ch < nch; ch += gridDim.x * blockDim.x) {
    double n2 = norm2[ch];
    if (n2 > 0.0) {
      invnorm[ch] = 1.0 / sqrt(n2);
    } else {
      invnorm[ch] = 0.0;
      meta[ch].active = 0;
      meta[ch].len = 0;
    }
  }
}
void launch_chain_norm_init(int nch, ChainMeta* meta, const double* norm2, double* invnorm,
                            cudaStream_t st) {
  COUNT_LAUNCH();
  k_chain_norm_init<<<nblocks(nch, 128), 128, 0, st>>>(nch, meta, norm2, invnorm);
}
__global__ void k_recip(int n, const double* in, double* out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    out[i] = (in[i] != 0.0) ? 1.0 / in[i] : 0.0;
}
void launch_recip(int n, const double* in, double* out, cudaStream_t st) {
  COUNT_LAUNCH();
  k_recip<<<nblocks(n, 128), 128, 0, st>>>(n, in, out);
}
// (Nlat,Nlat,Nspin,Nspin,Norb,Norb[,L]) -> lso N x N per slice (VCA_AUX_FUNX.f90:255-279)
__global__ void k_nnn2lso(int Nlat, int Nspin, int Norb, int64_t L, const double2* in, double2* out) {
  const int N = Nlat * Nspin * Norb;
  const int64_t NN = (int64_t)N * N;
  const int64_t n = NN * L;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t l = t / NN;
    const int ab = (int)(t % NN);
    const int a = ab % N, b = ab / N;
    const int io = a % Norb, il = (a / Norb) % Nlat, is = a / (Norb * Nlat);
    const int jo = b % Norb, jl = (b / Norb) % Nlat, js = b / (Norb * Nlat);
    const int64_t src = il + (int64_t)Nlat * (jl + (int64_t)Nlat * (is + (int64_t)Nspin *
                        (js + (int64_t)Nspin * (io + (int64_t)Norb * jo))));
    out[t] = in[l * NN + src];
  }
}
void launch_nnn2lso(int Nlat, int Nspin, int Norb, int64_t L, const double2* in, double2* out,
                    cudaStream_t st) {
  COUNT_LAUNCH();
  const int N = Nlat * Nspin * Norb;
  k_nnn2lso<<<nblocks((int64_t)N * N * L, 256), 256, 0, st>>>(Nlat, Nspin, Norb, L, in, out);
}
// P[w] = D[w] + H (lso), or H alone when D == nullptr
__global__ void k_add_hloc(int nw, int NN, const double2* D, const double2* H, double2* P) {
  const int64_t n = (int64_t)nw * NN;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    double2 h = H[t % NN];
    if (D) { h.x += D[t].x; h.y += D[t].y; }
    P[t] = h;
  }
}
void launch_add_hloc(int nw, int NN, const double2* D, const double2* H, double2* P, cudaStream_t st) {
  COUNT_LAUNCH();
  k_add_hloc<<<nblocks((int64_t)nw * NN, 256), 256, 0, st>>>(nw, NN, D, H, P);
}
// omega nodes: z = i*scale*s/(1-s), W = w*scale/(1-s)^2
__global__ void k_omega_nodes(int n, double scale, const double* s, const double* w, double2* z,
                              double* W) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double om = 1.0 - s[i];
    z[i] = make_double2(0.0, scale * s[i] / om);
    W[i] = w[i] * scale / (om * om);
  }
}
void launch_omega_nodes(int n, double scale, const double* s, const double* w, double2* z, double* W,
                        cudaStream_t st) {
  COUNT_LAUNCH();
  k_omega_nodes<<<nblocks(n, 128), 128, 0, st>>>(n, scale, s, w, z, W);
}
// deterministic weighted sum: out = sum_i a[i]*b[i] (single block)
__global__ void k_wsum(int n, const double* a, const double* b, double* out) {
  __shared__ double sh[256];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s = fma(a[i], b[i], s);
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h) sh[threadIdx.x] += sh[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = sh[0];
}
void launch_wsum(int n, const double* a, const double* b, double* out, cudaStream_t st) {
  COUNT_LAUNCH();
  k_wsum<<<1, 256, 0, st>>>(n, a, b, out);
}
// complex start vector (real values, zero imaginary part)
__global__ void k_real_to_cplx(int64_t n, const double* in, double2* out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = make_double2(in[i], 0.0);
}
void launch_real_to_cplx(int64_t n, const double* in, double2* out, cudaStream_t st) {
  COUNT_LAUNCH();
  k_real_to_cplx<<<nblocks(n, 256), 256, 0, st>>>(n, in, out);
}


// Fixed-point chain start vectors: the chain operators carry coefficients in
// {+-1, +-i}, so the gather from a fixed-point ground state is exact.
__global__ void k_chain_init_fx(SectorView tgt, int src_dimup, const long long* gs, int nchain,
                                const ChainInit* ci, int m, int swapped, const int* pinv, long long* X) {
  const int64_t D = (int64_t)tgt.dimup * tgt.dimdw;
  const int64_t n = D * nchain;
  const int W = fx_slab_w(m);  // slab-major batch
  for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < n;
       g += (int64_t)gridDim.x * blockDim.x) {
    const int ch = (int)(g % nchain);
    const int64_t i = g / nchain;
    const int idw = (int)(i / tgt.dimup);
    const int iup = (int)(i - (int64_t)idw * tgt.dimup);
    const ChainInit c = ci[ch];
    const unsigned w = (unsigned)(c.spin == 0 ? tgt.up_words[iup] : tgt.dw_words[idw]);
    long long vr = 0, vi = 0;
    for (int q = 0; q < c.nterm; q++) {
      const int pos = c.t[q].pos;
      const bool occ = (w >> pos) & 1u;
      if (c.dag ? !occ : occ) continue;
      const unsigned ws = w ^ (1u << pos);
      const bool neg = __popc(ws & ((1u << pos) - 1u)) & 1;
      const int rs = rank_word(ws);
      const int64_t si = (c.spin == 0) ? ((int64_t)rs + (int64_t)idw * src_dimup)
                                       : ((int64_t)iup + (int64_t)rs * src_dimup);
      const long long gv = neg ? -gs[si] : gs[si];
      const int cr = (int)c.t[q].re, cim = (int)c.t[q].im;  // in {-1,0,1}
      vr += cr * gv;
      vi += cim * gv;
    }
    // batch row: fast spin role (up, or down when swapped) first, its index
    // replaced by its position in the hop-count order when pinv is given
    const int fa = swapped ? idw : iup, fb = swapped ? iup : idw;
    const int64_t io = (int64_t)(pinv ? pinv[fa] : fa) + (int64_t)fb * (swapped ? tgt.dimdw : tgt.dimup);
    X[fx_off(D, W, io, c.col0)] = vr;
    if (c.cplxcol) X[fx_off(D, W, io, c.col0 + 1)] = vi;
  }
}
void launch_chain_init_fx(const SectorView& tgt, int src_dimup, const long long* gs, int nchain,
                          const ChainInit* d_ci, int m, bool swapped, const int* pinv, long long* X,
                          cudaStream_t st) {
  COUNT_LAUNCH();
  int64_t n = (int64_t)tgt.dimup * tgt.dimdw * nchain;
  k_chain_init_fx<<<nblocks(n, 256), 256, 0, st>>>(tgt, src_dimup, gs, nchain, d_ci, m, swapped ? 1 : 0, pinv,
                                                   X);
}


// ---------------------------------------------------------------------------
// Omega integrand, lane-parallel form.  Per (w, k, spin block) one warp:
//  A = M G with M = P_w - Hk_k restricted to the union sparsity pattern of
//  M over all k (rowptr/cols, within-block columns), one lane per element;
//  ln|det(1+A)| by LU with the trailing update spread over all 32 lanes.
//  ||A||_inf < 1/2: no pivoting, identity implicit, prod |1+a_kk|^2 = 1+delta
//  tracked as delta' = delta + x + delta*x, one log1p at the end.  Otherwise
//  partial pivoting with prod |u_kk|^2 kept as mantissa * 2^e (frexp), one
//  log at the end.  The complex form (finite T, sum_kmesh_complex,
//  VCA_OMEGA.f90:78-114) runs every spin block of one k in the same warp and
//  also sums the pivots' arguments (plus pi per row swap): arg det of the
//  whole matrix, reduced to (-pi, pi] as the principal log takes it.
// ---------------------------------------------------------------------------
// Lane groups: G lanes (8, 16 or 32) work on one (k, spin block) task and a
// warp runs 32/G tasks side by side.  GB300's FP64 pipe spends an issue slot
// per warp instruction however few of its lanes are active, so packing
// several small LUs into one warp divides the FP64 instructions per task
// (the per-column scalars of four tasks share one instruction, and so do the
// short trailing updates).  All syncs and shuffles inside a task use the
// group's lane mask: groups of one warp may take different branches.
struct KGroup {
  int gl;         // lane within the group
  int base;       // first lane of the group
  unsigned mask;  // the group's lanes
};

// A = (P - H) G for the nb x nb block at offset off, into the group's Aw;
// pre_m: H already holds M = P - H_k (node-independent P)
template <int G>
__device__ __forceinline__ void ksum_block_product(const KGroup& kg, double2* Aw, int nb, int off, int N,
                                                   const double2* Ps, const double2* Gs, const double2* H,
                                                   const int* rowptr, const int* cols, bool pre_m) {
  const int nbb = nb * nb;
  for (int e = kg.gl; e < nbb; e += G) {  // A(i,j), i fastest across lanes
    const int i = e % nb, j = e / nb;
    const int gi = off + i;
    double sr = 0.0, si = 0.0;
    for (int q = rowptr[gi]; q < rowptr[gi + 1]; q++) {
      const int gl = cols[q];
      const int il = gi + gl * N;
      double mr, mi;
      if (pre_m) {
        mr = H[il].x;
        mi = H[il].y;
      } else {
        mr = Ps[il].x - H[il].x;
        mi = Ps[il].y - H[il].y;
      }
      const double2 gg = Gs[gl + (off + j) * N];
      sr = fma(mr, gg.x, sr);
      sr = fma(-mi, gg.y, sr);
      si = fma(mr, gg.y, si);
      si = fma(mi, gg.x, si);
    }
    Aw[e] = make_double2(sr, si);
  }
  __syncwarp(kg.mask);
}

// Aw = G^-1 - 1 + M for the block at offset off (Gs holds G^-1 here):
// ksum_block_logdet adds the 1 back, so it returns ln|det(G^-1 + M)|.
template <int G>
__device__ __forceinline__ void ksum_block_inverse_plus_m(const KGroup& kg, double2* Aw, int nb, int off, int N,
                                                          const double2* Ps, const double2* Gs, const double2* H,
                                                          const int* rowptr, const int* cols, bool pre_m) {
  const int nbb = nb * nb;
  for (int e = kg.gl; e < nbb; e += G) {
    const int i = e % nb, j = e / nb;
    double2 a = Gs[(off + i) + (off + j) * N];
    if (i == j) a.x -= 1.0;
    Aw[e] = a;
  }
  __syncwarp(kg.mask);
  for (int i = kg.gl; i < nb; i += G) {  // one lane per row: M's entries of row off + i
    const int gi = off + i;
    for (int q = rowptr[gi]; q < rowptr[gi + 1]; q++) {
      const int gl = cols[q];
      const int il = gi + gl * N;
      double mr, mi;
      if (pre_m) {
        mr = H[il].x;
        mi = H[il].y;
      } else {
        mr = Ps[il].x - H[il].x;
        mi = Ps[il].y - H[il].y;
      }
      double2& t = Aw[i + (gl - off) * nb];
      t.x += mr;
      t.y += mi;
    }
  }
  __syncwarp(kg.mask);
}

// G^-1 and ln|det G| of every diagonal block of n lso matrices (one warp per
// (node, block), Gauss-Jordan with partial pivoting in shared memory, nb <= 32)
__global__ void k_ginv_blocks(int n, int N, int nblk, int nb, const double2* Glso, double2* Ginv, double* ldG) {
  extern __shared__ double2 gj[];  // per warp: nb x 2nb, column-major with 32-row columns
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  double2* M = gj + (size_t)wib * 64 * 32;
  const int task = blockIdx.x * (blockDim.x >> 5) + wib;
  if (task >= n * nblk) return;
  const int w = task / nblk, b = task % nblk, off = b * nb;
  const double2* Gw = Glso + (int64_t)w * N * N;
  for (int j = 0; j < 2 * nb; j++)
    if (lane < nb)
      M[j * 32 + lane] = (j < nb) ? Gw[(off + lane) + (off + j) * N] : make_double2(lane == j - nb ? 1.0 : 0.0, 0.0);
  __syncwarp();
  double logabs = 0.0;
  for (int k = 0; k < nb; k++) {
    double mag = -1.0;
    int arg = k;
    if (lane >= k && lane < nb) {
      const double2 a = M[k * 32 + lane];
      mag = a.x * a.x + a.y * a.y;
      arg = lane;
    }
    for (int o = 16; o > 0; o >>= 1) {
      const double om = __shfl_xor_sync(0xffffffffu, mag, o);
      const int oa = __shfl_xor_sync(0xffffffffu, arg, o);
      if (om > mag || (om == mag && oa < arg)) { mag = om; arg = oa; }
    }
    if (arg != k)  // swap rows k and arg, lanes over the 2nb columns
      for (int j = lane; j < 2 * nb; j += 32) {
        const double2 t = M[j * 32 + k];
        M[j * 32 + k] = M[j * 32 + arg];
        M[j * 32 + arg] = t;
      }
    __syncwarp();
    const double2 piv = M[k * 32 + k];
    const double pm = piv.x * piv.x + piv.y * piv.y;
    logabs += 0.5 * log(pm);
    const double ir = piv.x / pm, ii = -piv.y / pm;
    for (int j = lane; j < 2 * nb; j += 32) {  // scale row k
      const double2 a = M[j * 32 + k];
      M[j * 32 + k] = make_double2(a.x * ir - a.y * ii, a.x * ii + a.y * ir);
    }
    __syncwarp();
    if (lane < nb && lane != k) {  // eliminate column k from row `lane`
      const double2 f = M[k * 32 + lane];
      for (int j = 0; j < 2 * nb; j++) {
        const double2 u = M[j * 32 + k];
        double2& t = M[j * 32 + lane];
        t.x -= f.x * u.x - f.y * u.y;
        t.y -= f.x * u.y + f.y * u.x;
      }
    }
    __syncwarp();
  }
  double2* Gi = Ginv + (int64_t)w * N * N;
  for (int j = 0; j < nb; j++)
    if (lane < nb) Gi[(off + lane) + (off + j) * N] = M[(nb + j) * 32 + lane];
  if (lane == 0) ldG[(int64_t)w * nblk + b] = logabs;
}
void launch_ginv_blocks(int n, int N, int nblk, int nb, const double2* Glso, double2* Ginv, double* ldG,
                        cudaStream_t st) {
  COUNT_LAUNCH();
  const int warps = 4;
  const size_t shm = sizeof(double2) * warps * 64 * 32;
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_ginv_blocks, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm);
    attr = true;
  }
  const int tasks = n * nblk;
  k_ginv_blocks<<<(tasks + warps - 1) / warps, 32 * warps, shm, st>>>(n, N, nblk, nb, Glso, Ginv, ldG);
}

// ln|det(1 + A)| of the block in Aw (destroyed); with PH, *ph gains the sum
// of the pivots' arguments (plus pi per row swap).  Both are valid on the
// group's first lane only.
template <int G, bool PH>
__device__ double ksum_block_logdet(const KGroup& kg, double2* Aw, int nb, double* ph) {
  const int gl = kg.gl;
  const unsigned gm = kg.mask;
  // row sums of |re| + |im| in FP32 (>= the row sums of |a_ij|); the
  // elimination without pivoting needs them below 1/2, taken as < 0.49 to
  // cover the FP32 rounding
  float rmax = 0.0f;
  for (int i = gl; i < nb; i += G) {
    float r = 0.0f;
    for (int j = 0; j < nb; j++) {
      const double2 a = Aw[i + j * nb];
      r += fabsf((float)a.x) + fabsf((float)a.y);
    }
    rmax = fmaxf(rmax, r);
  }
  for (int o = G / 2; o > 0; o >>= 1) rmax = fmaxf(rmax, __shfl_xor_sync(gm, rmax, o));
  if (rmax < 0.49f) {
    // the per-column scalars (log1p accumulator, argument, 1/pivot) on the
    // first lane, 1/pivot broadcast to the group
    double delta = 0.0;
    for (int kk = 0; kk < nb; kk++) {
      double ir = 0.0, ii = 0.0;
      if (gl == 0) {
        const double2 akk = Aw[kk + kk * nb];
        const double pr = 1.0 + akk.x, pim = akk.y;
        const double x = 2.0 * akk.x + akk.x * akk.x + akk.y * akk.y;
        delta = delta + x + delta * x;
        if (PH) *ph += atan2(pim, pr);
        const double den = pr * pr + pim * pim;
        ir = pr / den;
        ii = -pim / den;  // 1/pivot
      }
      ir = __shfl_sync(gm, ir, kg.base);
      ii = __shfl_sync(gm, ii, kg.base);
      for (int i = kk + 1 + gl; i < nb; i += G) {
        const double2 a = Aw[i + kk * nb];
        Aw[i + kk * nb] = make_double2(a.x * ir - a.y * ii, a.x * ii + a.y * ir);
      }
      __syncwarp(gm);
      const int r = nb - kk - 1;
      for (int e = gl; e < r * r; e += G) {
        const int i = kk + 1 + e % r, j = kk + 1 + e / r;
        const double2 l = Aw[i + kk * nb], u = Aw[kk + j * nb];
        double2& t = Aw[i + j * nb];
        t.x = fma(-l.x, u.x, t.x);
        t.x = fma(l.y, u.y, t.x);
        t.y = fma(-l.x, u.y, t.y);
        t.y = fma(-l.y, u.x, t.y);
      }
      __syncwarp(gm);
    }
    return gl == 0 ? 0.5 * log1p(delta) : 0.0;
  }
  for (int i = gl; i < nb; i += G) Aw[i + i * nb].x += 1.0;
  __syncwarp(gm);
  double mant = 1.0;
  int ex = 0;
  bool zero = false;
  for (int kk = 0; kk < nb; kk++) {
    // pivot: the largest |re| + |im| of the column (FP32 comparison; any
    // row with a nonzero entry is a valid pivot, the largest keeps it stable)
    float fm = -1.0f;
    int arg = kk;
    for (int i = kk + gl; i < nb; i += G) {
      const double2 a = Aw[i + kk * nb];
      const float f = (a.x != 0.0 || a.y != 0.0) ? fmaxf(fabsf((float)a.x) + fabsf((float)a.y), 1e-37f) : 0.0f;
      if (f > fm) { fm = f; arg = i; }
    }
    for (int o = G / 2; o > 0; o >>= 1) {
      const float om = __shfl_xor_sync(gm, fm, o);
      const int oa = __shfl_xor_sync(gm, arg, o);
      if (om > fm || (om == fm && oa < arg)) { fm = om; arg = oa; }
    }
    if (!(fm > 0.0f)) { zero = true; break; }
    double mag;
    {
      const double2 a = Aw[arg + kk * nb];
      mag = a.x * a.x + a.y * a.y;
    }
    if (mag == 0.0) { zero = true; break; }  // |pivot| below 1e-154: treated as singular
    if (arg != kk) {
      for (int j = gl; j < nb; j += G) {
        const double2 t = Aw[kk + j * nb];
        Aw[kk + j * nb] = Aw[arg + j * nb];
        Aw[arg + j * nb] = t;
      }
      if (PH) *ph += 3.141592653589793;
    }
    __syncwarp(gm);
    double ir = 0.0, ii = 0.0;
    if (gl == 0) {  // per-column scalars on the first lane, 1/pivot broadcast
      const double2 piv = Aw[kk + kk * nb];
      if (PH) *ph += atan2(piv.y, piv.x);
      int e2;
      mant = frexp(mant * mag, &e2);
      ex += e2;
      ir = piv.x / mag;
      ii = -piv.y / mag;
    }
    ir = __shfl_sync(gm, ir, kg.base);
    ii = __shfl_sync(gm, ii, kg.base);
    for (int i = kk + 1 + gl; i < nb; i += G) {
      const double2 a = Aw[i + kk * nb];
      Aw[i + kk * nb] = make_double2(a.x * ir - a.y * ii, a.x * ii + a.y * ir);
    }
    __syncwarp(gm);
    const int r = nb - kk - 1;
    for (int e = gl; e < r * r; e += G) {
      const int i = kk + 1 + e % r, j = kk + 1 + e / r;
      const double2 l = Aw[i + kk * nb], u = Aw[kk + j * nb];
      double2& t = Aw[i + j * nb];
      t.x = fma(-l.x, u.x, t.x);
      t.x = fma(l.y, u.y, t.x);
      t.y = fma(-l.x, u.y, t.y);
      t.y = fma(-l.y, u.x, t.y);
    }
    __syncwarp(gm);
  }
  if (gl != 0) return 0.0;
  return zero ? -INFINITY : 0.5 * (log(mant) + ex * 0.6931471805599453);
}

template <bool CPLX, int G>
__global__ void __launch_bounds__(128) k_omega_ksum2(int N, int nblk, int nb, const double2* P,
                                                     const double2* Glso, int64_t Nk, const double2* Hk,
                                                     const double* kw, const int* rowptr, const int* cols,
                                                     double* fpart, double* fpart_im, int kchunks, int pre_m,
                                                     const double2* zn, const double2* Ginv, const double* ldG,
                                                     double omega_c) {
  extern __shared__ double2 shm[];
  constexpr int TPW = 32 / G;
  const int w = blockIdx.y;
  const int chunk = blockIdx.x;
  const int NN = N * N;
  double2* Gs = shm;
  double2* Ps = shm + NN;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nwarps = blockDim.x >> 5;
  const int grp = lane / G;
  KGroup kg;
  kg.gl = lane % G;
  kg.base = grp * G;
  kg.mask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << (grp * G));
  double2* Aw = shm + 2 * NN + ((int64_t)warp * TPW + grp) * nb * nb;
  // inverse form at this node: ln|det(1 + M G)| = ln|det(G^-1 + M)| + ln|det G|
  // (no product per k); kept below omega_c, where the two logs are O(1)
  const bool inv = !CPLX && Ginv != nullptr && zn[w].y <= omega_c;
  const double2* Gsrc = inv ? Ginv : Glso;
  for (int t = threadIdx.x; t < NN; t += blockDim.x) {
    Gs[t] = Gsrc[(int64_t)w * NN + t];
    Ps[t] = P[(int64_t)w * NN + t];
  }
  __syncthreads();
  const int64_t k0 = (Nk * chunk) / kchunks, k1 = (Nk * (chunk + 1)) / kchunks;
  double acc = 0.0, acc_im = 0.0;
  const int64_t ntask = CPLX ? (k1 - k0) : (k1 - k0) * nblk;
  for (int64_t task = (int64_t)warp * TPW + grp; task < ntask; task += (int64_t)nwarps * TPW) {
    const int64_t k = CPLX ? k0 + task : k0 + task / nblk;
    const double2* H = Hk + k * NN;
    const int b0 = CPLX ? 0 : (int)(task % nblk), b1 = CPLX ? nblk : b0 + 1;
    double ld = 0.0, ph = 0.0;
    for (int b = b0; b < b1; b++) {
      if (inv) {
        ksum_block_inverse_plus_m<G>(kg, Aw, nb, b * nb, N, Ps, Gs, H, rowptr, cols, pre_m != 0);
        const double l = ksum_block_logdet<G, CPLX>(kg, Aw, nb, &ph);
        ld += (kg.gl == 0) ? l + ldG[(int64_t)w * nblk + b] : 0.0;
      } else {
        ksum_block_product<G>(kg, Aw, nb, b * nb, N, Ps, Gs, H, rowptr, cols, pre_m != 0);
        ld += ksum_block_logdet<G, CPLX>(kg, Aw, nb, &ph);
      }
    }
    if (kg.gl == 0) {
      acc += kw ? kw[k] * ld : ld;
      if (CPLX) {
        double a = remainder(ph, 6.283185307179586);
        if (a <= -3.141592653589793) a += 6.283185307179586;
        acc_im += kw ? kw[k] * a : a;
      }
    }
    __syncwarp(kg.mask);
  }
  // every lane of the warp is here again: fixed-order warp sums
  for (int o = 16; o > 0; o >>= 1) {
    acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (CPLX) acc_im += __shfl_xor_sync(0xffffffffu, acc_im, o);
  }
  __shared__ double red[32], red_im[32];
  if (lane == 0) { red[warp] = acc; red_im[warp] = acc_im; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double sacc = 0.0, sim = 0.0;
    for (int q = 0; q < nwarps; q++) { sacc += red[q]; sim += red_im[q]; }
    fpart[(int64_t)w * kchunks + chunk] = sacc;
    if (CPLX) fpart_im[(int64_t)w * kchunks + chunk] = sim;
  }
}
__global__ void k_m_from_hk(int64_t n, int NN, const double2* Hl, const double2* Hk, double2* M) {
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
    const double2 h = Hl[q % NN], k = Hk[q];
    M[q] = make_double2(h.x - k.x, h.y - k.y);
  }
}
void launch_m_from_hk(int64_t Nk, int NN, const double2* Hl, const double2* Hk, double2* M, cudaStream_t st) {
  COUNT_LAUNCH();
  const int64_t n = Nk * NN;
  k_m_from_hk<<<nblocks(n, 256), 256, 0, st>>>(n, NN, Hl, Hk, M);
}

template <bool CPLX, int G>
static void ksum2_launch(int nw, int N, int nblk, int nb, const double2* P, const double2* Glso, int64_t Nk,
                         const double2* Hk, const double* kw, const int* rowptr, const int* cols, double* fpart,
                         double* fpart_im, int kchunks, bool pre_m, const KsumInverse& ki, cudaStream_t st) {
  const int threads = 128;
  const size_t shm = sizeof(double2) * (2 * (size_t)N * N + (size_t)(threads / G) * nb * nb);
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_omega_ksum2<CPLX, G>, cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024);
    attr = true;
  }
  k_omega_ksum2<CPLX, G><<<dim3(kchunks, nw, 1), threads, shm, st>>>(N, nblk, nb, P, Glso, Nk, Hk, kw, rowptr, cols,
                                                                     fpart, fpart_im, kchunks, pre_m ? 1 : 0, ki.z,
                                                                     ki.Ginv, ki.ldG, ki.omega_c);
}
template <bool CPLX>
static void ksum2_dispatch(int nw, int N, int nblk, int nb, const double2* P, const double2* Glso, int64_t Nk,
                           const double2* Hk, const double* kw, const int* rowptr, const int* cols, double* fpart,
                           double* fpart_im, int kchunks, bool pre_m, const KsumInverse& ki, cudaStream_t st) {
  // 8 lanes per task up to 12 x 12 blocks, 16 up to 16 x 16, else a warp
  if (nb <= 12)
    ksum2_launch<CPLX, 8>(nw, N, nblk, nb, P, Glso, Nk, Hk, kw, rowptr, cols, fpart, fpart_im, kchunks, pre_m, ki,
                          st);
  else if (nb <= 16)
    ksum2_launch<CPLX, 16>(nw, N, nblk, nb, P, Glso, Nk, Hk, kw, rowptr, cols, fpart, fpart_im, kchunks, pre_m, ki,
                           st);
  else
    ksum2_launch<CPLX, 32>(nw, N, nblk, nb, P, Glso, Nk, Hk, kw, rowptr, cols, fpart, fpart_im, kchunks, pre_m, ki,
                           st);
}
void launch_omega_ksum2(int nw, int N, int nblk, int nb, const double2* P, const double2* Glso, int64_t Nk,
                        const double2* Hk, const double* kw, const int* rowptr, const int* cols, double* fpart,
                        double* fpart_im, int kchunks, bool pre_m, const KsumInverse& ki, cudaStream_t st) {
  COUNT_LAUNCH();
  if (fpart_im)
    ksum2_dispatch<true>(nw, N, nblk, nb, P, Glso, Nk, Hk, kw, rowptr, cols, fpart, fpart_im, kchunks, pre_m, ki,
                         st);
  else
    ksum2_dispatch<false>(nw, N, nblk, nb, P, Glso, Nk, Hk, kw, rowptr, cols, fpart, nullptr, kchunks, pre_m, ki,
                          st);
}

// ---------------------------------------------------------------------------
// Self-energy and Weiss field on a frequency grid (build_sigma_normal,
// VCA_GF_NORMAL.f90:1045-1111): G0^-1(z) = (z + xmu) 1 - Hloc - Delta(z),
// Sigma = G0^-1 - G'^-1, G0 = (G0^-1)^-1, per z on N x N lso matrices
// (N <= 32).  One warp per z: Gauss-Jordan with partial pivoting on the
// augmented [A | 1] in shared memory, stored column-major with 32-row
// columns so that lane r (row r) works conflict-free.
// ---------------------------------------------------------------------------
__device__ void warp_gj_inverse(double2* M, int N) {
  const int lane = threadIdx.x & 31;
  const int N2 = 2 * N;
  for (int k = 0; k < N; k++) {
    double mag = -1.0;
    int arg = k;
    if (lane >= k && lane < N) {
      const double2 a = M[k * 32 + lane];
      mag = a.x * a.x + a.y * a.y;
      arg = lane;
    }
    for (int o = 16; o > 0; o >>= 1) {
      const double om = __shfl_xor_sync(0xffffffffu, mag, o);
      const int oa = __shfl_xor_sync(0xffffffffu, arg, o);
      if (om > mag || (om == mag && oa < arg)) { mag = om; arg = oa; }
    }
    if (!(mag > 0.0)) continue;  // singular column: left as is (the result is undefined, as in the reference)
    if (arg != k)
      for (int j = lane; j < N2; j += 32) {
        const double2 t = M[j * 32 + k];
        M[j * 32 + k] = M[j * 32 + arg];
        M[j * 32 + arg] = t;
      }
    __syncwarp();
    const double2 piv = M[k * 32 + k];
    const double ir = piv.x / mag, ii = -piv.y / mag;  // 1/piv
    __syncwarp();
    for (int j = lane; j < N2; j += 32) {
      const double2 a = M[j * 32 + k];
      M[j * 32 + k] = make_double2(a.x * ir - a.y * ii, a.x * ii + a.y * ir);
    }
    __syncwarp();
    if (lane < N && lane != k) {
      const double2 f = M[k * 32 + lane];
      for (int j = 0; j < N2; j++) {
        const double2 u = M[j * 32 + k];
        double2& t = M[j * 32 + lane];
        t.x -= f.x * u.x - f.y * u.y;
        t.y -= f.x * u.y + f.y * u.x;
      }
    }
    __syncwarp();
  }
}

// out[q] = A[q]^-1 for nz N x N matrices (lso, column-major), one warp each
__global__ void k_inverse_batch(int nz, int N, const double2* A, double2* out) {
  extern __shared__ double2 gjm[];
  const int q = blockIdx.x;
  if (q >= nz) return;
  const int lane = threadIdx.x & 31;
  const int NN = N * N;
  for (int c = 0; c < N; c++)
    if (lane < N) {
      gjm[c * 32 + lane] = A[(int64_t)q * NN + lane + c * N];
      gjm[(N + c) * 32 + lane] = make_double2(lane == c ? 1.0 : 0.0, 0.0);
    }
  __syncwarp();
  warp_gj_inverse(gjm, N);
  for (int c = 0; c < N; c++)
    if (lane < N) out[(int64_t)q * NN + lane + c * N] = gjm[(N + c) * 32 + lane];
}
void launch_inverse_batch(int nz, int N, const double2* A, double2* out, cudaStream_t st) {
  if (nz <= 0) return;
  COUNT_LAUNCH();
  const size_t shm = sizeof(double2) * 2 * (size_t)N * 32;
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_inverse_batch, cudaFuncAttributeMaxDynamicSharedMemorySize, 64 * 1024);
    attr = true;
  }
  k_inverse_batch<<<nz, 32, shm, st>>>(nz, N, A, out);
}

// Custom-observable integrand (sum_observable_kmesh / _complex,
// VCA_OBSERVABLES.f90:408-500): fpart[w][chunk] = sum over the chunk's k of
// Re{ Tr[s_k G_k(z_w)] - tail * Tr[s_k] / (z_w - 1.1) } with the lattice
// G_k = (G'^-1 - (H_k - P))^-1, P = Hloc + Delta.  G_k is inverted per spin
// block (nblk blocks of nb) by one warp (Gauss-Jordan); s_k is read only on
// the blocks (the trace with a block-diagonal G_k needs no more).  s holds
// one matrix per k (sk_stride = N*N) or one for all (sk_stride = 0).
__global__ void __launch_bounds__(128) k_obs_ksum(int N, int nblk, int nb, const double2* z, const double2* Ginv,
                                                  const double2* P, int64_t Nk, const double2* Hk, const double2* s,
                                                  int64_t sk_stride, int tail, double* fpart, int kchunks) {
  extern __shared__ double2 shm[];
  const int w = blockIdx.y;
  const int chunk = blockIdx.x;
  const int NN = N * N;
  double2* Gs = shm;
  double2* Ps = shm + NN;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nwarps = blockDim.x >> 5;
  double2* M = shm + 2 * NN + (int64_t)warp * 2 * nb * 32;
  for (int t = threadIdx.x; t < NN; t += blockDim.x) {
    Gs[t] = Ginv[(int64_t)w * NN + t];
    Ps[t] = P[(int64_t)w * NN + t];
  }
  __syncthreads();
  const double2 zw = z[w];
  // 1/(z - 1.1)
  const double dr = zw.x - 1.1, di = zw.y, dd = dr * dr + di * di;
  const double2 rz = make_double2(dr / dd, -di / dd);
  const int64_t k0 = (Nk * chunk) / kchunks, k1 = (Nk * (chunk + 1)) / kchunks;
  double acc = 0.0;
  for (int64_t k = k0 + warp; k < k1; k += nwarps) {
    const double2* H = Hk + k * NN;
    const double2* S = s + k * sk_stride;
    double tr = 0.0;
    for (int b = 0; b < nblk; b++) {
      const int off = b * nb;
      for (int c = 0; c < nb; c++)
        if (lane < nb) {
          const int il = (off + lane) + (off + c) * N;
          const double2 g = Gs[il], h = H[il], p = Ps[il];
          M[c * 32 + lane] = make_double2(g.x - (h.x - p.x), g.y - (h.y - p.y));
          M[(nb + c) * 32 + lane] = make_double2(lane == c ? 1.0 : 0.0, 0.0);
        }
      __syncwarp();
      warp_gj_inverse(M, nb);
      // Tr[s G] over the block: sum_{i,j} s(i,j) G(j,i), lane = i
      if (lane < nb)
        for (int j = 0; j < nb; j++) {
          const double2 sv = S[(off + lane) + (off + j) * N];
          const double2 gv = M[(nb + lane) * 32 + j];  // G(j, lane)
          tr += sv.x * gv.x - sv.y * gv.y;
        }
      __syncwarp();
    }
    if (tail && lane < N) {  // - Re[ s(lane,lane) / (z - 1.1) ]
      const double2 sv = S[lane + lane * N];
      tr -= sv.x * rz.x - sv.y * rz.y;
    }
    for (int o = 16; o > 0; o >>= 1) tr += __shfl_xor_sync(0xffffffffu, tr, o);
    if (lane == 0) acc += tr;
  }
  __shared__ double red[32];
  if (lane == 0) red[warp] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double sacc = 0.0;
    for (int q = 0; q < nwarps; q++) sacc += red[q];
    fpart[(int64_t)w * kchunks + chunk] = sacc;
  }
}
void launch_obs_ksum(int nw, int N, int nblk, int nb, const double2* z, const double2* Ginv, const double2* P,
                     int64_t Nk, const double2* Hk, const double2* s, int64_t sk_stride, bool tail, double* fpart,
                     int kchunks, cudaStream_t st) {
  COUNT_LAUNCH();
  const int threads = 128;
  const size_t shm = sizeof(double2) * (2 * (size_t)N * N + (size_t)(threads / 32) * 2 * nb * 32);
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_obs_ksum, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    attr = true;
  }
  k_obs_ksum<<<dim3(kchunks, nw, 1), threads, shm, st>>>(N, nblk, nb, z, Ginv, P, Nk, Hk, s, sk_stride, tail ? 1 : 0,
                                                         fpart, kchunks);
}

// want_g0 = 0: out = Sigma(z); 1: out = G0(z).  P = Delta + Hloc (lso, per z
// when per_z_p, else one matrix).
__global__ void k_sigma_g0(int nz, int N, const double2* z, const double2* Glso, const double2* P, int per_z_p,
                           double xmu, int want_g0, double2* out) {
  extern __shared__ double2 gjm[];
  const int q = blockIdx.x;
  if (q >= nz) return;
  const int lane = threadIdx.x & 31;
  const int NN = N * N;
  const double2 zz = make_double2(z[q].x + xmu, z[q].y);
  const double2* Pq = P + (per_z_p ? (int64_t)q * NN : 0);
  // A = G (Sigma) or G0^-1 (G0), augmented with the identity
  for (int c = 0; c < N; c++) {
    if (lane < N) {
      double2 a;
      if (want_g0) {
        const double2 p = Pq[lane + c * N];
        a = make_double2((lane == c ? zz.x : 0.0) - p.x, (lane == c ? zz.y : 0.0) - p.y);
      } else {
        a = Glso[(int64_t)q * NN + lane + c * N];
      }
      gjm[c * 32 + lane] = a;
      gjm[(N + c) * 32 + lane] = make_double2(lane == c ? 1.0 : 0.0, 0.0);
    }
  }
  __syncwarp();
  warp_gj_inverse(gjm, N);
  for (int c = 0; c < N; c++) {
    if (lane < N) {
      const double2 inv = gjm[(N + c) * 32 + lane];
      double2 r;
      if (want_g0) {
        r = inv;
      } else {  // Sigma = (z + xmu) 1 - P - G^-1
        const double2 p = Pq[lane + c * N];
        r = make_double2((lane == c ? zz.x : 0.0) - p.x - inv.x, (lane == c ? zz.y : 0.0) - p.y - inv.y);
      }
      out[(int64_t)q * NN + lane + c * N] = r;
    }
  }
}
void launch_sigma_g0(int nz, int N, const double2* z, const double2* Glso, const double2* P, bool per_z_p,
                     double xmu, bool want_g0, double2* out, cudaStream_t st) {
  if (nz <= 0) return;
  COUNT_LAUNCH();
  const size_t shm = sizeof(double2) * 2 * (size_t)N * 32;
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_sigma_g0, cudaFuncAttributeMaxDynamicSharedMemorySize, 64 * 1024);
    attr = true;
  }
  k_sigma_g0<<<nz, 32, shm, st>>>(nz, N, z, Glso, P, per_z_p ? 1 : 0, xmu, want_g0 ? 1 : 0, out);
}

// ---------------------------------------------------------------------------
// Ground-state observables (vca_lanc_observables, VCA_OBSERVABLES.f90:
// 185-316): for one state psi of a sector, sums over its elements of
// |psi_i|^2 n_up(l), |psi_i|^2 n_dw(l) and |psi_i|^2 n_up(l) n_dw(l) for each
// cluster spin-orbital bit l (imp_state_index = iorb + (ilat-1)*Norb).
// grid.y = l, grid.z = quantity; each block writes one partial, reduced by
// the host in a fixed order.  fmt: 0 int64 fixed point (scale 2^-F),
// 1 double, 2 double2.
// ---------------------------------------------------------------------------
__global__ void k_observables(SectorView sv, int fmt, const void* vec, int F, double* part) {
  const int l = blockIdx.y, qn = blockIdx.z;
  const int64_t D = (int64_t)sv.dimup * sv.dimdw;
  const double sc = ldexp(1.0, -F);
  double acc = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < D; i += (int64_t)gridDim.x * blockDim.x) {
    const int idw = (int)(i / sv.dimup);
    const int iup = (int)(i - (int64_t)idw * sv.dimup);
    const int nu = (sv.up_words[iup] >> l) & 1, nd = (sv.dw_words[idw] >> l) & 1;
    const int on = qn == 0 ? nu : (qn == 1 ? nd : nu & nd);
    if (!on) continue;
    double w;
    if (fmt == 0) {
      const double x = (double)((const long long*)vec)[i] * sc;
      w = x * x;
    } else if (fmt == 1) {
      const double x = ((const double*)vec)[i];
      w = x * x;
    } else {
      const double2 x = ((const double2*)vec)[i];
      w = x.x * x.x + x.y * x.y;
    }
    acc += w;
  }
  __shared__ double red[256];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[((int64_t)qn * gridDim.y + l) * gridDim.x + blockIdx.x] = red[0];
}
int observables_blocks(int64_t D) { return (int)std::max<int64_t>(1, std::min<int64_t>((D + 255) / 256, 304)); }
void launch_observables(const SectorView& sv, int fmt, const void* vec, int F, int nimp, double* part,
                        cudaStream_t st) {
  COUNT_LAUNCH();
  const dim3 grd(observables_blocks((int64_t)sv.dimup * sv.dimdw), nimp, 3);
  k_observables<<<grd, 256, 0, st>>>(sv, fmt, vec, F, part);
}

// dst[r] = src[idx[r]] for blocks of nel double2
__global__ void k_gather_blocks(int64_t nrep, int64_t nel, const int64_t* idx, const double2* src, double2* dst) {
  const int64_t n = nrep * nel;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = t / nel, x = t - r * nel;
    dst[t] = src[idx[r] * nel + x];
  }
}
void launch_gather_blocks(int64_t nrep, int64_t nel, const int64_t* idx, const double2* src, double2* dst,
                          cudaStream_t st) {
  if (nrep <= 0) return;
  COUNT_LAUNCH();
  k_gather_blocks<<<nblocks(nrep * nel, 256), 256, 0, st>>>(nrep, nel, idx, src, dst);
}

// ---------------------------------------------------------------------------
// Lanczos with full reorthogonalisation ("arpack" diagonalisation): the
// stored basis V (nq vectors of n elements, vector q at V + q*n), real
// (double) or complex (double2) elements.  Every reduction is fixed-order:
// block partials in a fixed tree, then one warp per output over the blocks.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double ap_cdot(double v, double w) { return v * w; }
__device__ __forceinline__ double2 ap_cdot(double2 v, double2 w) {  // conj(v) * w
  return make_double2(v.x * w.x + v.y * w.y, v.x * w.y - v.y * w.x);
}
__device__ __forceinline__ double ap_add(double a, double b) { return a + b; }
__device__ __forceinline__ double2 ap_add(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double ap_zero(double) { return 0.0; }
__device__ __forceinline__ double2 ap_zero(double2) { return make_double2(0.0, 0.0); }
__device__ __forceinline__ double ap_fms(double w, double c, double v) { return fma(-c, v, w); }
__device__ __forceinline__ double2 ap_fms(double2 w, double2 c, double2 v) {  // w - c v
  return make_double2(w.x - (c.x * v.x - c.y * v.y), w.y - (c.x * v.y + c.y * v.x));
}
__device__ __forceinline__ double ap_shfl(double v, int off) { return __shfl_xor_sync(0xffffffffu, v, off); }
__device__ __forceinline__ double2 ap_shfl(double2 v, int off) {
  return make_double2(__shfl_xor_sync(0xffffffffu, v.x, off), __shfl_xor_sync(0xffffffffu, v.y, off));
}

__device__ __forceinline__ double ap_scalar(double, double v) { return v; }
__device__ __forceinline__ double2 ap_scalar(double2, double v) { return make_double2(v, 0.0); }
// a = 0 ignores y (a fresh buffer may hold NaN bit patterns)
__device__ __forceinline__ double ap_lin(double a, double y, double s, double x) {
  return fma(-s, x, a == 0.0 ? 0.0 : a * y);
}
__device__ __forceinline__ double2 ap_lin(double a, double2 y, double s, double2 x) {
  return make_double2(fma(-s, x.x, a == 0.0 ? 0.0 : a * y.x), fma(-s, x.y, a == 0.0 ? 0.0 : a * y.y));
}

// partial[q*nblk + b] = sum over block b's rows of conj(V_q[i]) w[i]
template <typename T>
__global__ void __launch_bounds__(256) k_ap_proj(int64_t n, const T* __restrict__ V, const T* __restrict__ w,
                                                 T* partial) {
  __shared__ T red[256];
  const int q = blockIdx.y, nblk = gridDim.x;
  const int64_t chunk = (n + nblk - 1) / nblk;
  const int64_t i0 = (int64_t)blockIdx.x * chunk, i1 = min(n, i0 + chunk);
  const T* vq = V + (int64_t)q * n;
  T s = ap_zero(T());
  for (int64_t i = i0 + threadIdx.x; i < i1; i += blockDim.x) s = ap_add(s, ap_cdot(vq[i], w[i]));
  red[threadIdx.x] = s;
  __syncthreads();
  for (int h = 128; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h) red[threadIdx.x] = ap_add(red[threadIdx.x], red[threadIdx.x + h]);
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[(int64_t)q * nblk + blockIdx.x] = red[0];
}

// c[q] = sum_b partial[q*nblk + b], one warp per q
template <typename T>
__global__ void k_ap_sum(int nq, int nblk, const T* partial, T* c) {
  const int lane = threadIdx.x & 31;
  const int q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (q >= nq) return;
  T s = ap_zero(T());
  for (int b = lane; b < nblk; b += 32) s = ap_add(s, partial[(int64_t)q * nblk + b]);
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) s = ap_add(s, ap_shfl(s, off));
  if (lane == 0) c[q] = s;
}

// w[i] -= sum_q c[q] V_q[i]  (q ascending)
template <typename T>
__global__ void __launch_bounds__(256) k_ap_orth(int64_t n, int nq, const T* __restrict__ V, const T* __restrict__ c,
                                                 T* __restrict__ w) {
  extern __shared__ __align__(16) unsigned char ap_smem[];
  T* cs = (T*)ap_smem;
  for (int q = threadIdx.x; q < nq; q += blockDim.x) cs[q] = c[q];
  __syncthreads();
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    T x = w[i];
    for (int q = 0; q < nq; q++) x = ap_fms(x, cs[q], V[(int64_t)q * n + i]);
    w[i] = x;
  }
}

// x[i] = sum_q z[q] V_q[i] (real coefficients, q ascending)
template <typename T>
__global__ void __launch_bounds__(256) k_ap_combine(int64_t n, int nq, const T* __restrict__ V,
                                                    const double* __restrict__ z, T* __restrict__ x) {
  extern __shared__ __align__(16) unsigned char ap_smem[];
  double* zs = (double*)ap_smem;
  for (int q = threadIdx.x; q < nq; q += blockDim.x) zs[q] = z[q];
  __syncthreads();
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    T acc = ap_zero(T());
    for (int q = 0; q < nq; q++) acc = ap_fms(acc, ap_scalar(T(), -zs[q]), V[(int64_t)q * n + i]);
    x[i] = acc;
  }
}

// y = a*y - s*x (real scalars: y -= s x with a = 1, y = x/b with a = 0)
template <typename T>
__global__ void k_ap_axpby(int64_t n, double a, double s, const T* __restrict__ x, T* __restrict__ y) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = ap_lin(a, y[i], s, x[i]);
}

#define AP_NBLK 304
void launch_ap_proj(int64_t n, int nq, bool cplx, const void* V, const void* w, void* partial, void* c,
                    cudaStream_t st) {
  COUNT_LAUNCH();
  COUNT_LAUNCH();
  const dim3 grd(AP_NBLK, nq, 1);
  if (cplx) {
    k_ap_proj<double2><<<grd, 256, 0, st>>>(n, (const double2*)V, (const double2*)w, (double2*)partial);
    k_ap_sum<double2><<<(nq * 32 + 127) / 128, 128, 0, st>>>(nq, AP_NBLK, (const double2*)partial, (double2*)c);
  } else {
    k_ap_proj<double><<<grd, 256, 0, st>>>(n, (const double*)V, (const double*)w, (double*)partial);
    k_ap_sum<double><<<(nq * 32 + 127) / 128, 128, 0, st>>>(nq, AP_NBLK, (const double*)partial, (double*)c);
  }
}
int ap_partial_len(int nq) { return AP_NBLK * nq; }
void launch_ap_orth(int64_t n, int nq, bool cplx, const void* V, const void* c, void* w, cudaStream_t st) {
  COUNT_LAUNCH();
  if (cplx)
    k_ap_orth<double2><<<nblocks(n, 256), 256, sizeof(double2) * nq, st>>>(n, nq, (const double2*)V,
                                                                         (const double2*)c, (double2*)w);
  else
    k_ap_orth<double><<<nblocks(n, 256), 256, sizeof(double) * nq, st>>>(n, nq, (const double*)V, (const double*)c,
                                                                       (double*)w);
}
void launch_ap_combine(int64_t n, int nq, bool cplx, const void* V, const double* z, void* x, cudaStream_t st) {
  COUNT_LAUNCH();
  if (cplx)
    k_ap_combine<double2><<<nblocks(n, 256), 256, sizeof(double) * nq, st>>>(n, nq, (const double2*)V, z,
                                                                           (double2*)x);
  else
    k_ap_combine<double><<<nblocks(n, 256), 256, sizeof(double) * nq, st>>>(n, nq, (const double*)V, z,
                                                                          (double*)x);
}
void launch_ap_axpby(int64_t n, bool cplx, double a, double s, const void* x, void* y, cudaStream_t st) {
  COUNT_LAUNCH();
  if (cplx)
    k_ap_axpby<double2><<<nblocks(n, 256), 256, 0, st>>>(n, a, s, (const double2*)x, (double2*)y);
  else
    k_ap_axpby<double><<<nblocks(n, 256), 256, 0, st>>>(n, a, s, (const double*)x, (double*)y);
}

}  // namespace vca
