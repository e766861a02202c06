// vca_mlp.cu -- the Omega surrogate: a 4 -> 128 -> 128 -> 128 -> 1 SiLU
// network trained on the GPU on Omega values and gradients the solver
// produces (a Sobolev loss), with its own forward, tangent and backward
// kernels.  No counterpart in the reference: it replaces nothing there, it
// proposes candidates for the stationary-point search that the reference's
// drivers run with brent / fmin_bfgs (drivers/vca_hm_chain1d.f90:104-108,
// drivers/vca_bhz_2d.f90:244-305), and every accepted candidate is re-solved
// by the plain path.
//
// Arithmetic: FP32 master weights; the two 128 x 128 layers run on the
// tcgen05 tensor cores with BF16 operands and FP32 accumulation
// (vca_umma.cu); everything else (the 4 -> 128 input layer, the 128 -> 1
// head, SiLU and its derivatives, the loss, the reductions, Adam) in FP32 on
// the CUDA cores, with every reduction in a fixed order.
//
// Input gradients are carried forward-mode: every sample owns 1 + n_in rows
// (its value and one tangent per input), laid out channel-major, row
// ch * Spad + j for sample j, Spad = samples rounded up to 128.  Tangent
// rows carry dz/dx_d: the input layer gives W1[:, d], a SiLU multiplies by
// s'(z) of the sample's value row, a linear layer applies W (no bias).  The
// loss of sample j is
//   (f_j - y_j)^2 + lambda * sum_d (df_j/dx_d - dy_jd)^2,   averaged over j,
// and its parameter gradient is the reverse pass over that extended graph
// (for the tangent path s''(z) enters: d(s'(z) zdot)/dz = s''(z) zdot).
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/vca_gpu.h"
#include "vca_umma.cuh"

namespace vca {
void count_launch_external();
void set_api_error(const std::string& m);
}  // namespace vca

using namespace vca;

namespace {

#define MW 128  // hidden width
#define MAXIN 4

#define MFAIL(code, msg)   \
  do {                     \
    set_api_error(msg);    \
    return (code);         \
  } while (0)
#define MCU(x)                                                                                    \
  do {                                                                                            \
    cudaError_t e_ = (x);                                                                         \
    if (e_ != cudaSuccess) {                                                                      \
      set_api_error(std::string("CUDA error ") + cudaGetErrorString(e_) + " at " + #x);           \
      return e_ == cudaErrorMemoryAllocation ? VCA_ERR_ALLOC : VCA_ERR_CUDA;                      \
    }                                                                                             \
  } while (0)

typedef __nv_bfloat16 bf16;

struct Offs {  // flat FP32 parameter vector
  int W1, b1, W2, b2, W3, b3, w4, b4, n;
};
Offs offsets(int nin) {
  Offs o;
  o.W1 = 0;
  o.b1 = o.W1 + MW * nin;
  o.W2 = o.b1 + MW;
  o.b2 = o.W2 + MW * MW;
  o.W3 = o.b2 + MW;
  o.b3 = o.W3 + MW * MW;
  o.w4 = o.b3 + MW;
  o.b4 = o.w4 + MW;
  o.n = o.b4 + 1;
  return o;
}

struct Mlp {
  vca_mlp_config cfg{};
  int nin = 0, cap = 0, capPad = 0;
  Offs of{};
  cudaStream_t st = nullptr;
  std::vector<void*> mem;
  float *P = nullptr, *G = nullptr, *Mo = nullptr, *Ve = nullptr;
  bf16 *W2t = nullptr, *W2Tt = nullptr, *W3t = nullptr, *W3Tt = nullptr;
  float *X = nullptr, *Y = nullptr, *DY = nullptr;  // training set
  float* GW = nullptr;                              // per-sample weight of the gradient term
  float *Xq = nullptr;                              // prediction points
  bf16 *A1 = nullptr, *A1T = nullptr, *A2 = nullptr, *A2T = nullptr, *GZ = nullptr, *GZT = nullptr;
  float *Z2 = nullptr, *Z3 = nullptr, *GA = nullptr;
  float *E = nullptr, *F = nullptr, *Lj = nullptr;
  float *GZ1 = nullptr, *GDZ1 = nullptr, *T4 = nullptr, *GZB2 = nullptr, *GZB3 = nullptr;
  float* loss = nullptr;
  int* status = nullptr;
  int* step = nullptr;
  int S = 0;  // samples in the training set
  cudaGraphExec_t gexec = nullptr;
  int gS = -1;  // sample count the captured graph was built for
};
Mlp* m = nullptr;

template <class T>
int malloc_n(T** p, size_t n) {
  cudaError_t e = cudaMalloc((void**)p, std::max<size_t>(n, 1) * sizeof(T));
  if (e != cudaSuccess) {
    *p = nullptr;
    cudaGetLastError();
    MFAIL(VCA_ERR_ALLOC, std::string("cudaMalloc failed in the surrogate: ") + cudaGetErrorString(e));
  }
  m->mem.push_back(*p);
  return VCA_OK;
}

__device__ __forceinline__ void silu3(float z, float& s, float& s1, float& s2) {
  const float sg = 1.0f / (1.0f + expf(-z));
  s = z * sg;
  s1 = sg * (1.0f + z * (1.0f - sg));
  s2 = sg * (1.0f - sg) * (2.0f + z * (1.0f - 2.0f * sg));
}

// one activation value into both tiled layouts: row-major operand (K = 128
// features) and its transpose (K = R rows) for the weight-gradient GEMMs
__device__ __forceinline__ void put2(bf16* A, bf16* AT, int R, int r, int o, float v) {
  const bf16 b = __float2bfloat16_rn(v);
  A[umma_off(r, o, MW)] = b;
  AT[umma_off(o, r, R)] = b;
}

// input layer: value rows s(W1 x + b1), tangent rows s'(z) W1[:, d]
__global__ void k_mlp_l1(const float* P, Offs of, const float* X, int S, int Spad, int nin, int nch, bf16* A1,
                         bf16* A1T) {
  const int R = nch * Spad;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= Spad * MW) return;
  const int j = t / MW, o = t % MW;
  if (j >= S) {
    for (int c = 0; c < nch; c++) put2(A1, A1T, R, c * Spad + j, o, 0.0f);
    return;
  }
  float z = P[of.b1 + o];
  for (int i = 0; i < nin; i++) z = fmaf(P[of.W1 + o * nin + i], X[j * nin + i], z);
  float s, s1, s2;
  silu3(z, s, s1, s2);
  put2(A1, A1T, R, j, o, s);
  for (int d = 0; d + 1 < nch; d++) put2(A1, A1T, R, (d + 1) * Spad + j, o, s1 * P[of.W1 + o * nin + d]);
}

// hidden SiLU after a GEMM: value rows s(z + b), tangent rows s'(z) zdot
__global__ void k_mlp_act(const float* Z, const float* b, int S, int Spad, int nch, bf16* A, bf16* AT) {
  const int R = nch * Spad;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= Spad * MW) return;
  const int j = t / MW, o = t % MW;
  if (j >= S) {
    for (int c = 0; c < nch; c++) put2(A, AT, R, c * Spad + j, o, 0.0f);
    return;
  }
  float s, s1, s2;
  silu3(Z[(size_t)j * MW + o] + b[o], s, s1, s2);
  put2(A, AT, R, j, o, s);
  for (int c = 1; c < nch; c++) put2(A, AT, R, c * Spad + j, o, s1 * Z[((size_t)c * Spad + j) * MW + o]);
}

// head: F[c][j] = w4 . act3(row c*Spad + j) (+ b4 on the value row); one warp
// per (channel, sample), lanes over features in a fixed order
__global__ void k_mlp_head(const float* P, Offs of, const float* Z3, int S, int Spad, int nch, float* F) {
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (w >= nch * S) return;
  const int c = w / S, j = w % S;
  float acc = 0.0f;
  for (int o = lane; o < MW; o += 32) {
    float s, s1, s2;
    silu3(Z3[(size_t)j * MW + o] + P[of.b3 + o], s, s1, s2);
    const float v = (c == 0) ? s : s1 * Z3[((size_t)c * Spad + j) * MW + o];
    acc = fmaf(P[of.w4 + o], v, acc);
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
  if (lane == 0) F[c * Spad + j] = acc + (c == 0 ? P[of.b4] : 0.0f);
}

// per-sample loss and the seeds dL/df, dL/d(df/dx_d)
__global__ void k_mlp_loss(const float* F, const float* Y, const float* DY, const float* GW, int S, int Spad,
                           int nin, int nch, float lam0, float* E, float* Lj) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= Spad) return;
  if (j >= S) {
    for (int c = 0; c < nch; c++) E[c * Spad + j] = 0.0f;
    return;
  }
  const float inv = 1.0f / (float)S;
  const float lam = lam0 * GW[j];
  const float r0 = F[j] - Y[j];
  float L = r0 * r0;
  E[j] = 2.0f * r0 * inv;
  for (int d = 0; d + 1 < nch; d++) {
    const float rd = F[(d + 1) * Spad + j] - DY[j * nin + d];
    L += lam * rd * rd;
    E[(d + 1) * Spad + j] = 2.0f * lam * rd * inv;
  }
  Lj[j] = L * inv;
}

// reverse through the head and the third SiLU: GZ rows of layer 3, and the
// per-sample contributions to dL/dw4 and dL/db3
__global__ void k_mlp_head_bwd(const float* P, Offs of, const float* Z3, const float* E, int S, int Spad, int nch,
                               bf16* GZ, bf16* GZT, float* T4, float* GZB) {
  const int R = nch * Spad;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= Spad * MW) return;
  const int j = t / MW, o = t % MW;
  if (j >= S) {
    for (int c = 0; c < nch; c++) put2(GZ, GZT, R, c * Spad + j, o, 0.0f);
    T4[t] = 0.0f;
    GZB[t] = 0.0f;
    return;
  }
  float s, s1, s2;
  silu3(Z3[(size_t)j * MW + o] + P[of.b3 + o], s, s1, s2);
  const float w = P[of.w4 + o], e0 = E[j];
  float gz = e0 * w * s1, g4 = e0 * s;
  for (int c = 1; c < nch; c++) {
    const float zd = Z3[((size_t)c * Spad + j) * MW + o], ed = E[c * Spad + j];
    gz = fmaf(ed * w * zd, s2, gz);
    g4 = fmaf(ed * s1, zd, g4);
    put2(GZ, GZT, R, c * Spad + j, o, ed * w * s1);
  }
  put2(GZ, GZT, R, j, o, gz);
  T4[t] = g4;
  GZB[t] = gz;
}

// reverse through a hidden SiLU: from GA (dL/d act, value and tangent rows)
// to the GZ rows of the layer below
__global__ void k_mlp_act_bwd(const float* Z, const float* b, const float* GA, int S, int Spad, int nch, bf16* GZ,
                              bf16* GZT, float* GZB) {
  const int R = nch * Spad;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= Spad * MW) return;
  const int j = t / MW, o = t % MW;
  if (j >= S) {
    for (int c = 0; c < nch; c++) put2(GZ, GZT, R, c * Spad + j, o, 0.0f);
    GZB[t] = 0.0f;
    return;
  }
  float s, s1, s2;
  silu3(Z[(size_t)j * MW + o] + b[o], s, s1, s2);
  float gz = GA[(size_t)j * MW + o] * s1;
  for (int c = 1; c < nch; c++) {
    const size_t rc = ((size_t)c * Spad + j) * MW + o;
    const float gad = GA[rc];
    gz = fmaf(gad * Z[rc], s2, gz);
    put2(GZ, GZT, R, c * Spad + j, o, gad * s1);
  }
  put2(GZ, GZT, R, j, o, gz);
  GZB[t] = gz;
}

// reverse through the input layer's SiLU: dL/dz1 and dL/d zdot1_d per sample
__global__ void k_mlp_l1_bwd(const float* P, Offs of, const float* X, const float* GA, int S, int Spad, int nin,
                             int nch, float* GZ1, float* GDZ1) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= Spad * MW) return;
  const int j = t / MW, o = t % MW;
  if (j >= S) return;
  float z = P[of.b1 + o];
  for (int i = 0; i < nin; i++) z = fmaf(P[of.W1 + o * nin + i], X[j * nin + i], z);
  float s, s1, s2;
  silu3(z, s, s1, s2);
  float gz = GA[(size_t)j * MW + o] * s1;
  for (int c = 1; c < nch; c++) {
    const float gad = GA[((size_t)c * Spad + j) * MW + o];
    gz = fmaf(gad * P[of.W1 + o * nin + (c - 1)], s2, gz);
    GDZ1[((size_t)(c - 1) * Spad + j) * MW + o] = gad * s1;
  }
  GZ1[t] = gz;
}

// gradients of W1, b1, b2, b3, w4, b4 and the loss: fixed-order sums over the
// samples, one thread per output; W2 and W3 come from the GEMMs
__global__ void k_mlp_reduce(Offs of, const float* X, const float* E, const float* Lj, const float* GZ1,
                             const float* GDZ1, const float* T4, const float* GZB2, const float* GZB3, int S,
                             int Spad, int nin, int nch, float* G, float* loss) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int nW1 = MW * nin;
  if (t < nW1) {
    const int o = t / nin, i = t % nin;
    float acc = 0.0f;
    for (int j = 0; j < S; j++) acc = fmaf(GZ1[(size_t)j * MW + o], X[j * nin + i], acc);
    if (i + 1 < nch)
      for (int j = 0; j < S; j++) acc += GDZ1[((size_t)i * Spad + j) * MW + o];
    G[of.W1 + t] = acc;
    return;
  }
  int u = t - nW1;
  if (u < 4 * MW) {
    const int which = u / MW, o = u % MW;
    const float* src = which == 0 ? GZ1 : which == 1 ? GZB2 : which == 2 ? GZB3 : T4;
    float acc = 0.0f;
    for (int j = 0; j < S; j++) acc += src[(size_t)j * MW + o];
    const int dst = which == 0 ? of.b1 : which == 1 ? of.b2 : which == 2 ? of.b3 : of.w4;
    G[dst + o] = acc;
    return;
  }
  u -= 4 * MW;
  if (u == 0) {
    float acc = 0.0f;
    for (int j = 0; j < S; j++) acc += E[j];
    G[of.b4] = acc;
  } else if (u == 1) {
    float acc = 0.0f;
    for (int j = 0; j < S; j++) acc += Lj[j];
    *loss = acc;
  }
}

// Adam with decoupled weight decay on the weights (not the biases)
__global__ void k_mlp_adam(Offs of, float* P, const float* G, float* Mo, float* Ve, int* step, float lr, float b1,
                           float b2, float eps, float wd) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= of.n) return;
  const int k = *step + 1;
  const float g = G[t];
  const float mo = b1 * Mo[t] + (1.0f - b1) * g;
  const float ve = b2 * Ve[t] + (1.0f - b2) * g * g;
  Mo[t] = mo;
  Ve[t] = ve;
  const float mh = mo / (1.0f - powf(b1, (float)k)), vh = ve / (1.0f - powf(b2, (float)k));
  const bool is_w = (t < of.b1) || (t >= of.W2 && t < of.b2) || (t >= of.W3 && t < of.b3) || (t >= of.w4 && t < of.b4);
  float p = P[t];
  if (is_w) p -= lr * wd * p;
  P[t] = p - lr * mh / (sqrtf(vh) + eps);
}
__global__ void k_mlp_tick(int* step) { *step += 1; }

// BF16 tiled copies of W2, W3 and their transposes for the GEMMs
__global__ void k_mlp_pack(const float* P, Offs of, bf16* W2t, bf16* W2Tt, bf16* W3t, bf16* W3Tt) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= MW * MW) return;
  const int o = t / MW, i = t % MW;
  const bf16 a = __float2bfloat16_rn(P[of.W2 + t]), b = __float2bfloat16_rn(P[of.W3 + t]);
  W2t[umma_off(o, i, MW)] = a;
  W2Tt[umma_off(i, o, MW)] = a;
  W3t[umma_off(o, i, MW)] = b;
  W3Tt[umma_off(i, o, MW)] = b;
}

inline int nblk(int n, int t) { return (n + t - 1) / t; }

void launch_pack() {
  count_launch_external();
  k_mlp_pack<<<nblk(MW * MW, 256), 256, 0, m->st>>>(m->P, m->of, m->W2t, m->W2Tt, m->W3t, m->W3Tt);
}

// forward through both GEMMs for S points of X with nch channels
void launch_forward(const float* X, int S, int nch) {
  const int Spad = (S + 127) / 128 * 128, R = nch * Spad;
  const int nb = nblk(Spad * MW, 256);
  cudaStream_t st = m->st;
  count_launch_external();
  k_mlp_l1<<<nb, 256, 0, st>>>(m->P, m->of, X, S, Spad, m->nin, nch, m->A1, m->A1T);
  launch_umma_gemm(m->A1, m->W2t, m->Z2, R, MW, 0, m->status, st);
  count_launch_external();
  k_mlp_act<<<nb, 256, 0, st>>>(m->Z2, m->P + m->of.b2, S, Spad, nch, m->A2, m->A2T);
  launch_umma_gemm(m->A2, m->W3t, m->Z3, R, MW, 0, m->status, st);
  count_launch_external();
  k_mlp_head<<<nblk(nch * S * 32, 256), 256, 0, st>>>(m->P, m->of, m->Z3, S, Spad, nch, m->F);
}

// loss and every parameter gradient at the current weights (into G)
void launch_loss_grad() {
  const int S = m->S, nch = 1 + m->nin;
  const int Spad = (S + 127) / 128 * 128, R = nch * Spad;
  const int nb = nblk(Spad * MW, 256);
  cudaStream_t st = m->st;
  launch_forward(m->X, S, nch);
  count_launch_external();
  k_mlp_loss<<<nblk(Spad, 128), 128, 0, st>>>(m->F, m->Y, m->DY, m->GW, S, Spad, m->nin, nch, (float)m->cfg.grad_weight,
                                              m->E, m->Lj);
  count_launch_external();
  k_mlp_head_bwd<<<nb, 256, 0, st>>>(m->P, m->of, m->Z3, m->E, S, Spad, nch, m->GZ, m->GZT, m->T4, m->GZB3);
  launch_umma_gemm(m->GZ, m->W3Tt, m->GA, R, MW, 0, m->status, st);          // dL/d act2
  launch_umma_gemm(m->GZT, m->A2T, m->G + m->of.W3, MW, R, 0, m->status, st);  // dL/dW3
  count_launch_external();
  k_mlp_act_bwd<<<nb, 256, 0, st>>>(m->Z2, m->P + m->of.b2, m->GA, S, Spad, nch, m->GZ, m->GZT, m->GZB2);
  launch_umma_gemm(m->GZ, m->W2Tt, m->GA, R, MW, 0, m->status, st);          // dL/d act1
  launch_umma_gemm(m->GZT, m->A1T, m->G + m->of.W2, MW, R, 0, m->status, st);  // dL/dW2
  count_launch_external();
  k_mlp_l1_bwd<<<nb, 256, 0, st>>>(m->P, m->of, m->X, m->GA, S, Spad, m->nin, nch, m->GZ1, m->GDZ1);
  count_launch_external();
  k_mlp_reduce<<<nblk(MW * m->nin + 4 * MW + 2, 128), 128, 0, st>>>(m->of, m->X, m->E, m->Lj, m->GZ1, m->GDZ1,
                                                                     m->T4, m->GZB2, m->GZB3, S, Spad, m->nin, nch,
                                                                     m->G, m->loss);
}

void launch_train_step() {
  launch_loss_grad();
  cudaStream_t st = m->st;
  const vca_mlp_config& c = m->cfg;
  count_launch_external();
  k_mlp_adam<<<nblk(m->of.n, 256), 256, 0, st>>>(m->of, m->P, m->G, m->Mo, m->Ve, m->step, (float)c.lr,
                                                 (float)c.beta1, (float)c.beta2, (float)c.adam_eps,
                                                 (float)c.weight_decay);
  count_launch_external();
  k_mlp_tick<<<1, 1, 0, st>>>(m->step);
  launch_pack();
}

int check_status() {
  int s = 0;
  MCU(cudaMemcpyAsync(&s, m->status, sizeof(int), cudaMemcpyDeviceToHost, m->st));
  MCU(cudaStreamSynchronize(m->st));
  if (s != 0) {
    cudaMemsetAsync(m->status, 0, sizeof(int), m->st);
    MFAIL(VCA_ERR_TIMEOUT, "a bounded wait of the tensor-core GEMM ran out (status " + std::to_string(s) + ")");
  }
  return VCA_OK;
}

uint64_t mix64(uint64_t x) {
  uint64_t z = x + 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

void drop_graph() {
  if (m && m->gexec) {
    cudaGraphExecDestroy(m->gexec);
    m->gexec = nullptr;
    m->gS = -1;
  }
}

int umma_check(const uint16_t* A, const uint16_t* B, float* C, int32_t M, int32_t K, int32_t accumulate,
               uint32_t extra_tx);

}  // namespace

extern "C" {

void vca_mlp_config_defaults(vca_mlp_config* c) {
  if (!c) return;
  std::memset(c, 0, sizeof(*c));
  c->n_in = 4;
  c->capacity = 4096;
  c->seed = 20261203;
  c->lr = 2e-3;
  c->beta1 = 0.9;
  c->beta2 = 0.999;
  c->adam_eps = 1e-8;
  c->grad_weight = 1.0;
  c->weight_decay = 0.0;
}

int vca_mlp_finalize(void) {
  if (!m) return VCA_OK;
  drop_graph();
  for (void* p : m->mem) cudaFree(p);
  if (m->st) cudaStreamDestroy(m->st);
  delete m;
  m = nullptr;
  return VCA_OK;
}

int vca_mlp_init(const vca_mlp_config* cfg) {
  if (!cfg) MFAIL(VCA_ERR_ARG, "cfg is NULL");
  if (cfg->n_in < 1 || cfg->n_in > MAXIN) MFAIL(VCA_ERR_CONFIG, "the surrogate takes 1 to 4 inputs");
  if (cfg->capacity < 1 || cfg->capacity > (1 << 20)) MFAIL(VCA_ERR_CONFIG, "capacity must be in 1..2^20");
  vca_mlp_finalize();
  m = new Mlp();
  m->cfg = *cfg;
  m->nin = cfg->n_in;
  m->cap = cfg->capacity;
  m->capPad = (m->cap + 127) / 128 * 128;
  m->of = offsets(m->nin);
  const int nch = 1 + m->nin;
  const size_t R = (size_t)nch * m->capPad;
  int rc = VCA_OK;
  auto fail = [&](int r) { vca_mlp_finalize(); return r; };
  if (cudaStreamCreateWithFlags(&m->st, cudaStreamNonBlocking) != cudaSuccess || umma_prepare() != cudaSuccess) {
    vca_mlp_finalize();
    MFAIL(VCA_ERR_CUDA, "stream creation or tensor-core kernel set-up failed");
  }
  const size_t np = m->of.n;
  if ((rc = malloc_n(&m->P, np)) || (rc = malloc_n(&m->G, np)) || (rc = malloc_n(&m->Mo, np)) ||
      (rc = malloc_n(&m->Ve, np)) || (rc = malloc_n(&m->W2t, MW * MW)) || (rc = malloc_n(&m->W2Tt, MW * MW)) ||
      (rc = malloc_n(&m->W3t, MW * MW)) || (rc = malloc_n(&m->W3Tt, MW * MW)) ||
      (rc = malloc_n(&m->X, (size_t)m->cap * m->nin)) || (rc = malloc_n(&m->Y, m->cap)) ||
      (rc = malloc_n(&m->DY, (size_t)m->cap * m->nin)) || (rc = malloc_n(&m->GW, m->cap)) || (rc = malloc_n(&m->Xq, (size_t)m->cap * m->nin)) ||
      (rc = malloc_n(&m->A1, R * MW)) || (rc = malloc_n(&m->A1T, R * MW)) || (rc = malloc_n(&m->A2, R * MW)) ||
      (rc = malloc_n(&m->A2T, R * MW)) || (rc = malloc_n(&m->GZ, R * MW)) || (rc = malloc_n(&m->GZT, R * MW)) ||
      (rc = malloc_n(&m->Z2, R * MW)) || (rc = malloc_n(&m->Z3, R * MW)) || (rc = malloc_n(&m->GA, R * MW)) ||
      (rc = malloc_n(&m->E, R)) || (rc = malloc_n(&m->F, R)) || (rc = malloc_n(&m->Lj, m->capPad)) ||
      (rc = malloc_n(&m->GZ1, (size_t)m->capPad * MW)) ||
      (rc = malloc_n(&m->GDZ1, (size_t)m->nin * m->capPad * MW)) ||
      (rc = malloc_n(&m->T4, (size_t)m->capPad * MW)) || (rc = malloc_n(&m->GZB2, (size_t)m->capPad * MW)) ||
      (rc = malloc_n(&m->GZB3, (size_t)m->capPad * MW)) || (rc = malloc_n(&m->loss, 1)) ||
      (rc = malloc_n(&m->status, 1)) || (rc = malloc_n(&m->step, 1)))
    return fail(rc);
  if (cudaMemsetAsync(m->status, 0, sizeof(int), m->st) != cudaSuccess ||
      cudaMemsetAsync(m->step, 0, sizeof(int), m->st) != cudaSuccess ||
      cudaMemsetAsync(m->Mo, 0, np * sizeof(float), m->st) != cudaSuccess ||
      cudaMemsetAsync(m->Ve, 0, np * sizeof(float), m->st) != cudaSuccess ||
      cudaMemsetAsync(m->G, 0, np * sizeof(float), m->st) != cudaSuccess)
    return fail(VCA_ERR_CUDA);
  // Glorot-uniform weights from the seed, zero biases
  std::vector<float> p(np, 0.0f);
  uint64_t ctr = cfg->seed * 0x2545F4914F6CDD1Dull;
  auto uni = [&](double a) { return (float)(a * (2.0 * (double)(mix64(ctr++) >> 11) / 9007199254740992.0 - 1.0)); };
  const Offs& of = m->of;
  for (int t = 0; t < MW * m->nin; t++) p[of.W1 + t] = uni(std::sqrt(6.0 / (m->nin + MW)));
  for (int t = 0; t < MW * MW; t++) p[of.W2 + t] = uni(std::sqrt(6.0 / (2 * MW)));
  for (int t = 0; t < MW * MW; t++) p[of.W3 + t] = uni(std::sqrt(6.0 / (2 * MW)));
  for (int t = 0; t < MW; t++) p[of.w4 + t] = uni(std::sqrt(6.0 / (MW + 1)));
  if (cudaMemcpyAsync(m->P, p.data(), np * sizeof(float), cudaMemcpyHostToDevice, m->st) != cudaSuccess)
    return fail(VCA_ERR_CUDA);
  launch_pack();
  if (cudaStreamSynchronize(m->st) != cudaSuccess) return fail(VCA_ERR_CUDA);
  return VCA_OK;
}

int64_t vca_mlp_param_count(void) { return m ? (int64_t)m->of.n : -1; }

int vca_mlp_get_params(float* out, int64_t n) {
  if (!m) MFAIL(VCA_ERR_STATE, "vca_mlp_init has not been called");
  if (!out || n < m->of.n) MFAIL(VCA_ERR_ARG, "parameter buffer too small");
  MCU(cudaMemcpyAsync(out, m->P, sizeof(float) * m->of.n, cudaMemcpyDeviceToHost, m->st));
  MCU(cudaStreamSynchronize(m->st));
  return VCA_OK;
}

int vca_mlp_set_params(const float* in, int64_t n) {
  if (!m) MFAIL(VCA_ERR_STATE, "vca_mlp_init has not been called");
  if (!in || n != m->of.n) MFAIL(VCA_ERR_ARG, "parameter count mismatch");
  MCU(cudaMemcpyAsync(m->P, in, sizeof(float) * m->of.n, cudaMemcpyHostToDevice, m->st));
  MCU(cudaMemsetAsync(m->Mo, 0, sizeof(float) * m->of.n, m->st));
  MCU(cudaMemsetAsync(m->Ve, 0, sizeof(float) * m->of.n, m->st));
  MCU(cudaMemsetAsync(m->step, 0, sizeof(int), m->st));
  launch_pack();
  MCU(cudaStreamSynchronize(m->st));
  return VCA_OK;
}

int vca_mlp_set_data(int32_t n, const double* x, const double* y, const double* dy, const double* gw) {
  if (!m) MFAIL(VCA_ERR_STATE, "vca_mlp_init has not been called");
  if (n < 1 || n > m->cap) MFAIL(VCA_ERR_ARG, "sample count outside 1..capacity");
  if (!x || !y) MFAIL(VCA_ERR_ARG, "x and y are required");
  const int nin = m->nin;
  std::vector<float> fx((size_t)n * nin), fy(n), fd((size_t)n * nin, 0.0f), fw(n, 1.0f);
  for (size_t i = 0; i < fx.size(); i++) fx[i] = (float)x[i];
  if (gw)
    for (int i = 0; i < n; i++) {
      if (!(gw[i] >= 0.0) || !std::isfinite(gw[i])) MFAIL(VCA_ERR_NUMERIC, "gradient weights must be finite and >= 0");
      fw[i] = (float)gw[i];
    }
  for (int i = 0; i < n; i++) fy[i] = (float)y[i];
  if (dy)
    for (size_t i = 0; i < fd.size(); i++) fd[i] = (float)dy[i];
  for (float v : fx)
    if (!std::isfinite(v)) MFAIL(VCA_ERR_NUMERIC, "x holds NaN or Inf");
  for (float v : fy)
    if (!std::isfinite(v)) MFAIL(VCA_ERR_NUMERIC, "y holds NaN or Inf");
  MCU(cudaMemcpyAsync(m->X, fx.data(), fx.size() * sizeof(float), cudaMemcpyHostToDevice, m->st));
  MCU(cudaMemcpyAsync(m->Y, fy.data(), fy.size() * sizeof(float), cudaMemcpyHostToDevice, m->st));
  MCU(cudaMemcpyAsync(m->DY, fd.data(), fd.size() * sizeof(float), cudaMemcpyHostToDevice, m->st));
  MCU(cudaMemcpyAsync(m->GW, fw.data(), fw.size() * sizeof(float), cudaMemcpyHostToDevice, m->st));
  MCU(cudaStreamSynchronize(m->st));
  if (n != m->S) drop_graph();
  m->S = n;
  return VCA_OK;
}

int vca_mlp_loss_grad(double* loss, float* grad, int64_t n) {
  if (!m) MFAIL(VCA_ERR_STATE, "vca_mlp_init has not been called");
  if (m->S < 1) MFAIL(VCA_ERR_STATE, "no training data (vca_mlp_set_data)");
  if (grad && n < m->of.n) MFAIL(VCA_ERR_ARG, "gradient buffer too small");
  launch_loss_grad();
  MCU(cudaGetLastError());
  int rc = check_status();
  if (rc) return rc;
  float l = 0.0f;
  MCU(cudaMemcpyAsync(&l, m->loss, sizeof(float), cudaMemcpyDeviceToHost, m->st));
  if (grad) MCU(cudaMemcpyAsync(grad, m->G, sizeof(float) * m->of.n, cudaMemcpyDeviceToHost, m->st));
  MCU(cudaStreamSynchronize(m->st));
  if (loss) *loss = l;
  return VCA_OK;
}

int vca_mlp_train(int32_t steps, double* loss) {
  if (!m) MFAIL(VCA_ERR_STATE, "vca_mlp_init has not been called");
  if (m->S < 1) MFAIL(VCA_ERR_STATE, "no training data (vca_mlp_set_data)");
  if (steps < 0) MFAIL(VCA_ERR_ARG, "steps must be >= 0");
  if (m->gS != m->S) {  // one training step captured as a CUDA graph, replayed
    drop_graph();
    cudaGraph_t gr;
    MCU(cudaStreamBeginCapture(m->st, cudaStreamCaptureModeThreadLocal));
    launch_train_step();
    MCU(cudaStreamEndCapture(m->st, &gr));
    cudaError_t e = cudaGraphInstantiate(&m->gexec, gr, 0);
    cudaGraphDestroy(gr);
    MCU(e);
    m->gS = m->S;
  }
  for (int s = 0; s < steps; s++) MCU(cudaGraphLaunch(m->gexec, m->st));
  int rc = check_status();
  if (rc) return rc;
  if (loss) {  // the loss at the final weights
    double l;
    rc = vca_mlp_loss_grad(&l, nullptr, 0);
    if (rc) return rc;
    *loss = l;
  }
  return VCA_OK;
}

int vca_mlp_predict(int32_t n, const double* x, double* f, double* df) {
  if (!m) MFAIL(VCA_ERR_STATE, "vca_mlp_init has not been called");
  if (n < 1 || n > m->cap) MFAIL(VCA_ERR_ARG, "point count outside 1..capacity");
  if (!x || !f) MFAIL(VCA_ERR_ARG, "x and f are required");
  const int nin = m->nin, nch = df ? 1 + nin : 1;
  std::vector<float> fx((size_t)n * nin);
  for (size_t i = 0; i < fx.size(); i++) fx[i] = (float)x[i];
  MCU(cudaMemcpyAsync(m->Xq, fx.data(), fx.size() * sizeof(float), cudaMemcpyHostToDevice, m->st));
  launch_forward(m->Xq, n, nch);
  MCU(cudaGetLastError());
  int rc = check_status();
  if (rc) return rc;
  const int Spad = (n + 127) / 128 * 128;
  std::vector<float> out((size_t)nch * Spad);
  MCU(cudaMemcpyAsync(out.data(), m->F, out.size() * sizeof(float), cudaMemcpyDeviceToHost, m->st));
  MCU(cudaStreamSynchronize(m->st));
  for (int j = 0; j < n; j++) {
    f[j] = out[j];
    if (df)
      for (int d = 0; d < nin; d++) df[(size_t)j * nin + d] = out[(size_t)(d + 1) * Spad + j];
  }
  return VCA_OK;
}

// C = A B^T (+ C) through the tensor-core GEMM, for tests: A [M][K] and B
// [128][K] row-major bf16 bit patterns on the host, C [M][128] FP32
int vca_umma_gemm_check(const uint16_t* A, const uint16_t* B, float* C, int32_t M, int32_t K, int32_t accumulate) {
  return umma_check(A, B, C, M, K, accumulate, 0);
}

// The same GEMM with every load barrier expecting 16 bytes more than its
// copies deliver: the bounded wait must run out, the call must return
// VCA_ERR_TIMEOUT, and the context must stay usable.
int vca_umma_timeout_check(void) {
  std::vector<uint16_t> a((size_t)128 * 64, 0), b((size_t)128 * 64, 0);
  std::vector<float> c((size_t)128 * 128, 0.0f);
  return umma_check(a.data(), b.data(), c.data(), 128, 64, 0, 16);
}

}  // extern "C"

namespace {
int umma_check(const uint16_t* A, const uint16_t* B, float* C, int32_t M, int32_t K, int32_t accumulate,
               uint32_t extra_tx) {
  if (!A || !B || !C) MFAIL(VCA_ERR_ARG, "null buffer");
  if (M < 128 || M % 128 || K < 64 || K % 64 || (size_t)M * K > (size_t)1 << 28)
    MFAIL(VCA_ERR_ARG, "M must be a positive multiple of 128 and K of 64");
  std::vector<uint16_t> ta((size_t)M * K), tb((size_t)128 * K);
  for (int r = 0; r < M; r++)
    for (int k = 0; k < K; k++) ta[umma_off(r, k, K)] = A[(size_t)r * K + k];
  for (int r = 0; r < 128; r++)
    for (int k = 0; k < K; k++) tb[umma_off(r, k, K)] = B[(size_t)r * K + k];
  bf16 *dA = nullptr, *dB = nullptr;
  float* dC = nullptr;
  int* dst = nullptr;
  cudaStream_t st = nullptr;
  int rc = VCA_OK;
  int s = 0;
  if (umma_prepare() != cudaSuccess) MFAIL(VCA_ERR_CUDA, "tensor-core kernel set-up failed");
  if (cudaMalloc(&dA, ta.size() * 2) != cudaSuccess || cudaMalloc(&dB, tb.size() * 2) != cudaSuccess ||
      cudaMalloc(&dC, (size_t)M * 128 * 4) != cudaSuccess || cudaMalloc(&dst, 4) != cudaSuccess ||
      cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) {
    rc = VCA_ERR_ALLOC;
    set_api_error("device allocation failed in vca_umma_gemm_check");
  } else {
    cudaMemcpyAsync(dA, ta.data(), ta.size() * 2, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(dB, tb.data(), tb.size() * 2, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(dC, C, (size_t)M * 128 * 4, cudaMemcpyHostToDevice, st);
    cudaMemsetAsync(dst, 0, 4, st);
    launch_umma_gemm(dA, dB, dC, M, K, accumulate ? 1 : 0, dst, st, extra_tx);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(C, dC, (size_t)M * 128 * 4, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&s, dst, 4, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
      rc = VCA_ERR_CUDA;
      set_api_error(std::string("CUDA error in vca_umma_gemm_check: ") + cudaGetErrorString(e));
    } else if (s != 0) {
      rc = VCA_ERR_TIMEOUT;
      set_api_error("a bounded wait of the tensor-core GEMM ran out (status " + std::to_string(s) + ")");
    }
  }
  if (st) cudaStreamDestroy(st);
  cudaFree(dA);
  cudaFree(dB);
  cudaFree(dC);
  cudaFree(dst);
  return rc;
}

}  // namespace
