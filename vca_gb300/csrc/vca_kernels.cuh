// vca_kernels.cuh -- host-callable launchers of the sm_103a kernels.
#pragma once

#include "vca_common.cuh"

namespace vca {

// number of kernel launches issued by this library since load
long long launch_count();

// ---- Fock basis (VCA_SETUP.f90:660-695, 724-750) ---------------------------
void set_binomials(int Ns, cudaStream_t st);
void launch_build_words(int Ns, int n, int dim, int* words, cudaStream_t st);

struct HopPair {     // amplitude of c^dag_i c_j for one spin (i != j), 0-based bits
  int i, j;
  double re, im;
};
struct E1Params {    // one-body + same-spin diagonal energy of a spin word
  double2 eps[VCA_MAX_NS];   // per-level energy (incl. -xmu and Hartree shifts)
  double2 cst;               // constant added once (carried by the up word)
  double upar;               // (Ust - Jh), same site, parallel spins
  int norb;
  unsigned int omask[VCA_MAX_NORB];
};
// count hops per target word and return the ELL width (max count)
int launch_hop_count(int Ns, int n, int dim, const int* words, const HopPair* d_pairs, int npairs,
                     int* cnt, int* d_scratch_max, cudaStream_t st);
void launch_hop_fill(int Ns, int n, int dim, int width, const int* words, const HopPair* d_pairs,
                     int npairs, int* src, double2* amp, cudaStream_t st);
void launch_e1(int dim, const int* words, const E1Params& p, bool with_const, double2* e1,
               cudaStream_t st);

// ---- H x v on column batches (VCA_HAMILTONIAN_SPARSE_HxV.f90:152-200) -----
// real Hamiltonian, m real columns
void launch_hxv_real(const SectorView& sv, const MixedDiag& md, int m, const double* X, double* Y,
                     cudaStream_t st);
// complex Hamiltonian, m complex columns
void launch_hxv_cplx(const SectorView& sv, const MixedDiag& md, int m, const double2* X, double2* Y,
                     cudaStream_t st);

// ---- Lanczos vector operations on column batches --------------------------
// Work arrays: partial[nblk*m] (double2), chain arrays of length nch.
struct ColBatch {
  int64_t rows;     // sector dimension
  int m;            // columns (real doubles, or double2 when cplx)
  bool cplx;        // double2 columns
  int nch;          // chains
  const int* col2ch;  // [m]
  const ChainMeta* meta;  // [nch] device
};
// per-column dot: out_col[c] = sum_i conj(X)Y (real part used) ; deterministic
void launch_col_dot(const ColBatch& b, const void* X, const void* Y, double* partial, int nblk,
                    double* out_col, cudaStream_t st);
// Y -= coef[ch(c)] * X  for active chains
void launch_col_axpy(const ColBatch& b, const double* coef, const void* X, void* Y, bool negate,
                     cudaStream_t st);
// X = Y * scale[ch(c)] for active chains
void launch_col_scale(const ColBatch& b, const double* scale, const void* Y, void* X, cudaStream_t st);
// sum columns of each chain: out_ch[ch] = sum_{c in ch} in_col[c]
void launch_chain_sum(const ColBatch& b, const double* in_col, double* out_ch, cudaStream_t st);
// after alpha/beta^2 of step k are known: record, deactivate exhausted chains,
// produce 1/beta for the scale.  alpha/beta stored [ch*ldab + k-1].
void launch_lanczos_record(int nch, ChainMeta* meta, int k, const double* alpha_ch,
                           const double* beta2_ch, double* A, double* Bt, int ldab, double tol,
                           double* invbeta, double* beta_now, cudaStream_t st);
// psi += s[k] * X (single column batch of the GS second pass)
void launch_psi_accum(int64_t n, bool cplx, const double* s, int k, const void* X, void* psi,
                      cudaStream_t st);
// deterministic start vector (splitmix64) for the GS Lanczos
void launch_start_vector(int64_t n, uint64_t seed, int isector, double* X, cudaStream_t st);
void launch_fill(int64_t n, double v, double* X, cudaStream_t st);

// ---- tridiagonal problems --------------------------------------------------
// lowest eigenpair of T_k (a[0..k-1], b = beta_{2..k}), residual test;
// writes theta, s[0..k-1] and flag (1 = converged)
void launch_tri_lowest(const double* A, const double* Bt, int k, double btail, double* theta,
                       double* s, double* resid, cudaStream_t st);
// Device store of every Green's function chain: tridiagonal rows A, B
// ([nch*ld], B[j] = beta_j couples rows j-1 and j), length n, prefactor
// pes = norm^2*boltz/zeta (boltz = 1 at T=0), isign (+1 particle, -1 hole),
// channel weight factor, state energy Ei.
struct ChainStore {
  double* A;
  double* B;
  int* n;
  double* pes;
  int* isign;
  double2* wfac;
  double* Ei;
  int ld;
};
// copy one batch's chains (rows of A/Bt with stride ldab) into the store at
// chain offset base
void launch_chain_store(int nch, const ChainMeta* meta, const double* A, const double* Bt, int ldab,
                        const double* norm2, const double2* wfac, const int* isign, double Ei, double boltz,
                        double zeta, const ChainStore& cs, int base, cudaStream_t st);
// stored chains -> poles/weights (add_to_lanczos_gf_normal, VCA_GF_NORMAL.f90:970-1033);
// work: 3*ld doubles per chain; *fail counts chains whose QL needed more
// than max_iter sweeps for one eigenvalue
void launch_chain_poles(int nch, const ChainStore& cs, double* work, double* poles, double2* weights, int* nexc,
                        int max_iter, int* fail, cudaStream_t st);

// ---- chain initial vectors (VCA_GF_NORMAL.f90:179-197, :251-268, :608-646) -
struct OpTerm {
  int pos;          // 0-based bit
  double re, im;    // coefficient
};
struct ChainInit {
  int spin;         // 0 up, 1 down
  int dag;          // 1 = c^dag (particle), 0 = c (hole)
  int nterm;
  OpTerm t[2];
  int col0;         // first column of the chain
  int cplxcol;      // real-H batch: 1 when the chain owns (re,im) columns
};
// X (target sector tgt, m columns) from the ground state gs (source sector,
// its up dimension src_dimup): one thread per (target row, chain)
void launch_chain_init(const SectorView& tgt, int src_dimup, const void* gs, bool gs_cplx,
                       int nchain, const ChainInit* d_ci, int m, bool cols_cplx, void* X,
                       cudaStream_t st);

// ---- Green's function and Omega (VCA_IO/gf_cluster.f90, VCA_OMEGA.f90) ---
struct GfLayout {
  int nelem;              // spin-diagonal elements (il,jl,is,io,jo)
  const int* elem_ptr;    // [nelem+1] chains per element (CSR)
  const int* elem_chain;  // chain ids
  ChainStore cs;          // the chains' tridiagonals
};
// raw element sums at nz points z (complex): G[z*nelem + e]
void launch_gf_eval(const GfLayout& g, int nz, const double2* z, double2* G, cudaStream_t st);
// the same raw sums from pole tables (a GFmatrix read from a restart file):
// G[z*nelem + e] = sum over ptr[e] <= x < ptr[e+1] of weights[x] / (z - poles[x])
void launch_gf_eval_poles(int nelem, const int64_t* ptr, const double2* poles, const double2* weights, int nz,
                          const double2* z, double2* G, cudaStream_t st);
// recombination + lso assembly: Glso[z][N*N] from raw G
struct ClusterDims {
  int Nlat, Norb, Nspin, N;
  int chan4;  // 1 when VCA_GF_SYMMETRIC=F
};
void launch_gf_assemble(const ClusterDims& cd, int nz, const double2* Graw, double2* Glso,
                        cudaStream_t st);
// Omega integrand (sum_kmesh, VCA_OMEGA.f90:37-75): fpart[w][chunk] = sum
// over the chunk's k of kw[k] ln|det(1 + (P_w - Hk_k) G_w)| per spin block
// (kw == nullptr: weight 1), M = P - Hk on a sparse row pattern
// (rowptr/cols, lso indices), all lanes of a warp on the products and the LU
// updates.  With fpart_im (sum_kmesh_complex, :78-114) also the k-sum of the
// principal argument of det over all blocks of each k.
// pre_m: Hk holds M_k = P - H_k already (P the same at every node)
// The inverse form of the k-sum at nodes with Im z <= omega_c (T=0 real
// integrand only): Ginv / ldG from launch_ginv_blocks; Ginv = NULL: off.
struct KsumInverse {
  const double2* z = nullptr;      // the nodes
  const double2* Ginv = nullptr;   // per node, the inverse of each diagonal block of G' (lso)
  const double* ldG = nullptr;     // per node and block, ln|det G'_block|
  double omega_c = 0.0;
};
void launch_omega_ksum2(int nw, int N, int nblk, int nb, const double2* P, const double2* Glso, int64_t Nk,
                        const double2* Hk, const double* kw, const int* rowptr, const int* cols, double* fpart,
                        double* fpart_im, int kchunks, bool pre_m, const KsumInverse& ki, cudaStream_t st);
// G'^-1 and ln|det G'| of each diagonal block (nblk blocks of nb <= 32) of n lso matrices
void launch_ginv_blocks(int n, int N, int nblk, int nb, const double2* Glso, double2* Ginv, double* ldG,
                        cudaStream_t st);
// M[k] = Hl - Hk[k] for Nk lso matrices of NN elements
void launch_m_from_hk(int64_t Nk, int NN, const double2* Hl, const double2* Hk, double2* M, cudaStream_t st);
// Sigma(z) (want_g0 = false) or G0(z) on nz frequencies from G' (lso) and
// P = Delta + Hloc (per z, or one matrix): build_sigma_normal,
// VCA_GF_NORMAL.f90:1045-1111.  N <= 32.
void launch_sigma_g0(int nz, int N, const double2* z, const double2* Glso, const double2* P, bool per_z_p,
                     double xmu, bool want_g0, double2* out, cudaStream_t st);
// out[q] = A[q]^-1 (nz N x N complex, N <= 32)
void launch_inverse_batch(int nz, int N, const double2* A, double2* out, cudaStream_t st);
// custom-observable integrand partials (sum_observable_kmesh,
// VCA_OBSERVABLES.f90:408-500): fpart[w][chunk] = sum_k Re{Tr[s_k G_k(z_w)]
// - tail*Tr[s_k]/(z_w - 1.1)}, G_k = (Ginv_w - (H_k - P_w))^-1 per spin block
void launch_obs_ksum(int nw, int N, int nblk, int nb, const double2* z, const double2* Ginv, const double2* P,
                     int64_t Nk, const double2* Hk, const double2* s, int64_t sk_stride, bool tail, double* fpart,
                     int kchunks, cudaStream_t st);
// Ground-state observable partials of one state: part[(q*nimp + l)*nb + b]
// for q = n_up, n_dw, n_up*n_dw, bit l, block b < observables_blocks(D)
int observables_blocks(int64_t D);
void launch_observables(const SectorView& sv, int fmt, const void* vec, int F, int nimp, double* part,
                        cudaStream_t st);
// dst[r] = src[idx[r]] for blocks of nel double2 (k-point representatives)
void launch_gather_blocks(int64_t nrep, int64_t nel, const int64_t* idx, const double2* src, double2* dst,
                          cudaStream_t st);
void launch_reduce_rows(int nrows, int ncols, const double* in, double scale, double* out,
                        cudaStream_t st);
// Gauss-Legendre nodes on (0,1); inv: work array of n+1 doubles
void launch_gauss_legendre(int n, double* inv, double* x, double* w, cudaStream_t st);
// Delta_bath(z) (VCA_BATH_FUNCTIONS.f90:127-150) for nz points, lso N x N
void launch_delta_bath(int nz, const double2* z, int N, int Nb, const double2* hb, const double2* V,
                       double xmu, double2* work, double2* out, cudaStream_t st);

void launch_chain_init_fx(const SectorView& tgt, int src_dimup, const long long* gs, int nchain,
                          const ChainInit* d_ci, int m, bool swapped, const int* pinv, long long* X,
                          cudaStream_t st);
void count_launch_external();

// ---- helpers ---------------------------------------------------------------
void launch_chain_norm_init(int nch, ChainMeta* meta, const double* norm2, double* invnorm,
                            cudaStream_t st);
void launch_recip(int n, const double* in, double* out, cudaStream_t st);
void launch_nnn2lso(int Nlat, int Nspin, int Norb, int64_t L, const double2* in, double2* out,
                    cudaStream_t st);
void launch_add_hloc(int nw, int NN, const double2* D, const double2* H, double2* P, cudaStream_t st);
void launch_omega_nodes(int n, double scale, const double* s, const double* w, double2* z, double* W,
                        cudaStream_t st);
void launch_wsum(int n, const double* a, const double* b, double* out, cudaStream_t st);
void launch_real_to_cplx(int64_t n, const double* in, double2* out, cudaStream_t st);

// ---- Lanczos with full reorthogonalisation ("arpack" diagonalisation) ----
// V: nq stored vectors of n elements (double, or double2 when cplx).
// c[q] = <V_q, w> (conj(V_q) . w; partial needs ap_partial_len(nq) elements)
void launch_ap_proj(int64_t n, int nq, bool cplx, const void* V, const void* w, void* partial, void* c,
                    cudaStream_t st);
int ap_partial_len(int nq);
// w -= sum_q c[q] V_q
void launch_ap_orth(int64_t n, int nq, bool cplx, const void* V, const void* c, void* w, cudaStream_t st);
// x = sum_q z[q] V_q (z real, on the device)
void launch_ap_combine(int64_t n, int nq, bool cplx, const void* V, const double* z, void* x, cudaStream_t st);
// y = a*y - s*x
void launch_ap_axpby(int64_t n, bool cplx, double a, double s, const void* x, void* y, cudaStream_t st);

}  // namespace vca
