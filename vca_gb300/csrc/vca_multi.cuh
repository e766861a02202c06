// vca_multi.cuh -- batched multi-sector ground-state Lanczos (fixed point).
#pragma once

#include <algorithm>

#include "vca_fx.cuh"

namespace vca {

#define MS_TILE 1024

struct MsSector {
  SectorView sv;
  FxView fv;
  int64_t off;   // element offset of this sector in the packed vectors
  int64_t D;
  int tile0, ntile;
  int isector;   // 1-based sector number (start-vector seed)
  int ncomp;     // FP64 tasks: 2 when the task's vector is [re; im] of a complex
                 // chain on a real H (length 2 * DimUp * DimDw), else 0 or 1
};

struct MsGroup {   // device tables of one group of sectors
  const MsSector* secs;
  const int* tsec;        // tile -> sector (group-local index)
  const int64_t* tstart;  // tile -> first element within its sector
  int nsec, ntiles;
};

struct MsBufs {
  i64 *X, *Xp, *YW;       // packed vectors
  i64* tpart;             // int128 partial per tile
  ChainMeta* meta;        // per sector
  double *alpha, *bnow, *A, *Bt, *svec, *theta, *resid;
  i64 *afx, *bfx, *mul;
  int *msh, *state, *mconv, *undone;
  int ld;                 // coefficient stride per sector (nmax + 1)
};

void ms_launch_start(const MsGroup& gp, uint64_t seed, int F, i64* R, i64* X, i64* tpart, ChainMeta* meta,
                     i64* mul, int* msh, cudaStream_t st);
void ms_launch_step(const MsGroup& gp, const FxScales& fs, int K, int k, double tol, MsBufs& b, cudaStream_t st);
void ms_launch_check(const MsGroup& gp, MsBufs& b, double tol, cudaStream_t st);

// the same search in FP64: vectors of double (real H) or double2 (complex H)
struct Ms64Bufs {
  void *X, *Xp, *Y;       // packed vectors
  double* tpart;          // per-tile partial sums
  ChainMeta* meta;        // per sector
  double *alpha, *bnow, *invb, *A, *Bt, *svec, *theta, *resid;
  int *state, *mconv, *undone;
  int ld;
};
void m64_launch_start(const MsGroup& gp, bool cplx, uint64_t seed, Ms64Bufs& b, cudaStream_t st);
void m64_launch_step(const MsGroup& gp, bool cplx, const MixedDiag& md, int k, double tol, Ms64Bufs& b,
                     cudaStream_t st);
void m64_launch_check(const MsGroup& gp, Ms64Bufs& b, double tol, cudaStream_t st);

// ---- multi-task Lanczos over many variational points (the batched form) --
// The FP64 step kernels above run any list of tasks: the (point, sector)
// ground-state searches and their eigenvector passes; a task's SectorView
// carries its point's hop tables.  (The chains run as column batches,
// vca_batch.cuh.)
//
// A chain's start vector is an operator applied to its point's ground
// state: sum_q coef_q c^(dag)_{pos_q, spin}|gs> (VCA_GF_NORMAL.f90:121-318,
// 561-958), gathered per target element with the reference's one-word signs.
struct MtChain {
  const void* gs;   // source ground state: double (real H) or double2 (complex H)
  int src_dimup;    // DimUp of the ground state's sector
  int spin, dag, nterm;
  int pos[2];
  double cre[2], cim[2];
};
// per task: n2 = |x|^2 (fixed-order sum of the tile partials), invn = 1/|x|
// (0 and the task retired when the vector vanishes)
void mt_launch_norm(const MsGroup& gp, const double* tpart, ChainMeta* meta, double* n2, double* invn,
                    cudaStream_t st);
// Xo = f[task] Xi
void m64_launch_scale(const MsGroup& gp, bool cplx, const double* f, const void* Xi, void* Xo, cudaStream_t st);
// psi += svec[task * ld5 + k - 1] X for the tasks with k <= mconv[task]
void m64_launch_psi(const MsGroup& gp, bool cplx, const double* svec, int ld5, const int* mconv, int k,
                    const void* X, void* psi, cudaStream_t st);
// per-tile |x|^2 partials
void m64_launch_sqnorm(const MsGroup& gp, bool cplx, const void* X, double* tpart, cudaStream_t st);

}  // namespace vca
