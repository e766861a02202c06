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
  int pad;
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

}  // namespace vca
