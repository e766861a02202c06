// vca_batch.cuh -- column batches of many (point, target sector) tasks: the
// Green's-function chains of the batched form.
//
// A task is one point's chains into one target sector, m columns stored
// element-major at X[xoff + i*m + c] (a complex chain on a real H owns two
// columns, re and im, as in the single-sector column batches).  Every task's
// rows are cut into tiles (their height and the block's row lanes are the
// autotuned shape); each Lanczos phase is one launch over all tiles of all
// tasks, so the hop tables of a task's point are read once per element for
// all its columns.  Reductions are fixed-order: per (tile,
// column) partials, then one warp per chain over its columns and tiles.
#pragma once

#include "vca_common.cuh"
#include "vca_kernels.cuh"
#include "vca_multi.cuh"

namespace vca {

#define MC_ROWS 64    // default rows per tile
#define MC_BY_MAX 16  // most row lanes per block (blockDim.y)

struct McTask {
  SectorView sv;
  int64_t D;      // rows: the target sector's dimension
  int m;          // columns
  int col0;       // first column of the task (global column numbering)
  int64_t xoff;   // element offset of the task's block
  int tile0, ntile;
  int64_t part0;  // partial (tile, c) at part0 + c * ntile + (tile - tile0): a column's tiles contiguous
};

struct McChain {  // one chain: columns col0 .. col0 + ncol - 1 of task `task`
  int task, col0, ncol;
  MtChain op;     // its start vector: operator terms on its point's ground state
};

struct McGroup {  // device tables of one group of tasks
  const McTask* tasks;
  const int* tile_task;
  const int64_t* tile_row0;
  const int64_t* tile_row1;  // rows [row0, row1) of each tile
  const int* col_chain;   // global column -> chain
  const int* col_part;    // global column -> 0 (re) / 1 (im) part of its chain
  const McChain* chains;
  int ntasks, ntiles, ncols, nch;
  int by;     // row lanes per block (blockDim = 32 x by, by <= MC_BY_MAX)
};

// start vectors of every chain's columns and the per-(tile, column) |x|^2
void mc_launch_chain_init(const McGroup& gp, bool cplx, void* X, double* tpart, cudaStream_t st);
// out[ch] = sum over the chain's columns and its task's tiles of tpart (fixed order)
void mc_launch_reduce(const McGroup& gp, const double* tpart, double* out, cudaStream_t st);
// Y = H X - bnow[ch] Xp (use_b) and <x, y> partials
void mc_launch_hxv(const McGroup& gp, bool cplx, const MixedDiag& md, const ChainMeta* meta, const double* bnow,
                   int use_b, const void* X, const void* Xp, void* Y, double* tpart, cudaStream_t st);
// Y -= alpha[ch] X and |y|^2 partials (inactive chains: partial 0)
void mc_launch_update(const McGroup& gp, bool cplx, const ChainMeta* meta, const double* alpha, const void* X,
                      void* Y, double* tpart, cudaStream_t st);
// Xo = f[ch] Xi (0 for inactive chains)
void mc_launch_scale(const McGroup& gp, bool cplx, const ChainMeta* meta, const double* f, const void* Xi, void* Xo,
                     cudaStream_t st);

}  // namespace vca
