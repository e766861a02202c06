// vca_common.cuh -- shared types of the GB300 cluster-ED path.
//
// Layout conventions (fixed across kernels):
//  * A sector (n_up, n_dw) vector is the DimUp x DimDw matrix V with the up
//    index fastest: element i = iup + idw*DimUp (0-based), the state order of
//    VCA_SETUP.f90:505-518.
//  * A "column batch" holds m vectors of one sector interleaved element-major:
//    X[i*m + c].  Real Hamiltonians store real columns (a complex chain owns
//    two consecutive columns, re and im); complex Hamiltonians store double2
//    columns.
//  * Fock words are the reference's: bit l-1 = orbital l, cluster orbitals
//    first (is = iorb + (ilat-1)*Norb), bath levels after (VCA_SETUP.f90:
//    341-349, 705-710).  Maps are ascending words of fixed popcount
//    (build_sector, VCA_SETUP.f90:660-695), i.e. the colex order of the
//    combinatorial number system, so rank(w) = sum_i C(c_i, i).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#define VCA_MAX_NS 24      // Fock words are int32; 2^24 words per spin max
#define VCA_MAX_NORB 5
#define VCA_MAX_PAIRS 576  // ordered (i,j) one-body pairs with nonzero amplitude

namespace vca {

struct Binom {
  int64_t c[VCA_MAX_NS + 1][VCA_MAX_NS + 1];
};

// One spin-resolved Fock space of fixed filling n: map + pull hop table.
// Row r (target word) lists hops from source rank src[k*dim + r] with
// amplitude amp[k*dim + r], k < cnt[r] (ELL, k-major for coalescing).
struct SpinSpace {
  int n = -1;
  int dim = 0;
  int width = 0;          // ELL width = max hops per row
  int* words = nullptr;   // [dim]
  int* cnt = nullptr;     // [dim]
  int* src = nullptr;     // [width*dim]
  double2* amp = nullptr; // [width*dim]
  double2* e1 = nullptr;  // [dim] one-body + same-spin diagonal energy
};

// Device view of one sector for the H x v kernels.
struct SectorView {
  int dimup, dimdw;
  int wup, wdw;              // ELL widths
  const int* up_words;
  const int* dw_words;
  const int* up_cnt;
  const int* dw_cnt;
  const int* up_src;
  const int* dw_src;
  const double2* up_amp;
  const double2* dw_amp;
  const double2* up_e1;
  const double2* dw_e1;
};

// Opposite-spin (mixed) diagonal terms: sum_o U_o popc(u & d & m_o)
// + Ust sum_{o<p} [popc(u & m_o & (d >> (p-o))) + popc(u & m_p & (d << (p-o)))]
struct MixedDiag {
  int norb;
  unsigned int omask[VCA_MAX_NORB];
  double U[VCA_MAX_NORB];
  double Ust;
  double c0;  // constant Hartree shifts (H_cluster_local.f90:59-76), hfmode only
};

#ifdef __CUDACC__
// opposite-spin density-density terms (H_cluster_local.f90:26-45)
__device__ __forceinline__ double mixed_diag(const MixedDiag& md, unsigned u, unsigned d) {
  double s = 0.0;
  for (int o = 0; o < md.norb; o++) s += md.U[o] * (double)__popc(u & d & md.omask[o]);
  int c = 0;
  for (int o = 0; o < md.norb; o++)
    for (int q = o + 1; q < md.norb; q++)
      c += __popc(u & md.omask[o] & (d >> (q - o))) + __popc(u & md.omask[q] & (d << (q - o)));
  if (c) s += md.Ust * (double)c;
  return s + md.c0;
}
#endif

// Per-chain Lanczos bookkeeping for a column batch.
struct ChainMeta {
  int ncol;       // columns of this chain (1 real, 2 complex on real H)
  int col0;       // first column
  int nlanc;      // requested steps
  int active;     // 1 while running
  int len;        // steps done
};

}  // namespace vca
