// vca_tri.cuh -- lowest eigenpair of a Lanczos tridiagonal, one warp.
//
// T_k has diagonal A[0..k-1] and off-diagonal Bt[1..k-1] (Bt[j] = beta_{j+1}
// couples rows j-1 and j).  The lowest eigenvalue comes from warp
// multisection on the Sturm count (32 interior points per round, then plain
// bisection to adjacent doubles); the eigenvector from three steps of inverse
// iteration with a partially pivoted tridiagonal LU (Wilkinson, The Algebraic
// Eigenvalue Problem, ch. 5).  The Lanczos residual estimate is
// |beta_{k+1} s_{k-1}|.  All 32 lanes must call; lane 0 writes the results.
// s needs 5*k doubles (eigenvector + LU work).  k <= 512.
#pragma once

#include <cuda_runtime.h>

namespace vca {

__device__ __forceinline__ int sturm_count_tri(const double* a, const double* b1, int k, double x) {
  int cnt = 0;
  double q = a[0] - x;
  if (q < 0) cnt++;
  for (int j = 1; j < k; j++) {
    if (q == 0.0) q = 1e-300;
    q = a[j] - x - b1[j] * b1[j] / q;
    if (q < 0) cnt++;
  }
  return cnt;
}

static __device__ void warp_tri_lowest(const double* A, const double* Bt, int k, double btail, double* theta_out,
                                double* s, double* resid) {
  const int lane = threadIdx.x & 31;
  double lo = A[0], hi = A[0];
  for (int j = 0; j < k; j++) {  // Gershgorin bounds (every lane, same values)
    double r = (j > 0 ? fabs(Bt[j]) : 0.0) + (j < k - 1 ? fabs(Bt[j + 1]) : 0.0);
    lo = fmin(lo, A[j] - r);
    hi = fmax(hi, A[j] + r);
  }
  for (int round = 0; round < 100; round++) {
    const double x = lo + (hi - lo) * (double)(lane + 1) / 33.0;
    const int c = (x > lo && x < hi) ? sturm_count_tri(A, Bt, k, x) : (x >= hi ? 1 : 0);
    const unsigned ball = __ballot_sync(0xffffffffu, c >= 1);
    const int f = ball ? (__ffs(ball) - 1) : 32;  // first point above the lowest eigenvalue
    double nlo = (f == 0) ? lo : lo + (hi - lo) * (double)f / 33.0;
    double nhi = (f == 32) ? hi : lo + (hi - lo) * (double)(f + 1) / 33.0;
    if (nlo < lo) nlo = lo;
    if (nhi > hi) nhi = hi;
    const bool stop = (nhi - nlo <= 2.220446049250313e-16 * fmax(fabs(nlo), fabs(nhi))) || !(nlo < nhi) ||
                      (nlo == lo && nhi == hi);
    lo = nlo;
    hi = nhi;
    if (stop) break;
  }
  if (lane != 0) return;
  for (int it = 0; it < 200; it++) {
    const double mid = 0.5 * (lo + hi);
    if (mid <= lo || mid >= hi) break;
    if (sturm_count_tri(A, Bt, k, mid) >= 1) hi = mid; else lo = mid;
  }
  const double th = 0.5 * (lo + hi);
  theta_out[0] = th;
  double* y = s;
  for (int j = 0; j < k; j++) y[j] = 1.0;
  if (k == 1) {
    resid[0] = fabs(btail);
    return;
  }
  double* dl = s + k;
  double* dd = s + 2 * k;
  double* du = s + 3 * k;
  double* du2 = s + 4 * k;
  for (int it = 0; it < 3; it++) {
    for (int j = 0; j < k; j++) dd[j] = A[j] - th;
    for (int j = 0; j < k - 1; j++) { dl[j] = Bt[j + 1]; du[j] = Bt[j + 1]; du2[j] = 0.0; }
    unsigned long long piv[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int j = 0; j < k - 1; j++) {
      if (fabs(dd[j]) >= fabs(dl[j])) {
        if (dd[j] == 0.0) dd[j] = 1e-300;
        const double f = dl[j] / dd[j];
        dl[j] = f;
        dd[j + 1] -= f * du[j];
      } else {
        const double f = dd[j] / dl[j];
        dd[j] = dl[j];
        dl[j] = f;
        const double t = du[j];
        du[j] = dd[j + 1];
        dd[j + 1] = t - f * dd[j + 1];
        if (j < k - 2) { du2[j] = du[j + 1]; du[j + 1] = -f * du[j + 1]; }
        piv[j >> 6] |= 1ull << (j & 63);
      }
    }
    if (dd[k - 1] == 0.0) dd[k - 1] = 1e-300;
    for (int j = 0; j < k - 1; j++) {
      if (!((piv[j >> 6] >> (j & 63)) & 1ull)) y[j + 1] -= dl[j] * y[j];
      else { const double t = y[j]; y[j] = y[j + 1]; y[j + 1] = t - dl[j] * y[j]; }
    }
    y[k - 1] /= dd[k - 1];
    y[k - 2] = (y[k - 2] - du[k - 2] * y[k - 1]) / dd[k - 2];
    for (int j = k - 3; j >= 0; j--) y[j] = (y[j] - du[j] * y[j + 1] - du2[j] * y[j + 2]) / dd[j];
    double nr = 0.0;
    for (int j = 0; j < k; j++) nr += y[j] * y[j];
    nr = sqrt(nr);
    for (int j = 0; j < k; j++) y[j] /= nr;
  }
  if (y[0] < 0) for (int j = 0; j < k; j++) y[j] = -y[j];
  resid[0] = fabs(btail * y[k - 1]);
}

}  // namespace vca
