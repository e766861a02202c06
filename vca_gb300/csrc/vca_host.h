// vca_host.h -- host-only logic of the solve that needs no GPU: the state
// lists replayed on the sector energies, the k-point pairing of the Omega
// k-sum and the contour rule of the finite-T integral.  The C-ABI exports
// them (vca_state_list_t0/_finite_t, vca_pair_kpoints, vca_contour_rule) so
// that they run without a device.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/vca_gpu.h"

namespace vca {

struct ListEntry {
  double e;
  int sector;
};

// finite T, one state per sector (VCA_DIAG.f90:78-256, vca_post_diag :357-451)
void replay_finite_t(const std::vector<double>& E, const vca_config& c, int& nstates_total,
                     std::vector<ListEntry>& lst, double& zeta, double& emin);
// T=0 (VCA_DIAG.f90:224-236)
void replay_t0(const std::vector<double>& E, double thr, std::vector<ListEntry>& lst);
// conjugate k-point pairs H_k' = conj(H_k) of the Omega k-sum
void pair_kpoints_host(const double* Hk, int64_t Nk, size_t nel, std::vector<int64_t>& reps,
                       std::vector<double>& wts);
// Gauss-Legendre on (0,1) and the contour rule of the finite-T integral
void gauss_legendre01_host(int n, std::vector<double>& x, std::vector<double>& w);
void contour_nodes_host(double R, double beta, double mu, int ngl, std::vector<double>& th,
                        std::vector<double>& wt);

// Symmetric tridiagonal eigenproblem (diagonal d[0..n-1], off-diagonal
// e[i] coupling i and i+1, i < n-1) by implicit QL iterations with
// Wilkinson shifts: eigenvalues ascending in w, eigenvectors as columns of
// Z (column-major n x n).  Returns false if an eigenvalue needed more than
// 60 iterations.
bool tridiag_eig(int n, const double* d, const double* e, std::vector<double>& w, std::vector<double>& Z);
// Hermitian dense eigenproblem (A row-major n x n, complex interleaved) by
// cyclic complex Jacobi rotations: eigenvalues ascending in w, eigenvectors
// as columns of Z (column-major n x n, complex interleaved).  Returns false
// if 100 sweeps did not bring the off-diagonal norm to 1e-15 of the total.
bool herm_eig(int n, const double* A, std::vector<double>& w, std::vector<double>& Z);

// sets the text vca_gpu_last_error returns and hands the code back
int set_error(int code, const std::string& msg);

}  // namespace vca
