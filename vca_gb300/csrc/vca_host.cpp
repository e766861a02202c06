// vca_host.cpp -- host-only logic of the solve (see vca_host.h), with the
// C-ABI entry points that run it and the restart-file codec without a GPU.
#include "vca_host.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <complex>
#include <cstring>

#include "vca_gfmatrix.h"

#define HFAIL(code, msg) return vca::set_error((code), (msg))

namespace vca {

// The finite-T state list from every sector's lowest energy E[isector-1]
// (one state per sector): the annealing sweeps of VCA_DIAG.f90:78-256 replayed
// on the host -- each sweep rebuilds the list capped at LANC_NSTATES_TOTAL
// (es_add_state_c with size, VCA_EIGENSPACE.f90:136-159; insertion before the
// first entry with e <= its energy, es_insert_state_c :167-216; the last entry
// popped, es_pop_state :230-312), tests exp(-beta(emax-emin)) < CUTOFF, then
// vca_post_diag (:357-451) sums zeta over the whole list and either grows the
// cap by LANC_NSTATES_STEP or trims the states beyond the cut-off and resets
// the cap to max(size, step) + step.  Every sweep finds the same energies, so
// the search runs once.  Host only.
void replay_finite_t(const std::vector<double>& E, const vca_config& c, int& nstates_total,
                     std::vector<ListEntry>& lst, double& zeta, double& emin) {
  const int nsec = (int)E.size();
  double lo = DBL_MAX, hi = -DBL_MAX;
  auto put = [&](int isector) {
    const double e = E[isector - 1];
    auto at = std::find_if(lst.begin(), lst.end(), [&](const ListEntry& x) { return e <= x.e; });
    lst.insert(at, ListEntry{e, isector});
    if (e > hi) hi = e;
    if (e < lo) lo = e;
  };
  auto drop = [&]() {
    lst.pop_back();
    if (!lst.empty()) { hi = lst.back().e; lo = lst.front().e; }
  };
  const double beta = c.beta;
  zeta = 0.0;
  lst.clear();
  bool done = false;
  for (int sweep = 0; !done && sweep < c.lanc_niter_spectrum; sweep++) {
    lst.clear();
    lo = DBL_MAX;
    hi = -DBL_MAX;
    for (int isector = 1; isector <= nsec; isector++) {
      if ((int)lst.size() < nstates_total) put(isector);
      else if (E[isector - 1] < lst.back().e) { drop(); put(isector); }
    }
    const double spread = std::exp(-beta * (hi - lo));
    done = spread < c.cutoff;
    zeta = 0.0;
    for (const ListEntry& x : lst) zeta += std::exp(-beta * (x.e - lo));
    if (spread > c.cutoff) {
      nstates_total += c.lanc_nstates_step;
    } else {
      while (std::exp(-beta * (lst.back().e - lo)) <= c.cutoff) drop();
      nstates_total = std::max((int)lst.size(), c.lanc_nstates_step) + c.lanc_nstates_step;
    }
  }
  emin = lo;
}

// The T=0 list from every sector's lowest energy: VCA_DIAG.f90:224-236 in
// sector order (a new lowest energy below oldzero - 10*GS_THRESHOLD empties
// the list, one within GS_THRESHOLD of oldzero joins it), each state
// inserted before the first entry with e <= its energy.  Host only.
void replay_t0(const std::vector<double>& E, double thr, std::vector<ListEntry>& lst) {
  double oz = 1000.0;
  lst.clear();
  for (int isector = 1; isector <= (int)E.size(); isector++) {
    const double e = E[isector - 1];
    if (e < oz - 10.0 * thr) {
      oz = e;
      lst.assign(1, ListEntry{e, isector});
    } else if (std::fabs(e - oz) <= thr) {
      oz = std::min(oz, e);
      auto at = std::find_if(lst.begin(), lst.end(), [&](const ListEntry& x) { return e <= x.e; });
      lst.insert(at, ListEntry{e, isector});
    }
  }
}

// k-points paired by H_k' = conj(H_k), entry-wise to 1e-13 (1 + max|H|):
// each pair is summed once with weight 2 (the Omega integrand is equal at
// the two points of a pair for the models that take this path), an unpaired
// point with weight 1.  Candidates are found through a random real linear
// signature of H_k and of conj(H_k), sorted; every match is verified entry by
// entry.  reps in ascending order of k.  Host only.
void pair_kpoints_host(const double* Hk, int64_t Nk, size_t nel, std::vector<int64_t>& reps,
                       std::vector<double>& wts) {
  std::vector<double> cr(nel), ci(nel);
  uint64_t st = 0x9E3779B97F4A7C15ull;
  auto rnd = [&]() {
    st ^= st << 13;
    st ^= st >> 7;
    st ^= st << 17;
    return 0.5 + (double)(st >> 11) * (1.0 / 9007199254740992.0);
  };
  double hmax = 0.0, wsum = 0.0;
  for (size_t x = 0; x < nel; x++) {
    cr[x] = rnd();
    ci[x] = rnd();
    wsum += cr[x] + ci[x];
  }
  for (size_t i = 0; i < 2 * nel * (size_t)Nk; i++) hmax = std::max(hmax, std::fabs(Hk[i]));
  const double tol = 1e-13 * (1.0 + hmax);
  std::vector<std::pair<double, int64_t>> sig(Nk);
  std::vector<double> csig(Nk);
  for (int64_t k = 0; k < Nk; k++) {
    double a = 0.0, b = 0.0;
    const double* h = Hk + 2 * nel * k;
    for (size_t x = 0; x < nel; x++) {
      a += cr[x] * h[2 * x] + ci[x] * h[2 * x + 1];
      b += cr[x] * h[2 * x] - ci[x] * h[2 * x + 1];
    }
    sig[k] = {a, k};
    csig[k] = b;
  }
  std::sort(sig.begin(), sig.end());
  reps.clear();
  wts.clear();
  if (Nk == 0) return;
  const double stol = tol * wsum * 2.0 + 1e-12 * (std::fabs(sig.front().first) + std::fabs(sig.back().first));
  std::vector<char> used(Nk, 0);
  auto conj_of = [&](int64_t j, int64_t k) {
    const double* a = Hk + 2 * nel * j;
    const double* b = Hk + 2 * nel * k;
    for (size_t x = 0; x < nel; x++)
      if (std::fabs(a[2 * x] - b[2 * x]) > tol || std::fabs(a[2 * x + 1] + b[2 * x + 1]) > tol) return false;
    return true;
  };
  for (int64_t k = 0; k < Nk; k++) {
    if (used[k]) continue;
    used[k] = 1;
    int64_t partner = -1;
    auto lo = std::lower_bound(sig.begin(), sig.end(), std::make_pair(csig[k] - stol, (int64_t)-1));
    for (auto it = lo; it != sig.end() && it->first <= csig[k] + stol; ++it)
      if (!used[it->second] && conj_of(it->second, k)) { partner = it->second; break; }
    reps.push_back(k);
    if (partner >= 0) {
      used[partner] = 1;
      wts.push_back(2.0);
    } else {
      wts.push_back(1.0);
    }
  }
}

// Gauss-Legendre nodes/weights on (0,1), host (Newton on the three-term
// recurrence of P_n)
void gauss_legendre01_host(int n, std::vector<double>& x, std::vector<double>& w) {
  x.assign(n, 0.0);
  w.assign(n, 0.0);
  for (int i = 0; i < (n + 1) / 2; i++) {
    double z = std::cos(M_PI * (i + 0.75) / (n + 0.5)), dp = 1.0;
    for (int it = 0; it < 100; it++) {
      double p0 = 1.0, p1 = z;  // P_0, P_1
      for (int j = 2; j <= n; j++) {
        const double p2 = ((2.0 * j - 1.0) * z * p1 - (j - 1.0) * p0) / j;
        p0 = p1;
        p1 = p2;
      }
      if (n == 1) { p1 = z; p0 = 1.0; }
      dp = n * (z * p1 - p0) / (z * z - 1.0);
      const double dz = p1 / dp;
      z -= dz;
      if (std::fabs(dz) < 1e-16) break;
    }
    double p0 = 1.0, p1 = z;
    for (int j = 2; j <= n; j++) {
      const double p2 = ((2.0 * j - 1.0) * z * p1 - (j - 1.0) * p0) / j;
      p0 = p1;
      p1 = p2;
    }
    dp = n * (z * p1 - p0) / (z * z - 1.0);
    const double wt = 1.0 / ((1.0 - z * z) * dp * dp);  // 2/((1-z^2)P'^2), halved for (0,1)
    x[i] = 0.5 * (1.0 - z);
    x[n - 1 - i] = 0.5 * (1.0 + z);
    w[i] = wt;
    w[n - 1 - i] = wt;
  }
}

// Angles and weights of the fixed rule replacing quad(integral_contour, 0,
// pi, key=6) (VCA_OMEGA.f90:172).  The sharp structure of the integrand
// comes from the poles xmu + i(2n+1)pi/beta of fermi(w - xmu) next to the
// arc |w| = R; the rule is composite Gauss-Legendre (contour_nodes per
// panel) on panels growing geometrically (factor 2, at most pi/16) away from
// the angle of the pole nearest to the arc, the first panel's width that
// pole's distance from the arc over R.
void contour_nodes_host(double R, double beta, double mu, int ngl, std::vector<double>& th,
                        std::vector<double>& wt) {
  const double ymid = std::sqrt(std::max(R * R - mu * mu, 0.0));
  const double n0 = std::floor((ymid * beta / M_PI - 1.0) / 2.0);
  double dist = INFINITY, center = 0.5 * M_PI;
  for (int d = -1; d <= 2; d++) {
    const double nn = n0 + d;
    if (nn < 0.0) continue;
    const double y = (2.0 * nn + 1.0) * M_PI / beta;
    const double dd = std::fabs(std::hypot(mu, y) - R);
    if (dd < dist) { dist = dd; center = std::atan2(y, mu); }
  }
  const double h0 = std::max(dist / R, 1e-15), hmax = M_PI / 16.0;
  std::vector<double> edge{center};
  for (double b = center, h = h0; b > 0.0; h = std::min(2.0 * h, hmax)) edge.push_back(b = std::max(b - h, 0.0));
  for (double b = center, h = h0; b < M_PI; h = std::min(2.0 * h, hmax)) edge.push_back(b = std::min(b + h, M_PI));
  std::sort(edge.begin(), edge.end());
  std::vector<double> x, w;
  gauss_legendre01_host(ngl, x, w);
  th.clear();
  wt.clear();
  for (size_t p = 0; p + 1 < edge.size(); p++) {
    const double a = edge[p], h = edge[p + 1] - edge[p];
    for (int i = 0; i < ngl; i++) {
      th.push_back(a + h * x[i]);
      wt.push_back(h * w[i]);
    }
  }
}

// Implicit QL with Wilkinson shifts on a symmetric tridiagonal matrix.  Each
// sweep deflates at the first negligible off-diagonal element below l, then
// chases the bulge from m back up to l with Givens rotations, accumulating
// them in the columns of Z.
bool tridiag_eig(int n, const double* d_in, const double* e_in, std::vector<double>& w, std::vector<double>& Z) {
  std::vector<double> d(d_in, d_in + n), e(n, 0.0);
  for (int i = 0; i + 1 < n; i++) e[i] = e_in[i];
  Z.assign((size_t)n * n, 0.0);
  for (int i = 0; i < n; i++) Z[i + (size_t)i * n] = 1.0;
  for (int l = 0; l < n; l++) {
    for (int iter = 0;; iter++) {
      int m = l;
      for (; m + 1 < n; m++) {
        const double scale = std::fabs(d[m]) + std::fabs(d[m + 1]);
        if (std::fabs(e[m]) <= DBL_EPSILON * scale) break;
      }
      if (m == l) break;
      if (iter == 60) return false;
      // shift: the eigenvalue of the leading 2x2 block nearer d[l]
      double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
      double r = std::hypot(g, 1.0);
      g = d[m] - d[l] + e[l] / (g + (g >= 0.0 ? r : -r));
      double s = 1.0, c = 1.0, p = 0.0;
      int i = m - 1;
      bool early = false;
      for (; i >= l; i--) {
        const double f = s * e[i], b = c * e[i];
        r = std::hypot(f, g);
        e[i + 1] = r;
        if (r == 0.0) {  // the bulge vanished: split here
          d[i + 1] -= p;
          e[m] = 0.0;
          early = true;
          break;
        }
        s = f / r;
        c = g / r;
        g = d[i + 1] - p;
        r = (d[i] - g) * s + 2.0 * c * b;
        p = s * r;
        d[i + 1] = g + p;
        g = c * r - b;
        double* zi = Z.data() + (size_t)i * n;
        double* zj = Z.data() + (size_t)(i + 1) * n;
        for (int k = 0; k < n; k++) {
          const double t = zj[k];
          zj[k] = s * zi[k] + c * t;
          zi[k] = c * zi[k] - s * t;
        }
      }
      if (early) continue;
      d[l] -= p;
      e[l] = g;
      e[m] = 0.0;
    }
  }
  std::vector<int> ord(n);
  for (int i = 0; i < n; i++) ord[i] = i;
  std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return d[a] < d[b]; });
  w.resize(n);
  std::vector<double> Zs((size_t)n * n);
  for (int j = 0; j < n; j++) {
    w[j] = d[ord[j]];
    std::memcpy(Zs.data() + (size_t)j * n, Z.data() + (size_t)ord[j] * n, sizeof(double) * n);
  }
  Z.swap(Zs);
  return true;
}

// Cyclic Jacobi for a Hermitian matrix: for each pair (p, q) the phase of
// a_pq is moved into column q (making a_pq real and positive), then a real
// rotation zeroes it; the same unitary is accumulated in Z.
bool herm_eig(int n, const double* A_in, std::vector<double>& w, std::vector<double>& Z) {
  typedef std::complex<double> cdd;
  std::vector<cdd> a((size_t)n * n), z((size_t)n * n, 0.0);
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) a[i + (size_t)j * n] = cdd(A_in[2 * ((size_t)i * n + j)], A_in[2 * ((size_t)i * n + j) + 1]);
  for (int i = 0; i < n; i++) z[i + (size_t)i * n] = 1.0;
  auto A = [&](int i, int j) -> cdd& { return a[i + (size_t)j * n]; };
  bool ok = false;
  for (int sweep = 0; sweep < 100; sweep++) {
    double off = 0.0, tot = 0.0;
    for (int j = 0; j < n; j++)
      for (int i = 0; i < n; i++) {
        const double v = std::norm(A(i, j));
        tot += v;
        if (i != j) off += v;
      }
    if (off <= 1e-30 * tot || off == 0.0) { ok = true; break; }
    for (int p = 0; p < n; p++)
      for (int q = p + 1; q < n; q++) {
        const double r = std::abs(A(p, q));
        if (r == 0.0) continue;
        const cdd ph = std::conj(A(p, q)) / r;  // column q times ph, row q times conj(ph)
        for (int k = 0; k < n; k++) A(k, q) *= ph;
        for (int k = 0; k < n; k++) A(q, k) *= std::conj(ph);
        for (int k = 0; k < n; k++) z[k + (size_t)q * n] *= ph;
        const double app = A(p, p).real(), aqq = A(q, q).real(), apq = A(p, q).real();
        const double th = 0.5 * (aqq - app) / apq;
        const double t = (th >= 0 ? 1.0 : -1.0) / (std::fabs(th) + std::sqrt(th * th + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), sn = t * c;
        for (int k = 0; k < n; k++) {
          const cdd akp = A(k, p), akq = A(k, q);
          A(k, p) = c * akp - sn * akq;
          A(k, q) = sn * akp + c * akq;
        }
        for (int k = 0; k < n; k++) {
          const cdd apk = A(p, k), aqk = A(q, k);
          A(p, k) = c * apk - sn * aqk;
          A(q, k) = sn * apk + c * aqk;
        }
        A(p, q) = A(q, p) = 0.0;
        for (int k = 0; k < n; k++) {
          const cdd zkp = z[k + (size_t)p * n], zkq = z[k + (size_t)q * n];
          z[k + (size_t)p * n] = c * zkp - sn * zkq;
          z[k + (size_t)q * n] = sn * zkp + c * zkq;
        }
      }
  }
  std::vector<int> ord(n);
  for (int i = 0; i < n; i++) ord[i] = i;
  std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) { return A(x, x).real() < A(y, y).real(); });
  w.resize(n);
  Z.assign(2 * (size_t)n * n, 0.0);
  for (int j = 0; j < n; j++) {
    w[j] = A(ord[j], ord[j]).real();
    for (int k = 0; k < n; k++) {
      Z[2 * (k + (size_t)j * n)] = z[k + (size_t)ord[j] * n].real();
      Z[2 * (k + (size_t)j * n) + 1] = z[k + (size_t)ord[j] * n].imag();
    }
  }
  return ok;
}

}  // namespace vca

using namespace vca;

int vca_tridiag_eig(int32_t n, const double* d, const double* e, double* w, double* Z) {
  if (n < 1 || !d || !w || (n > 1 && !e)) HFAIL(VCA_ERR_ARG, "bad arguments");
  std::vector<double> ww, zz;
  if (!tridiag_eig(n, d, e, ww, zz)) HFAIL(VCA_ERR_NUMERIC, "tridiagonal QL did not converge");
  std::memcpy(w, ww.data(), sizeof(double) * n);
  if (Z) std::memcpy(Z, zz.data(), sizeof(double) * zz.size());
  return VCA_OK;
}

int vca_herm_eig(int32_t n, const double* A, double* w, double* Z) {
  if (n < 1 || !A || !w) HFAIL(VCA_ERR_ARG, "bad arguments");
  std::vector<double> ww, zz;
  if (!herm_eig(n, A, ww, zz)) HFAIL(VCA_ERR_NUMERIC, "Jacobi rotations did not converge");
  std::memcpy(w, ww.data(), sizeof(double) * n);
  if (Z) std::memcpy(Z, zz.data(), sizeof(double) * zz.size());
  return VCA_OK;
}

extern "C" {

int vca_pair_kpoints(const double* Hk, int64_t Nk, int64_t nel, int64_t* reps, double* weights, int64_t cap,
                     int64_t* nrep) {
  if (!Hk || Nk < 0 || nel < 1 || !nrep || cap < 0 || (cap > 0 && (!reps || !weights)))
    HFAIL(VCA_ERR_ARG, "bad arguments");
  std::vector<int64_t> r;
  std::vector<double> w;
  pair_kpoints_host(Hk, Nk, (size_t)nel, r, w);
  *nrep = (int64_t)r.size();
  for (int64_t i = 0; i < (int64_t)r.size() && i < cap; i++) {
    reps[i] = r[i];
    weights[i] = w[i];
  }
  return VCA_OK;
}

int vca_contour_rule(double R, double beta, double mu, int32_t ngl, double* theta, double* weights, int32_t cap,
                     int32_t* n) {
  if (!n || ngl < 2 || !(R > 0.0) || !(beta > 0.0) || cap < 0 || (cap > 0 && (!theta || !weights)))
    HFAIL(VCA_ERR_ARG, "bad arguments");
  std::vector<double> th, wt;
  contour_nodes_host(R, beta, mu, ngl, th, wt);
  *n = (int32_t)th.size();
  for (int i = 0; i < (int)th.size() && i < cap; i++) {
    theta[i] = th[i];
    weights[i] = wt[i];
  }
  return VCA_OK;
}

int vca_state_list_t0(const double* E, int32_t nsectors, double gs_threshold, int32_t* sectors, double* energies,
                      int32_t cap, int32_t* n) {
  if (!E || nsectors < 0 || !n || cap < 0 || (cap > 0 && !sectors)) HFAIL(VCA_ERR_ARG, "bad arguments");
  std::vector<ListEntry> lst;
  replay_t0(std::vector<double>(E, E + nsectors), gs_threshold, lst);
  *n = (int32_t)lst.size();
  for (int i = 0; i < (int)lst.size() && i < cap; i++) {
    sectors[i] = lst[i].sector;
    if (energies) energies[i] = lst[i].e;
  }
  return VCA_OK;
}

int vca_state_list_finite_t(const double* E, int32_t nsectors, const vca_config* cfg, int32_t nstates_total,
                            int32_t* sectors, int32_t cap, int32_t* n, double* zeta, double* emin,
                            int32_t* nstates_total_out) {
  if (!E || nsectors < 0 || !cfg || !n || cap < 0 || (cap > 0 && !sectors) || nstates_total < 1)
    HFAIL(VCA_ERR_ARG, "bad arguments");
  if (!(cfg->cutoff > 0.0 && cfg->cutoff < 1.0) || !(cfg->beta > 0.0) || cfg->lanc_niter_spectrum < 1)
    HFAIL(VCA_ERR_CONFIG, "CUTOFF in (0,1), BETA > 0 and LANC_NITER_SPECTRUM >= 1 are required");
  std::vector<ListEntry> lst;
  int nt = nstates_total;
  double z = 0.0, lo = 0.0;
  replay_finite_t(std::vector<double>(E, E + nsectors), *cfg, nt, lst, z, lo);
  *n = (int32_t)lst.size();
  for (int i = 0; i < (int)lst.size() && i < cap; i++) sectors[i] = lst[i].sector;
  if (zeta) *zeta = z;
  if (emin) *emin = lo;
  if (nstates_total_out) *nstates_total_out = nt;
  return VCA_OK;
}

int vca_gfm_write(const char* path, int32_t formatted, int64_t nelem, const int32_t* nstates, const int32_t* nchan,
                  const int32_t* nexc, const double* poles, const double* weights) {
  if (!path || nelem < 0 || (nelem > 0 && !nstates)) HFAIL(VCA_ERR_ARG, "bad arguments");
  GfmTable t;
  t.nstates.assign(nstates, nstates + nelem);
  int64_t ns = 0, nc = 0, ne = 0;
  for (int32_t v : t.nstates) {
    if (v < 0) HFAIL(VCA_ERR_ARG, "negative state count");
    ns += v;
  }
  if (ns > 0 && !nchan) HFAIL(VCA_ERR_ARG, "nchan is NULL");
  t.nchan.assign(nchan, nchan + ns);
  for (int32_t v : t.nchan) {
    if (v < 0) HFAIL(VCA_ERR_ARG, "negative channel count");
    nc += v;
  }
  if (nc > 0 && !nexc) HFAIL(VCA_ERR_ARG, "nexc is NULL");
  t.nexc.assign(nexc, nexc + nc);
  for (int32_t v : t.nexc) {
    if (v < 0) HFAIL(VCA_ERR_ARG, "negative excitation count");
    ne += v;
  }
  if (ne > 0 && (!poles || !weights)) HFAIL(VCA_ERR_ARG, "poles or weights is NULL");
  t.poles.assign(poles, poles + 2 * ne);
  t.weights.assign(weights, weights + 2 * ne);
  std::string err;
  if (gfm_write(path, formatted != 0, t, err)) HFAIL(VCA_ERR_IO, err);
  return VCA_OK;
}

int vca_gfm_read(const char* path, int32_t formatted, int64_t nelem, int64_t* sizes, int32_t* nstates,
                 int32_t* nchan, int32_t* nexc, double* poles, double* weights) {
  if (!path || !sizes || nelem < 0) HFAIL(VCA_ERR_ARG, "bad arguments");
  GfmTable t;
  std::string err;
  if (gfm_read(path, formatted != 0, nelem, t, err)) HFAIL(VCA_ERR_IO, err);
  const int64_t ns = (int64_t)t.nchan.size(), nc = (int64_t)t.nexc.size(), ne = (int64_t)t.poles.size() / 2;
  if (nstates) {
    if (sizes[0] < ns || sizes[1] < nc || sizes[2] < ne) HFAIL(VCA_ERR_ARG, "arrays smaller than the file's table");
    if ((ns && !nchan) || (nc && !nexc) || (ne && (!poles || !weights))) HFAIL(VCA_ERR_ARG, "NULL array");
    std::copy(t.nstates.begin(), t.nstates.end(), nstates);
    std::copy(t.nchan.begin(), t.nchan.end(), nchan);
    std::copy(t.nexc.begin(), t.nexc.end(), nexc);
    std::copy(t.poles.begin(), t.poles.end(), poles);
    std::copy(t.weights.begin(), t.weights.end(), weights);
  }
  sizes[0] = ns;
  sizes[1] = nc;
  sizes[2] = ne;
  return VCA_OK;
}

}  // extern "C"
