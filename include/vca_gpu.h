/*
 * vca_gpu.h -- C-ABI of the GB300 cluster exact-diagonalization path of VCA.
 *
 * One process, one GPU, one global solver context (not thread-safe, not
 * reentrant), one CUDA stream, synchronous return.  Every array argument is a
 * HOST pointer in Fortran column-major order and is neither retained nor
 * modified after return unless it is an output.  complex(8) arrays are passed
 * as `double*` pointing at interleaved (re, im) pairs: the memory layout of a
 * Fortran complex(c_double_complex) array and of a C99 double _Complex array.
 *
 * Reference interface replaced (paths inside QcmPlab/VCA):
 *   vca_init_solver  VCA_MAIN.f90:51-76   (MPI form :79-115)
 *   vca_solve        VCA_MAIN.f90:124-215 (MPI form :220-323)
 *   vca_get_sft_potential   VCA_IO/get_sft_potential.f90:1-4
 *   vca_gf_cluster   VCA_IO/gf_cluster.f90:1-88 (generic at VCA_IO.f90:38-62)
 *   spHtimesV_p / cc_sparse_HxV  VCA_VARS_GLOBAL.f90:83-89,137
 * Configuration mirrors the module variables of VCA_INPUT_VARS.f90:14-81 with
 * the defaults of VCA_INPUT_VARS.f90:112-172 (vca_config_defaults).
 *
 * Status codes: 0 = OK, negative = error (vca_gpu_last_error gives the text).
 */
#ifndef VCA_GPU_H
#define VCA_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VCA_OK 0
#define VCA_ERR_CONFIG (-1)      /* invalid or unsupported input variable     */
#define VCA_ERR_SHAPE (-2)       /* array extents inconsistent with config    */
#define VCA_ERR_STATE (-3)       /* call order: init missing, no solve yet    */
#define VCA_ERR_CUDA (-4)        /* CUDA runtime error                        */
#define VCA_ERR_TIMEOUT (-5)     /* a bounded device wait ran out             */
#define VCA_ERR_UNSUPPORTED (-6) /* feature outside the implemented path      */
#define VCA_ERR_NUMERIC (-7)     /* NaN/Inf input, zero-norm vector, breakdown */
#define VCA_ERR_ALLOC (-8)       /* device memory exhausted                   */
#define VCA_ERR_ARG (-9)         /* null pointer or out-of-range index        */
#define VCA_ERR_IO (-10)         /* file open, read, write or layout error    */

#define VCA_LANC_ARPACK 0
#define VCA_LANC_LANCZOS 1

/* Vector arithmetic of the Lanczos kernels.  FX keeps vectors as exact
 * 64-bit fixed point with integer hop sums (real Hamiltonians whose hopping
 * amplitudes take at most 4 magnitudes); FP64 is the general path.  AUTO
 * picks FX when it applies. */
#define VCA_ARITH_AUTO 0
#define VCA_ARITH_FP64 1
#define VCA_ARITH_FX 2

/*
 * Input variables.  Field names, meanings and defaults follow
 * VCA_INPUT_VARS.f90:14-81 / :112-172.  Integers are 32-bit, logicals are
 * 0/1.  Fields from `omega_nodes` to `hxv_variant`, and `contour_nodes`, have
 * no counterpart in the reference: they fix what the reference leaves to
 * SciFortran defaults (Lanczos stopping rule, start vector) or replaces (the
 * adaptive QUADPACK integrals become fixed Gauss-Legendre rules).
 */
typedef struct vca_config {
  int32_t Norb;      /* NORB       orbitals per cluster site (<= 5)          */
  int32_t Nspin;     /* NSPIN      1 or 2                                   */
  int32_t Nlat;      /* NLAT       cluster sites                            */
  int32_t Nlat_bath; /* NLAT_BATH  bath "site" levels                       */
  int32_t Norb_bath; /* NORB_BATH  bath "orb" levels                        */
  int32_t no_sector_screen; /* no counterpart: 1 makes the batched form of      */
                           /* vca_gpu_solve_batch search every (point, sector); */
                           /* 0 (default) skips sectors whose one-body lower    */
                           /* bound proves them above the T=0 window            */
  double Uloc[5];    /* ULOC       on-site interaction per orbital          */
  double Ust;        /* UST        inter-orbital opposite-spin interaction  */
  double Jh;         /* JH         Hund coupling (Ust-Jh parallel spins)    */
  double Jx;         /* JX         parsed, not part of H (as reference)     */
  double Jp;         /* JP         parsed, not part of H (as reference)     */
  double xmu;        /* XMU        chemical potential                       */
  double beta;       /* BETA       inverse temperature (IR cut-off at T=0)  */
  double eps;        /* EPS        real-axis broadening                     */
  double wini;       /* WINI       real-axis grid start                     */
  double wfin;       /* WFIN       real-axis grid end                       */
  int32_t hfmode;    /* HFMODE     U(n-1/2)(n-1/2) form                     */
  int32_t hfshift;   /* HFSHIFT    bath half-filling shift                  */
  int32_t Lmats;     /* LMATS      Matsubara frequencies                    */
  int32_t Lreal;     /* LREAL      real-axis frequencies                    */
  int32_t lanc_method;         /* LANC_METHOD  VCA_LANC_ARPACK | VCA_LANC_LANCZOS */
  int32_t lanc_niter;          /* LANC_NITER                              */
  int32_t lanc_ngfiter;        /* LANC_NGFITER  GF chain length           */
  int32_t lanc_dim_threshold;  /* LANC_DIM_THRESHOLD  dense path below    */
  int32_t lanc_nstates_sector; /* LANC_NSTATES_SECTOR                     */
  int32_t lanc_nstates_total;  /* LANC_NSTATES_TOTAL  1 => T=0            */
  double lanc_tolerance;       /* LANC_TOLERANCE                          */
  double gs_threshold;         /* GS_THRESHOLD  GS degeneracy window      */
  int32_t vca_gf_symmetric;    /* VCA_GF_SYMMETRIC  2-channel off-diag GF */
  int32_t vca_sparse_H;        /* VCA_SPARSE_H  stored semantics (always) */
  int32_t vca_twin;            /* VCA_TWIN                                */
  int32_t vca_sectors;         /* VCA_SECTORS   accepted; every sector is */
  int32_t vca_sectors_shift;   /* VCA_SECTORS_SHIFT  scanned (a superset)  */
  int32_t verbose;             /* VERBOSE                                 */
  /* ---- no counterpart in the reference ---------------------------------- */
  int32_t omega_nodes;     /* Gauss-Legendre nodes on [0,inf) for Omega     */
  int32_t gs_check_every;  /* Lanczos GS convergence test interval          */
  double omega_scale;      /* map w = omega_scale * s/(1-s), s in (0,1)     */
  double gs_residual_tol;  /* GS stop: |beta_{k+1} s_k| <= tol*max(1,|E|)   */
  double gf_beta_tol;      /* GF chain stop: beta_{k+1} < tol (exhausted)   */
                           /* (the ground-state search uses gs_beta_tol)     */
  uint64_t start_seed;     /* seed of the deterministic Lanczos start vector */
  int32_t arith;           /* VCA_ARITH_AUTO | VCA_ARITH_FP64 | VCA_ARITH_FX   */
  int32_t hxv_variant;     /* FX column H x v of the hxv entry points: 0 auto, */
                           /* 1 warp form only, 2 rows in hop-count order     */
  /* ---- finite temperature (LANC_NSTATES_TOTAL > 1) ---------------------- */
  int32_t lanc_nstates_step;   /* LANC_NSTATES_STEP   list growth per sweep   */
  int32_t lanc_niter_spectrum; /* LANC_NITER_SPECTRUM annealing sweeps        */
  int32_t contour_nodes;   /* Gauss-Legendre nodes per panel of the contour  */
                           /* rule replacing quad(integral_contour, 0, pi)   */
  int32_t sector_at_a_time; /* 1: the ground-state search diagonalises one   */
                           /* sector after the other, as the reference's loop */
                           /* (VCA_DIAG.f90:83-249); 0 (default): every      */
                           /* sector in one batched search                   */
  double cutoff;           /* CUTOFF     spectrum cut-off exp(-beta dE)      */
  double bandwidth;        /* bandwidth  lattice bandwidth (a module variable */
                           /* the reference's drivers assign, default 0)     */
  double gs_beta_tol;      /* ground-state Lanczos: beta_{k+1} < tol ends it */
  /* ---- output files ----------------------------------------------------- */
  int32_t print_sigma;     /* PRINT_SIGMA  splot files of Sigma after a solve */
  int32_t print_impg;      /* PRINT_IMPG   ... of G'  (VCA_INPUT_VARS.f90:137-139; */
  int32_t print_impg0;     /* PRINT_IMPG0  ... of G0   the reference's default is */
                           /* on, here off: see vca_gpu_print_impSigma)           */
  int32_t batch_loop;      /* 1: vca_gpu_solve_batch solves its points one      */
                           /* after another (the plain path); 0 (default): the  */
                           /* batched form at T=0 (FP64, every point per launch) */
  char file_suffix[64];    /* the reference's file_suffix, NUL-terminated: ends  */
                           /* the stem of every file name (VCA_IO.f90:126-128)   */
} vca_config;

/* Fill *cfg with the reference defaults (VCA_INPUT_VARS.f90:112-172) plus
 * the build-specific defaults above. */
void vca_config_defaults(vca_config* cfg);

/*
 * vca_init_solver replacement (VCA_MAIN.f90:51-76).  Validates the config,
 * builds the sector tables (VCA_SETUP.f90:81-94,259-390), selects the GPU and
 * creates the stream.  bath_h/bath_v are optional (both NULL = no bath, which
 * sets Nlat_bath = Norb_bath = 0 as VCA_MAIN.f90:64-66 does); when given their
 * shapes are (Nlat_bath,Nlat_bath,Nspin,Nspin,Norb_bath,Norb_bath) and
 * (Nlat,Nlat_bath,Nspin,Nspin,Norb,Norb_bath).  A second call re-initialises.
 */
int vca_gpu_init(const vca_config* cfg, const double* bath_h, const double* bath_v);

/*
 * vca_solve replacement (VCA_MAIN.f90:124-215).
 *   Hloc  (Nlat,Nlat,Nspin,Nspin,Norb,Norb)        complex, read-only
 *   Hk    (Nlat,Nlat,Nspin,Nspin,Norb,Norb,Nk)     complex, read-only
 *   bath_h/bath_v as in vca_gpu_init (NULL when the model has no bath)
 *   omega_out  receives the SFT grand potential Omega' - Omega_int (may be NULL)
 * Diagonalises every sector, builds the cluster Green's function chains and
 * integrates the Potthoff functional.  T=0 (LANC_NSTATES_TOTAL = 1):
 * Omega' = E_gs and the integral runs on the imaginary axis.  Finite T: the
 * lowest state of every sector enters an annealed, capped state list
 * (VCA_DIAG.f90:78-256, :395-471), the chains carry Boltzmann weights,
 * Omega' = E_min - T ln sum_i exp(-beta (E_i - E_min)) and the integral is a
 * Matsubara sum plus a contour integral (VCA_OMEGA.f90:153-204).  The list
 * size LANC_NSTATES_TOTAL adapts from solve to solve, as the reference's
 * module variable does; vca_gpu_init resets it.
 */
int vca_gpu_solve(const double* Hloc, const double* Hk, int64_t Nk,
                  const double* bath_h, const double* bath_v, double* omega_out);

/*
 * Batched solve: B variational points in one call.  No counterpart in the
 * reference (it replaces a driver loop of vca_solve calls, e.g.
 * drivers/vca_hm_chain1d.f90:88-111).  Point b uses Hloc + b*stride_hloc
 * complex elements, and bath_h/bath_v likewise (NULL = no bath); Hk is shared
 * by all points.  omega_out[b] receives the SFT potential of point b.
 * At T=0 with B >= 2 (and batch_loop = 0) the points run in the batched
 * form: in FP64, every (point, sector) ground-state search in one multi-task
 * Lanczos, the kept eigenvectors in one second pass, every point's
 * Green's-function chains in memory-bounded groups of (point, chain) tasks,
 * then Omega per point; the points of one call are processed in waves that
 * fit device memory.  Afterwards the context holds the last point's solve
 * (re-run on the plain path; the call fails with VCA_ERR_NUMERIC if its two
 * Omega values differ by more than 1e-10 relative).  Finite T, B = 1 or
 * batch_loop = 1: one point after another through vca_gpu_solve's path.
 */
int vca_gpu_solve_batch(int32_t B, const double* Hloc, int64_t stride_hloc,
                        const double* Hk, int64_t Nk,
                        const double* bath_h, int64_t stride_bath_h,
                        const double* bath_v, int64_t stride_bath_v,
                        double* omega_out);

/* Results of the last vca_gpu_solve (VCA_IO/get_sft_potential.f90:1-4). */
int vca_gpu_get_sft_potential(double* omega);
/* Ground-state energy E_gs and Omega integral: sft = egs - omega_int. */
int vca_gpu_get_energies(double* egs, double* omega_int);

/*
 * Cluster Green's function G'(z) at nz complex points (VCA_IO/gf_cluster.f90:
 * 1-64, including the off-diagonal recombination :50-62).  gf_out has shape
 * (Nlat,Nlat,Nspin,Nspin,Norb,Norb,nz), complex, spin-off-diagonal blocks 0.
 */
int vca_gpu_gf_cluster(const double* z, int64_t nz, double* gf_out);

/*
 * Matsubara / real-axis cluster Green's function on the reference grids
 * wm = pi/beta*(2n-1), n=1..Lmats and wr = linspace(wini,wfin,Lreal)+i*eps
 * (VCA_GF_SHARED.f90:43-56, accumulation VCA_GF_NORMAL.f90:1024-1031):
 * shapes (Nlat,Nlat,Nspin,Nspin,Norb,Norb,Lmats|Lreal).
 */
int vca_gpu_get_gimp_matsubara(double* g_out);
int vca_gpu_get_gimp_realaxis(double* g_out);
/* Cluster self-energy Sigma = G0^-1 - G'^-1 with G0^-1(z) = (z + xmu) - Hloc
 * - Delta(z), on the Matsubara grid (Lmats points) or the real axis (Lreal
 * points, + i*eps); same layout as the G getters.  Replaces
 * vca_get_sigma_matsubara / vca_get_sigma_realaxis (VCA_IO/get_sigma_*.f90,
 * filled by build_sigma_normal, VCA_GF_NORMAL.f90:1045-1111). */
int vca_gpu_get_sigma_matsubara(double* s_out);
int vca_gpu_get_sigma_realaxis(double* s_out);
/* The non-interacting cluster G0 = (G0^-1)^-1 on the same grids; the
 * reference forms impG0mats/impG0real in build_sigma_normal and writes them
 * with vca_print_impG0 (VCA_IO.f90:179-205). */
int vca_gpu_get_g0_matsubara(double* g0_out);
int vca_gpu_get_g0_realaxis(double* g0_out);
/* splot files of the last solve (vca_print_impSigma / vca_print_impG /
 * vca_print_impG0, VCA_IO.f90:112-205): Sigma, G' or G0 on the Matsubara and
 * the real-axis grid, one file per spin-diagonal element and grid in the
 * working directory, named
 *   <impSigma|impG|impG0>_Isite<ilat:4 digits>_Jsite<jlat:4 digits>_l<iorb><jorb>_s<ispin>_<iw|realw><file_suffix>.vca
 * one line per frequency: x, Im, Re (SciFortran splot's column order) with
 * 17 significant digits.  vca_gpu_solve, _solve_batch (its last point) and
 * _solve_resident call them when cfg.print_sigma / print_impg / print_impg0
 * are set, as vca_solve does with PRINT_SIGMA / PRINT_IMPG / PRINT_IMPG0
 * (VCA_GREENS_FUNCTIONS.f90:37-41).  The flags default to off here: at the
 * reference's grid sizes the files hold ~10^6 lines per solve, more time
 * than the GPU solve itself. */
int vca_gpu_print_impSigma(void);
int vca_gpu_print_impG(void);
int vca_gpu_print_impG0(void);
/* vca_read_impSigma (VCA_IO.f90:208-239): Sigma on both grids from the
 * impSigma splot files above (cfg.file_suffix, the config's Lmats/Lreal
 * lines each); until the next solve the Sigma getters return it, as the
 * reference's read fills impSmats / impSreal.  Needs vca_gpu_init only.
 * vca_splot_read: one such file, n lines of x, Im, Re, into x (may be NULL)
 * and y (complex); host only. */
int vca_read_impSigma(void);
int vca_splot_read(const char* path, int64_t n, double* x, double* y);

/* Ground-state observables of the last solve, (Nlat,Norb) column-major:
 * density n_up + n_dw, its spin parts, double occupancy n_up n_dw and
 * magnetisation n_up - n_dw, averaged over the kept states with weight
 * 1/zeta (T=0) or exp(-beta (E_i - E_min))/zeta (finite T).  Replace vca_get_dens / vca_get_docc / vca_get_mag
 * (VCA_IO/get_dens.f90, get_docc.f90, get_mag.f90), filled by
 * vca_lanc_observables (VCA_OBSERVABLES.f90:185-316). */
int vca_gpu_get_dens(double* out);
int vca_gpu_get_dens_up(double* out);
int vca_gpu_get_dens_dw(double* out);
int vca_gpu_get_docc(double* out);
int vca_gpu_get_mag(double* out);

/*
 * State list of the last solve (VCA_DIAG.f90:220-236, VCA_EIGENSPACE.f90:
 * 136-312): number of retained states (the T=0 ground states, or the trimmed
 * finite-T list), and per state, in list order (ascending energy), its
 * sector (1-based, as get_Sector) and energy.
 */
int vca_gpu_get_state_count(int32_t* nstates);
int vca_gpu_get_state(int32_t istate, int32_t* isector, double* energy);
/* Lowest eigenvalue found in every sector (Nsectors entries, 1-based order);
 * sectors not scanned hold +inf. */
int vca_gpu_get_sector_energies(double* e_out, int32_t n);

/*
 * Pole/weight table of one Green's function element, the GFmatrix of
 * VCA_VARS_GLOBAL.f90:54-71 filled by VCA_GF_NORMAL.f90:970-1033:
 * element (ilat,jlat,ispin,iorb,jorb) 1-based, state istate, channel ichan.
 * *nexc receives the number of excitations, min(target dimension,
 * LANC_NGFITER) as the reference allocates it: a chain that stopped early
 * also lists the eigenvalues 0 of its zero-padded coefficients (poles
 * isign*(0 - E_i), weight 0).  poles and weights (complex, capacity cap)
 * receive them when cap >= *nexc.
 */
int vca_gpu_get_gf_channel(int32_t ilat, int32_t jlat, int32_t ispin, int32_t iorb,
                           int32_t jorb, int32_t istate, int32_t ichan, int32_t* nexc,
                           double* poles, double* weights, int32_t cap);

/*
 * GFmatrix restart files (save_gfprime / read_gfprime, VCA_AUX_FUNX.f90:
 * 601-697): the pole tables of every spin-diagonal element in file
 * file//suffix//".restart" (".used" when used != 0), formatted = list-directed
 * text or 0 = sequential unformatted records (write_formatted /
 * write_unformatted, :486-593).  suffix NULL means cfg.file_suffix, the
 * module variable the reference appends.
 * save: the tables of the last solve, as vca_gpu_get_gf_channel lists them.
 * read: needs vca_gpu_init only; the tables replace the solve's until the
 * next solve, for vca_gpu_gf_cluster (evaluated on the GPU as
 * sum weight/(z - pole) per element, then the recombination) and
 * vca_gpu_get_gf_channel.  The Sigma/G0 getters keep the solve's grids, as
 * the reference's read_gfprime replaces impGmatrix only.
 */
int vca_gpu_save_gfprime(const char* file, const char* suffix, int32_t used, int32_t formatted);
int vca_gpu_read_gfprime(const char* file, const char* suffix, int32_t used, int32_t formatted);
/*
 * The file layout alone, host code that needs no GPU and no context.  A
 * table of nelem elements (file order: ilat, jlat, ispin, iorb, jorb from the
 * outer to the inner loop) is flattened as
 *   nstates[nelem], nchan[sum nstates], nexc[sum nchan],
 *   poles and weights: 2*sum nexc doubles each (re, im pairs).
 * vca_gfm_read: sizes[3] receives (sum nstates, sum nchan, sum nexc).  With
 * nstates == NULL only the sizes are returned; otherwise sizes holds on entry
 * the capacities of nchan, nexc and of the poles/weights in complex entries
 * (nstates holds nelem), and VCA_ERR_ARG is returned when the file needs
 * more.
 */
int vca_gfm_write(const char* path, int32_t formatted, int64_t nelem, const int32_t* nstates,
                  const int32_t* nchan, const int32_t* nexc, const double* poles, const double* weights);
int vca_gfm_read(const char* path, int32_t formatted, int64_t nelem, int64_t* sizes, int32_t* nstates,
                 int32_t* nchan, int32_t* nexc, double* poles, double* weights);

/*
 * The state-list logic the solve runs on the host, without a context or a
 * GPU.  E holds every sector's lowest energy (Nsectors entries, 1-based
 * sector order), as the batched ground-state search returns them.
 * T=0 (VCA_DIAG.f90:224-236): the kept states, each inserted before the
 * first entry with e <= its energy (es_insert_state_c, VCA_EIGENSPACE.f90:
 * 167-216); *n = their number, sectors/energies the first cap of them.
 * Finite T with one state per sector (VCA_DIAG.f90:78-256, vca_post_diag
 * :357-451): the annealed list from LANC_NSTATES_TOTAL = nstates_total, zeta
 * (before the trim), E_min and the adjusted LANC_NSTATES_TOTAL; cfg gives
 * BETA, CUTOFF, LANC_NSTATES_STEP and LANC_NITER_SPECTRUM.
 */
int vca_state_list_t0(const double* E, int32_t nsectors, double gs_threshold, int32_t* sectors, double* energies,
                      int32_t cap, int32_t* n);
/* More host logic of the solve, without a context or a GPU.
 * vca_pair_kpoints: the k-points the Omega k-sum keeps for Hk (nel complex
 * entries per k, Nk points): a point and its partner with H_k' = conj(H_k)
 * (entry-wise to 1e-13 (1 + max|H|)) as one representative of weight 2,
 * other points with weight 1; representatives ascending.
 * vca_contour_rule: the nodes and weights on theta in [0, pi] of the fixed
 * rule that replaces quad(integral_contour, 0, pi) (VCA_OMEGA.f90:172) at
 * radius R: ngl Gauss-Legendre nodes per panel, panels graded from the angle
 * of the Fermi pole xmu + i(2n+1)pi/beta nearest the arc. */
int vca_pair_kpoints(const double* Hk, int64_t Nk, int64_t nel, int64_t* reps, double* weights, int64_t cap,
                     int64_t* nrep);
int vca_contour_rule(double R, double beta, double mu, int32_t ngl, double* theta, double* weights, int32_t cap,
                     int32_t* n);
int vca_state_list_finite_t(const double* E, int32_t nsectors, const vca_config* cfg, int32_t nstates_total,
                            int32_t* sectors, int32_t cap, int32_t* n, double* zeta, double* emin,
                            int32_t* nstates_total_out);
/* The host eigensolvers of the "arpack" diagonalisation, without a context
 * or a GPU.  vca_tridiag_eig: the symmetric tridiagonal matrix with diagonal
 * d[0..n-1] and off-diagonal e[0..n-2] (implicit QL, Wilkinson shifts);
 * vca_herm_eig: the Hermitian n x n matrix A (row-major, complex
 * interleaved; cyclic Jacobi).  Eigenvalues ascending in w; eigenvectors as
 * the columns of Z (column-major; complex interleaved for vca_herm_eig), or
 * Z = NULL.  They stand in for SciFortran's sp_eigh/eigh (VCA_DIAG.f90:
 * 153-170) on the Ritz problem and below LANC_DIM_THRESHOLD. */
int vca_tridiag_eig(int32_t n, const double* d, const double* e, double* w, double* Z);
/* The host-side hop orders of the fixed-point H x v, without a context or a
 * GPU.  vca_hop_schedule: the bank schedule of the paired-column kernel for
 * one spin space of dim configurations (hop words src | class << 24 |
 * sign << 31, width per row, k-major [h*dim + row]; cnt per row): warp w's
 * rounds start at wround[w] (nwarps + 1 entries) in groups of one class and
 * sign with wgrp[w*2K + g] rounds each; sched holds 32 words per round, the
 * byte offset (16 per unit) of the 16-byte unit each lane reads, units >= dim
 * being the zero units of idle lanes; *nrounds = total rounds, *conflicts =
 * quarter-warp rounds left with a bank conflict.  vca_hop_parity_order: the
 * chains' kernel's up hops (the same word layout, sign sorted, npos
 * positive ones per row) re-ordered in place so that rows 2i and 2i+1 read
 * sources of opposite parity where the counts allow. */
int vca_hop_schedule(int32_t dim, int32_t width, int32_t K, const int32_t* cnt, const uint32_t* hop, uint32_t* sched,
                     int64_t sched_cap, int32_t* wround, int32_t* wgrp, int64_t* nrounds, int64_t* conflicts);
int vca_hop_parity_order(int32_t dim, int32_t width, const int32_t* cnt, const int32_t* npos, uint32_t* rhop);
int vca_herm_eig(int32_t n, const double* A, double* w, double* Z);

/* Omega integrand f(w) = (1/Lk) sum_k ln|det(1+(Delta+Hloc-Hk)G'(iw))|
 * (VCA_OMEGA.f90:37-75) at nw real frequencies, from the last solve. */
int vca_gpu_sum_kmesh(const double* w, int64_t nw, double* f_out);
/* Complex integrand F(z) = (1/Lk) sum_k log det(1+(Delta+Hloc-Hk)G'(z)),
 * principal branch per k (sum_kmesh_complex, VCA_OMEGA.f90:78-114), at nz
 * complex points z (interleaved re, im); f_out complex[nz]. */
int vca_gpu_sum_kmesh_complex(const double* z, int64_t nz, double* f_out);

/*
 * One custom observable of the last solve: init_custom_observables /
 * add_custom_observable / get_custom_observables (VCA_OBSERVABLES.f90:
 * 76-165) for a single item, whose value the reference prints and writes
 * (write_custom_observables).  s is (Nlat,Nlat,Nspin,Nspin,Norb,Norb)
 * complex, the same at every k (kdep = 0, add_custom_observable_local), or
 * (...,Nk) (kdep = 1, add_custom_observable_kdep).  With the lattice
 * G_k(z) = (G'(z)^-1 - (H_k - Hloc - Delta(z)))^-1 the value is, at T=0,
 * (3-Nspin)/pi * int_0^inf (1/Lk) sum_k Re{Tr[s_k G_k(iw)] - Tr[s_k]/(iw -
 * 1.1)} dw (:337-347, :408-452) on the fixed rule of the Omega integral; at
 * finite T the Matsubara sum up to nmax plus the contour over the whole
 * circle |w| = R (:351-388, :454-500) with the reference's real part of the
 * trace, times (3-Nspin).
 */
int vca_gpu_custom_observable(const double* s, int32_t kdep, double* value);

/* Thermal bookkeeping of the last solve. */
typedef struct vca_thermal {
  double zeta;           /* zeta_function (VCA_DIAG.f90:357-363), before trimming */
  double omega_prime;    /* Omega' of the cluster (VCA_MAIN.f90:186-193)       */
  double e_min;          /* state_list%emin                                    */
  double max_exc;        /* largest pole excitation of all chains (VCA_GF_NORMAL.f90:1018) */
  double integration_R;  /* radius of the contour (VCA_OMEGA.f90:158-166)      */
  double sum_part;       /* 2/beta sum_{n=0..nmax} Re F(i w_n)                 */
  double contour_part;   /* integral over the contour                          */
  int32_t nmax;          /* last Matsubara index of the sum                    */
  int32_t nstates_total; /* LANC_NSTATES_TOTAL after this solve's adjustment  */
  int32_t contour_points;/* nodes of the contour rule                          */
  int32_t finite_t;      /* 1 when the solve ran the finite-T path             */
} vca_thermal;
/* At T=0: zeta = number of kept states, omega_prime = e_min = E_gs and the
 * Omega fields after e_min are 0. */
int vca_gpu_get_thermal(vca_thermal* out);

/* Release every device buffer and the stream. */
int vca_gpu_finalize(void);

/* Text of the last error (empty when none).  Returns the string length. */
int vca_gpu_last_error(char* buf, int32_t len);

/* ---- parity hooks on the H x v contract ------------------------------- */
/*
 * Sector information (VCA_SETUP.f90:404-458,660-695): 1-based isector,
 * n_up, n_dw, DimUp, DimDw.  Needs vca_gpu_init only.
 */
int vca_gpu_sector_info(int32_t isector, int32_t* nup, int32_t* ndw, int64_t* dimup,
                        int64_t* dimdw);
/* Fock words of the up (spin=1) or down (spin=2) map of a sector, built on
 * the GPU (build_sector, VCA_SETUP.f90:660-695): map[k] = word, k = 0..Dim-1. */
int vca_gpu_sector_map(int32_t isector, int32_t spin, int64_t* map, int64_t cap);
/*
 * Load the one-body data of a solve point without solving: Hloc, bath_h,
 * bath_v as in vca_gpu_solve.  Used before vca_gpu_hxv.
 */
int vca_gpu_set_hamiltonian(const double* Hloc, const double* bath_h, const double* bath_v);
/*
 * Hv = H v on sector isector: the cc_sparse_HxV(Nloc,v,Hv) contract of
 * VCA_VARS_GLOBAL.f90:83-89 with the stored semantics of
 * VCA_HAMILTONIAN_SPARSE_HxV.f90:152-200.  v, hv: complex[dim] host arrays,
 * index i = iup + (idw-1)*DimUp (1-based, VCA_SETUP.f90:505-518).
 */
int vca_gpu_hxv(int32_t isector, const double* v, double* hv);
/* Same product on DEVICE buffers: v/hv are complex[dim] (is_complex=1) or
 * real[dim] (is_complex=0, only for a real Hamiltonian), on the library stream. */
int vca_gpu_hxv_device(int32_t isector, const void* d_v, void* d_hv, int32_t is_complex);
/* Run the H x v kernel `reps` times on device buffers holding ncols vectors
 * interleaved element-major (v[i*ncols + c]) and report the mean device time
 * per launch in milliseconds (CUDA events on the library stream).  No
 * counterpart in the reference: a measurement hook. */
int vca_gpu_hxv_timed(int32_t isector, const void* d_v, void* d_hv, int32_t is_complex,
                      int32_t ncols, int32_t reps, double* ms_per_call);

/* Allocation-free column H x v: Y = H X on ncols real columns of sector
 * isector (device buffers laid out as for vca_gpu_hxv_timed) and
 * d_alpha[c] = <x_c, H x_c> (device, ncols doubles), on the library stream.
 * For callers that cannot call cudaMalloc while they run (device memory owned
 * by their own pool allocator, or a sweep that must not reach the driver's
 * allocator mid-run): the partial sums behind alpha live in a static 8 MiB
 * device array, so the call allocates nothing.  Batches whose partial sums
 * exceed 8 MiB are rejected with VCA_ERR_ARG.  The first call on a device
 * looks the array up (make it before any stream capture); the address is
 * kept until vca_gpu_finalize, so after a device reset finalize and init
 * again.  All calls share the array, so calls whose work overlaps on the GPU
 * race.  No counterpart in the reference. */
int vca_gpu_hxv_alpha_noalloc(int32_t isector, const void* d_v, void* d_hv, int32_t ncols,
                              double* d_alpha);
/* (Device vectors passed to the H x v entry points must be 16-byte aligned,
 * as cudaMalloc and torch allocations are; others are rejected with
 * VCA_ERR_ARG.) */

/* ---- residency and diagnostics (no counterpart in the reference) -------- */
/* Upload Hk (as in vca_gpu_solve) and keep it resident on the device. */
int vca_gpu_upload_hk(const double* Hk, int64_t Nk);
/* vca_gpu_solve with the resident Hk of the last upload/solve. */
int vca_gpu_solve_resident(const double* Hloc, const double* bath_h, const double* bath_v,
                           double* omega_out);
/* Kernel launches issued by the library since it was loaded. */
int64_t vca_gpu_kernel_launches(void);
/* The k lowest eigenpairs of sector isector of the loaded Hamiltonian as the
 * "arpack" diagonalisation finds them (LANC_METHOD="arpack", VCA_DIAG.f90:
 * 153-170): dense below LANC_DIM_THRESHOLD (or k >= dim), else a Lanczos
 * with full reorthogonalisation to LANC_TOLERANCE.  *n = pairs found
 * (<= min(k, dim)); energies ascending; vecs (NULL or n*dim complex
 * interleaved doubles, vector j at j*dim) unit-norm FP64.  No counterpart
 * in the reference (its sp_eigh call). */
int vca_gpu_sector_pairs(int32_t isector, int32_t k, double* energies, double* vecs, int32_t* n);
/* Wall-clock milliseconds of the last solve's stages: [0] one-body tables,
 * [1] sector diagonalisation, [2] Green's function chains, [3] Omega; with
 * n >= 10 also the last batched-form vca_gpu_solve_batch's stages over all
 * its points: [4] tables, [5] ground-state search, [6] eigenvectors,
 * [7] chains, [8] Omega, [9] the closing plain solve of the last point;
 * with n >= 11, [10] the (point, sector) searches its screening skipped;
 * with n >= 13, [11] rows per tile and [12] row lanes per block of its
 * chains' (autotuned) tile shape; with n >= 16, the last solve's chain
 * stage split into [13] start vectors and [14] Lanczos steps (ms) and
 * [15] its column batches. */
int vca_gpu_get_timings(double* ms, int32_t n);
/* Arithmetic of the loaded Hamiltonian: *fx = 1 when the fixed-point path is
 * active, with vector scale 2^-F and H v scale 2^-G.  In that case the device
 * buffers of vca_gpu_hxv_device / vca_gpu_hxv_timed hold int64 fixed-point
 * columns (unit norm, scale 2^-F in, 2^-G out), slab-major once there are 8
 * or more: slabs of 8 adjacent columns, each a contiguous [dim][8] block
 * (element (i, c) at ((c/8)*dim + i)*8 + c%8), ncols a multiple of 8. */
int vca_gpu_arith_info(int32_t* fx, int32_t* F, int32_t* G);
/* Row order of a sector's fixed-point column batches under hxv_variant 2
 * (the order the library's Green's function chains use): order[r] is the
 * sector element index (iup + idw*DimUp) held in batch row r; up
 * configurations are sorted by decreasing hop count.  cap >= DimUp*DimDw. */
int vca_gpu_sector_row_order(int32_t isector, int64_t* order, int64_t cap);
/* Wait for all work on the library stream. */
int vca_gpu_synchronize(void);
/* The batched form's Green's-function chains run as column tasks whose tile
 * shape (rows per tile, row lanes per block) is tuned at first use for each
 * problem class: every candidate's H x v is timed on the call's own first
 * tasks and the fastest kept for the life of the process (on = 1, default).
 * on = 0 runs the fixed shape (64 rows, 8 lanes).  The shape changes only
 * the summation order of the chains' dot products.  No counterpart in the
 * reference. */
int vca_gpu_set_autotune(int32_t on);
/* The position-ordered column H x v (the Green's-function chains' kernel)
 * reads its up hops in an order that pairs the two rows of each quarter
 * warp with sources of opposite parity, so their 16-byte shared-memory
 * reads fall in different banks (on = 1, default); on = 0 keeps the plain
 * sign-sorted order.  Takes effect when the next Hamiltonian's tables are
 * built; results are bit-identical either way.  No counterpart in the
 * reference. */
int vca_gpu_set_hop_pairing(int32_t on);
/* The Green's-function chains run as column groups; n = 1 (default) runs
 * one group after another, n = 2 keeps two groups in flight on two
 * streams with their Lanczos steps interleaved, so that one group's H x v
 * could overlap the other's element passes (each group then gets a quarter
 * of the free memory instead of half).  On the 4x3 benchmark solve two
 * streams are 1 % slower: the chains' H x v fills every SM.  Results are
 * bit-identical either way.  No counterpart in the reference. */
int vca_gpu_set_chain_streams(int32_t n);
/* Test hook of the bounded waits in the chains' column H x v: its own-block
 * bulk copy (cp.async.bulk, mbarrier completion) is awaited for at most one
 * second; with bytes > 0 the barrier expects that many bytes more than are
 * copied, so the wait runs out (no fault), the kernel returns early, and
 * the call that ran it (vca_gpu_solve, vca_gpu_hxv_timed) returns
 * VCA_ERR_TIMEOUT.  bytes = 0 (default) restores normal operation.  No
 * counterpart in the reference. */
int vca_gpu_set_stage_extra_tx(int32_t bytes);
/* The T=0 Omega integrand ln|det(1 + M_k G'(iw))| (VCA_OMEGA.f90:66-67) is
 * evaluated as ln|det(G'^-1 + M_k)| + ln|det G'| at nodes w <= 10, with G'^-1
 * and ln|det G'| formed once per node, which saves the M_k G' product at
 * every k (on = 1, the default); on = 0 keeps the product form everywhere.
 * No counterpart in the reference; a switch for tests and measurements. */
int vca_gpu_set_omega_inverse_form(int32_t on);
/* Lower bound of every sector's lowest energy for the loaded Hamiltonian
 * (out[isector-1]): the one-body part's ground energy in that sector, valid
 * when U, Ust and Ust - Jh are non-negative (VCA_ERR_UNSUPPORTED otherwise).
 * The batched form skips sectors with it; no counterpart in the reference. */
int vca_gpu_sector_bounds(double* out, int32_t n);
/* QL sweeps allowed per eigenvalue when the chains' tridiagonals are turned
 * into poles and weights (default 60).
 * A chain that needs more makes the call that asked for poles (the channel
 * getter, the finite-T max_exc, save_gfprime) return VCA_ERR_NUMERIC instead
 * of poles from an unfinished QL.  No counterpart in the reference (SciFortran's
 * eigh stops the process); lowering it makes the failure path testable. */
int vca_gpu_set_ql_max_iter(int32_t max_iter);
/* CUDA events on the library stream: device time between start and stop. */
int vca_gpu_timer_start(void);
int vca_gpu_timer_stop(double* ms);

/* ---- the Omega surrogate (no counterpart in the reference) -------------- */
/*
 * A 4 -> 128 -> 128 -> 128 -> 1 SiLU network fitted on the GPU to Omega
 * values and gradients that the solver produces (loss per sample
 * (f - y)^2 + grad_weight * |grad f - dy|^2, averaged), with BF16 tensor-core
 * GEMMs and FP32 master weights, trained by Adam.  It proposes candidates for
 * the stationary-point search that the reference's drivers run with brent or
 * fmin_bfgs (drivers/vca_hm_chain1d.f90:104-108, drivers/vca_bhz_2d.f90:
 * 244-305); each accepted candidate is re-solved by vca_gpu_solve.  Inputs
 * and targets are expected already scaled to O(1).  One global network, not
 * thread-safe, like the solver context.
 */
typedef struct vca_mlp_config {
  int32_t n_in;          /* network inputs, 1..4                              */
  int32_t capacity;      /* most training samples / prediction points         */
  uint64_t seed;         /* Glorot-uniform initial weights                    */
  double lr;             /* Adam step size                                    */
  double beta1, beta2, adam_eps;
  double grad_weight;    /* weight of the gradient term of the loss           */
  double weight_decay;   /* decoupled weight decay on the weights (not biases) */
} vca_mlp_config;
void vca_mlp_config_defaults(vca_mlp_config* cfg);
int vca_mlp_init(const vca_mlp_config* cfg);
int vca_mlp_finalize(void);
/* Flat FP32 parameters: W1[128][n_in], b1[128], W2[128][128], b2[128],
 * W3[128][128], b3[128], w4[128], b4 (W[out][in], row-major). */
int64_t vca_mlp_param_count(void);
int vca_mlp_get_params(float* out, int64_t n);
int vca_mlp_set_params(const float* in, int64_t n); /* also resets Adam */
/* Training set: x[n][n_in], y[n], dy[n][n_in] and per-sample weights gw[n]
 * of the gradient term (the loss of sample j uses grad_weight * gw[j]; gw
 * NULL: all 1; dy NULL: zero targets -- give samples without gradient data
 * gw = 0). */
int vca_mlp_set_data(int32_t n, const double* x, const double* y, const double* dy,
                     const double* gw);
/* Loss and its gradient with respect to every parameter at the current
 * weights (no update): the check against the CPU restatement. */
int vca_mlp_loss_grad(double* loss, float* grad, int64_t n);
/* `steps` full-batch Adam steps (one step is a replayed CUDA graph); *loss =
 * the loss at the final weights.  VCA_ERR_TIMEOUT if a bounded tensor-core
 * wait ran out. */
int vca_mlp_train(int32_t steps, double* loss);
/* f[n] and, when df is not NULL, the input gradients df[n][n_in]. */
int vca_mlp_predict(int32_t n, const double* x, double* f, double* df);
/* Test hook of the tensor-core GEMM: C[M][128] (+)= A[M][K] B[128][K]^T with
 * A, B row-major bf16 bit patterns, M a multiple of 128, K of 64. */
int vca_umma_gemm_check(const uint16_t* A, const uint16_t* B, float* C, int32_t M, int32_t K,
                        int32_t accumulate);
/* Test hook of the GEMM's bounded waits: a 128 x 64 GEMM whose load barrier
 * expects bytes that never arrive.  Returns VCA_ERR_TIMEOUT after about a
 * second, with the CUDA context still usable. */
int vca_umma_timeout_check(void);

#ifdef __cplusplus
}
#endif

#endif /* VCA_GPU_H */
