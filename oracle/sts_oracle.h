/* CPU oracle for the diffusion_2D super-time-stepping path — TEST INFRASTRUCTURE ONLY.
 *
 * This library restates, in plain C on the host, the arithmetic of the path that the
 * reference runs through SUNDIALS (ARKODE LSRKStep + NVECTOR + PCG) and its own
 * problem callbacks (diffusion_2D/diffusion.cpp, preconditioner_jacobi.cpp, main.cpp).
 * It is the checker for the CUDA library in ceda_demonstrations_gb300/csrc: tests,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg are the only callers.
 * Nothing in the product links or calls it.
 *
 * Parity status: SUNDIALS (git submodule deps/sundials) is empty in the reference
 * tree, so the integrator constants are restated from the RKC/RKL2 papers and the
 * SUNDIALS/ARKODE documentation; results cannot be compared with a SUNDIALS build
 * ("parity unpinned" with respect to SUNDIALS). The oracle is pinned against the
 * reference's own known-answer tests (gkeyll_diffusion/test_nvector_gkylzero.c,
 * gkeyll_diffusion/analytic_CR_test.c) and analytic facts of the discretisation.
 */
#ifndef STS_ORACLE_H
#define STS_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

/* Problem kinds. */
#define ORC_MANUFACTURED 0 /* [0,1]^2, homogeneous Dirichlet, u=sin^2(pi x)sin^2(pi y)cos^2(2 pi t) */
#define ORC_UNFORCED 1     /* [0,1]^2, homogeneous Dirichlet, no forcing (batched instances) */
#define ORC_PERIODIC 2     /* reference mode: periodic, Gaussian x sine IC, optional k(1+0.99 sin) */

typedef struct orc_prob {
  int nx, ny, kind, inhomogeneous;
  double kx, ky, xl, xu, yl, yu, dx, dy;
  double cx, cy, cc; /* kx/dx^2, ky/dy^2, -2(cx+cy) */
  double *Sx, *Sxx, *Sy, *Syy;
  double *Dxw, *Dxe, *Dys, *Dyn; /* periodic-mode face coefficients / d^2 */
} orc_prob;

typedef struct orc_opts {
  int method;      /* 0 = RKC2, 1 = RKL2 */
  int mixed;       /* 0 = FP64 stages, 1 = FP32 increments relative to the FP64 step start */
  int controller;  /* 0 = PID, 1 = PI, 2 = I (ARK_ADAPT_PID / PI / I) */
  int smax;        /* stage limit (SUNDIALS default 200) */
  int internaleig; /* 0 = analytic dom_eig (main.cpp:536-550), 1 = power iteration */
  int dee_maxiters;
  int dom_eig_freq;
  int pad_;
  long maxsteps;   /* per evolve call; <= 0 means 500 */
  double rtol, atol, hfixed, eig_safety, dee_reltol;
  int dee_init_warmups, dee_succ_warmups; /* power iterations before the first / later estimates */
} orc_opts;

/* stop time and dense output of an evolve (the product's ARKodeEvolve return rules): the
 * integrator's state y_n, the last step's y_old and f_old, the stop time, the time last
 * returned */
typedef struct orc_dense {
  double *ycur, *yold, *fold;
  double tstop, tretlast;
  int tstopset, interp_ready;
} orc_dense;

typedef struct orc_state {
  double t, hnext, hlast, spectral_radius, ep1, ep2;
  long nst, nst_attempts, netf, nfe, nfe_dee, ndee, nst_exp, stage_max, stages_total;
  long nhist, steps_since_dee;
  int initialized, after_fail;
  double *F;  /* F(t_n, y_n) in FP64 (FSAL) */
  float *Ff;  /* FP32 copy used by the mixed stages */
  double *evec; /* power-iteration eigenvector (warm start) */
  orc_dense d;
} orc_state;

/* exact, order-independent reductions (value = RN(sum of trunc(x_i * 2^160)) * 2^-160) */
double orc_xsum(const double* x, long n);
double orc_xdot(const double* x, const double* y, long n);
double orc_wrms(const double* x, const double* w, long n);
double orc_maxnorm(const double* x, long n);

orc_prob* orc_prob_create(int kind, int nx, int ny, double kx, double ky, int inhomogeneous,
                          double xl, double xu, double yl, double yu);
void orc_prob_free(orc_prob* p);
void orc_initial(const orc_prob* p, double* u);
void orc_initial_modes(const orc_prob* p, int nmodes, const int* pm, const int* qm,
                       const double* amp, double* u);
void orc_exact(const orc_prob* p, double t, double* u);
double orc_c(double t);
double orc_cdot(double t);
void orc_rhs(const orc_prob* p, double t, const double* u, double* f);
void orc_rhs_ref(const orc_prob* p, double t, const double* u, double* f);
void orc_apply_A(const orc_prob* p, const double* v, double* w);
double orc_dom_eig(const orc_prob* p);
int orc_power_iteration(const orc_prob* p, double* v, int maxiters, double reltol, double* lambda);

int orc_stage_coeffs(int method, int s, double* mu, double* nu, double* mus, double* ajm1,
                     double* cjm1);
int orc_stages_needed(int method, double h, double rho, int smax, double* hmax);
double orc_pow(double x, double y); /* deterministic pow of the controllers */
/* SSP methods (type 2 = SSP(s,2), 3 = SSP(s,3), 4 = SSP(10,4)) */
int orc_ssp_weights(int type, int s, double* b, double* c, double* w);
int orc_ssp_evolve(const orc_prob* p, const orc_opts* o, int type, int s, orc_state* st, double tout, double* y);
double orc_controller(int controller, double h, double dsm, double ep1, double ep2, double hp, long nhist);

/* evolve: y is the initial state on the first call and the output afterwards (the integrator
 * keeps its own y_n); a stop time clips the steps and is cleared when returned (return 1);
 * the time returned is st->d.tretlast */
void orc_state_init(orc_state* st, double t0);
void orc_state_free(orc_state* st);
int orc_lsrk_evolve(const orc_prob* p, const orc_opts* o, orc_state* st, double tout, double* y);

int orc_pcg(const orc_prob* p, double gamma, int jacobi, const double* b, double* x,
            double tol, int maxit, double* relres);
int orc_sdirk2(const orc_prob* p, double t0, double h, int nsteps, double tol, int maxit,
               double* y, long* total_iters);

/* generic SUNLinSol_PCG / SUNLinSol_SPGMR on (I - gamma A) x = b, Jacobi or none; SDIRK2 with them */
int orc_pcg_generic(const orc_prob* p, double gamma, int jacobi, const double* b, double* x, double tol,
                    int maxl, int* iters, double* relres);
int orc_spgmr(const orc_prob* p, double gamma, int jacobi, const double* b, double* x, double tol, int maxl,
              int max_restarts, int gstype, int* iters, double* relres);
int orc_spfgmr(const orc_prob* p, double gamma, int jacobi, const double* b, double* x, double tol, int maxl,
               int max_restarts, int gstype, int* iters, double* relres);
int orc_sdirk2_ls(const orc_prob* p, double t0, double h, int nsteps, double tol, int ls, int maxl,
                  int max_restarts, int gstype, int jacobi, double* y, long* total_iters);
/* PFMG-role V-cycle (relax 1 weighted Jacobi, 2 symmetric red/black Gauss-Seidel) and CG with it */
int orc_pfmg_vcycle(const orc_prob* p, double gamma, int relax, int nrelax, const double* r, double* z, int* nlevels);
int orc_pcg_pfmg(const orc_prob* p, double gamma, int relax, int nrelax, const double* b, double* x, double tol,
                 int maxl, int* iters, double* relres);
int orc_sdirk2_pfmg(const orc_prob* p, double t0, double h, int nsteps, double tol, int maxl, int relax, int nrelax,
                    double* y, long* total_iters);
/* ARKStep (csrc/arkstep.cu): implicit DIRK (order 2 / 3) with Newton + PCG (ls 0) or SPGMR
 * (ls 1), preconditioner prec 0 none / 1 Jacobi / 2 PFMG; explicit ERK (order 2 / 3 / 4) */
typedef struct orc_ark_opts {
  int implicit, order, controller, ls, maxl, max_restarts, gstype, prec, pfmg_relax, pfmg_nrelax, msbp,
      linear, onestep;
  long maxsteps;
  double rtol, atol, hfixed, eplifac;
} orc_ark_opts;
typedef struct orc_ark_state {
  double t, hnext, hlast, h0, ep1, ep2, gamma_setup;
  long nst, nst_att, netf, ncfn, nfe, nfi, nni, nnf, nli, nlcf, npe, nps, njv, nsetups, nhist, nst_setup;
  int initialized, after_fail, force_setup, fn_current;
  double* Fn; /* f(t_n, y_n) when fn_current */
  orc_dense d;
} orc_ark_state;
void orc_ark_state_free(orc_ark_state* st);
/* dense output p(tq) of degree 1..3 on [t - h, t], tau = (tq - t) / h (the product's
 * sts_hermite, csrc/lsrk.cu) */
void orc_hermite(long n, int deg, double tau, double h, const double* yold, const double* ynew,
                 const double* fold, const double* fnew, double* out);
int orc_arkstep_evolve(const orc_prob* p, const orc_ark_opts* o, orc_ark_state* st, double tout, double* y);
int orc_ark_table(int implicit, int order, int* s, int* q, int* pe, double* A, double* b, double* d, double* c);
int orc_nthreads(void);
void orc_set_nthreads(int n);

#ifdef __cplusplus
}
#endif
#endif
