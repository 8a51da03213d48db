// ARKStep: the additive Runge-Kutta stepper of ARKODE in the two forms diffusion_2D/main.cpp
// creates (main.cpp:239-253): implicit DIRK, ARKStepCreate(nullptr, diffusion, ...), with a
// Newton iteration whose linear systems go to a SUNLinearSolver with the user's PSetup /
// PSolve (main.cpp:199-231, 296-330); and explicit ERK, ARKStepCreate(diffusion, nullptr, ...)
// for a non-negative --order. Host C++ over the N_Vector ops; every vector operation is a
// device kernel of nvector.cu and every reduction is exact, so the CPU oracle
// (orc_arkstep_evolve) reproduces a run bit for bit.
//
// Restated from the ARKODE documentation (SUNDIALS is not in the reference tree):
//   Tables (ARKodeSetOrder): implicit order 2 ARKODE_SDIRK_2_1_2 (gamma 1, A = [1 0; -1 1],
//   c = (1, 0), b = (1/2, 1/2), embedding (1, 0)); implicit order 3
//   ARKODE_ARK324L2SA_DIRK_4_2_3 (Kennedy & Carpenter 2003, ESDIRK, gamma ~ 0.4359, stiffly
//   accurate, embedding of order 2); explicit orders 2 / 3 / 4 ARKODE_HEUN_EULER_2_1_2,
//   ARKODE_BOGACKI_SHAMPINE_4_2_3, ARKODE_ZONNEVELD_5_3_4.
//   Implicit stage i: z = sdata + h A_ii f(t_n + c_i h, z), sdata = y_n + h sum_{j<i} A_ij F_j,
//   trivial predictor z = y_n, Newton corrections (I - gamma J) d = sdata + gamma f(z) - z
//   (gamma = h A_ii, J v exact for STS_Diffusion, else a difference quotient), convergence
//   test of ARKODE (crate = max(0.3 crate, del/del_prev), dcon = del min(1, crate) / 0.1,
//   at most 3 corrections, divergence when del > 2.3 del_prev), del = ||d||_WRMS. The linear
//   solve stops at ||r||_WRMS <= eplifac * 0.1 (eplifac 0.05, ARKodeSetEpsLin): the solver's
//   relative 2-norm tolerance is that bound over the WRMS norm of the right side, and a right
//   side already below it gives d = 0 without iterating. ARKodeSetLinear: one correction, no
//   convergence test. PSetup at the first step, every msbp steps (ARKodeSetLSetupFrequency,
//   0 = 20), when gamma moved by more than 20 % since the last setup, and after a convergence
//   failure. After convergence F_i = f(t_i, z) is evaluated again.
//   Step: y_{n+1} = y_n + h sum b_i F_i, error h sum (b_i - d_i) F_i in the WRMS norm with
//   ewt = 1/(rtol |y_n| + atol); the LSRKStep controllers and limits (lsrk.cu) with order
//   p + 1 (p = embedding order); a Newton failure retries with h / 4 (at most 10 per step),
//   at most 7 error-test failures per step. The first stage of an ESDIRK / ERK table reuses
//   f(t_n, y_n), evaluated once per step start.
//   Output: the return rules of STS_ARKodeEvolve (lsrk.cu) with the Hermite dense output of
//   degree min(q - 1, 5); a degree >= 2 output evaluates f(t_n, y_n) when no step start has.
#include <cuda_runtime.h>

#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <utility>
#include <vector>

#include "portable_math.cuh"
#include "sts_internal.cuh"

namespace {

struct Table {
  int s = 0, q = 0, p = 0;
  std::vector<double> A, b, d, c; // A row-major s x s
};

bool make_table(bool implicit, int order, Table* T)
{
  auto set = [&](int s, int q, int p, std::vector<double> A, std::vector<double> b, std::vector<double> d,
                 std::vector<double> c) {
    T->s = s;
    T->q = q;
    T->p = p;
    T->A = A;
    T->b = b;
    T->d = d;
    T->c = c;
  };
  if (implicit && order == 2) set(2, 2, 1, {1.0, 0.0, -1.0, 1.0}, {0.5, 0.5}, {1.0, 0.0}, {1.0, 0.0});
  else if (implicit && order == 3)
  {
    const double g = 1767732205903.0 / 4055673282236.0;
    set(4, 3, 2,
        {0.0, 0.0, 0.0, 0.0,                                                                //
         g, g, 0.0, 0.0,                                                                    //
         2746238789719.0 / 10658868560708.0, -640167445237.0 / 6845629431997.0, g, 0.0,   //
         1471266399579.0 / 7840856788654.0, -4482444167858.0 / 7529755066697.0,
         11266239266428.0 / 11593286722821.0, g},
        {1471266399579.0 / 7840856788654.0, -4482444167858.0 / 7529755066697.0,
         11266239266428.0 / 11593286722821.0, g},
        {2756255671327.0 / 12835298489170.0, -10771552573575.0 / 22201958757719.0,
         9247589265047.0 / 10645013368117.0, 2193209047091.0 / 5459859503100.0},
        {0.0, 2.0 * g, 3.0 / 5.0, 1.0});
  }
  else if (!implicit && order == 2) set(2, 2, 1, {0.0, 0.0, 1.0, 0.0}, {0.5, 0.5}, {1.0, 0.0}, {0.0, 1.0});
  else if (!implicit && order == 3)
    set(4, 3, 2,
        {0.0, 0.0, 0.0, 0.0, 0.5, 0.0, 0.0, 0.0, 0.0, 0.75, 0.0, 0.0, 2.0 / 9.0, 1.0 / 3.0, 4.0 / 9.0, 0.0},
        {2.0 / 9.0, 1.0 / 3.0, 4.0 / 9.0, 0.0}, {7.0 / 24.0, 0.25, 1.0 / 3.0, 0.125}, {0.0, 0.5, 0.75, 1.0});
  else if (!implicit && order == 4)
    set(5, 4, 3,
        {0.0, 0.0, 0.0, 0.0, 0.0,  //
         0.5, 0.0, 0.0, 0.0, 0.0,  //
         0.0, 0.5, 0.0, 0.0, 0.0,  //
         0.0, 0.0, 1.0, 0.0, 0.0,  //
         5.0 / 32.0, 7.0 / 32.0, 13.0 / 32.0, -1.0 / 32.0, 0.0},
        {1.0 / 6.0, 1.0 / 3.0, 1.0 / 3.0, 1.0 / 6.0, 0.0},
        {-0.5, 7.0 / 3.0, 7.0 / 3.0, 13.0 / 6.0, -16.0 / 3.0}, {0.0, 0.5, 0.5, 1.0, 0.75});
  else return false;
  return true;
}

constexpr double NLSCOEF = 0.1, CRDOWN = 0.3, RDIV = 2.3, DGMAX = 0.2, ETACF = 0.25;
constexpr int MAXCOR = 3, MAXNCF = 10, MAXNEF = 7, MSBP_DEFAULT = 20;
constexpr double SAFETY = 0.96, GROWTH = 20.0, ETAMX1 = 10000.0, ETAMXF = 0.3, ETAMIN = 0.1;
constexpr double LBOUND = 1.0, UBOUND = 1.5;
constexpr int SMALL_NEF = 2;

} // namespace

struct ARKStepMem {
  uint32_t kind   = STS_MEM_ARKSTEP; // first member: the ARKode* calls of lsrk.cu dispatch on it
  STS_Context ctx = nullptr;
  STS_ARKRhsFn f  = nullptr; // fe (explicit) or fi (implicit)
  bool implicit   = false;
  void* user_data = nullptr;
  int order       = 0;
  Table T;
  bool table_ok = false;
  double rtol = 1e-4, atol = 1e-9, hfixed = 0.0, tstop = INFINITY;
  int controller     = STS_ADAPT_PID;
  long long maxsteps = 500;
  // implicit solver
  void* LS                    = nullptr;
  STS_ARKLsPrecSetupFn psetup = nullptr;
  STS_ARKLsPrecSolveFn psolve = nullptr;
  void* pdata                 = nullptr; // user data of PSetup / PSolve (default: the RHS user data)
  int msbp                    = 0;
  double eplifac              = 0.05;
  bool linear                 = false;
  // state
  long long n = 0;
  double t = 0, hnext = 0, hlast = 0, h0u = 0, ep1 = 0, ep2 = 0;
  double gamma_setup = 0;
  long long nst = 0, nst_att = 0, netf = 0, ncfn = 0, nfe = 0, nfi = 0, nni = 0, nnf = 0, nli = 0, nlcf = 0;
  long long npe = 0, nps = 0, njv = 0, nsetups = 0, nfe_dq = 0, nhist = 0, nst_setup = 0;
  bool initialized = false, after_fail = false, fn_current = false, force_setup = true;
  // stop time and dense output: after an accepted step `ynew` holds y_old (the vectors are
  // swapped) and F[0] holds f(t_old, y_old) for the explicit-first-stage tables
  bool tstopset = false, interp_ready = false;
  double tretlast = 0;
  // vectors
  N_Vector y = nullptr, Fn = nullptr, sdata = nullptr, z = nullptr, res = nullptr, del = nullptr, ewt = nullptr,
           tmp = nullptr, tmp2 = nullptr, ynew = nullptr;
  std::vector<N_Vector> F;
  // linear-solve context of the current stage
  double cur_t = 0, cur_gamma = 0, cur_tol = 0;
  int cur_i = 0;
};

#define AM(v) ((ARKStepMem*)(v))

static int rhs(ARKStepMem* m, double t, N_Vector y, N_Vector f)
{
  const int rc = m->f(t, y, f, m->user_data);
  if (m->implicit) m->nfi++;
  else m->nfe++;
  return rc;
}

static void* prec_data(ARKStepMem* m) { return m->pdata ? m->pdata : m->user_data; }

// ewt = 1/(rtol |y| + atol) with the same four vector operations the LSRK generic path uses
static void compute_ewt(ARKStepMem* m, N_Vector y)
{
  N_VAbs_Sts(y, m->ewt);
  N_VScale_Sts(m->rtol, m->ewt, m->ewt);
  N_VAddConst_Sts(m->ewt, m->atol, m->ewt);
  N_VInv_Sts(m->ewt, m->ewt);
}

// the shifted operator v -> v - gamma J v at the current stage iterate (t_i, z, F_i)
static int ark_atimes(void* d, N_Vector v, N_Vector out)
{
  ARKStepMem* m = AM(d);
  m->njv++;
  if (m->f == STS_Diffusion)
  {
    if (STS_JacTimes(v, m->tmp, m->cur_t, nullptr, nullptr, m->user_data, nullptr)) return -1;
  }
  else
  { // difference quotient at the current iterate: (f(t, z + sig v) - f(t, z)) / sig,
    // sig = 1 / ||v||_WRMS
    const double vn = N_VWrmsNorm_Sts(v, m->ewt);
    if (!(vn > 0.0))
    {
      N_VConst_Sts(0.0, out);
      return 0;
    }
    const double sig = 1.0 / vn;
    N_VLinearSum_Sts(sig, v, 1.0, m->z, m->tmp2);
    if (m->f(m->cur_t, m->tmp2, m->tmp, m->user_data)) return 1;
    m->nfe_dq++;
    N_VLinearSum_Sts(1.0 / sig, m->tmp, -1.0 / sig, m->F[m->cur_i], m->tmp); // F_i = f(t_i, z)
  }
  N_VLinearSum_Sts(1.0, v, -m->cur_gamma, m->tmp, out);
  return 0;
}

static int ark_psolve(void* d, N_Vector r, N_Vector z, double tol, int lr)
{
  (void)tol;
  ARKStepMem* m = AM(d);
  m->nps++;
  return m->psolve(m->cur_t, m->z, m->F[m->cur_i], r, z, m->cur_gamma, m->cur_tol, lr, prec_data(m));
}

// Newton solve of implicit stage i; returns 0 converged, 1 not converged (recoverable),
// 2 recoverable RHS failure, < 0 fatal
static int solve_stage(ARKStepMem* m, int i, double ti, double gamma)
{
  const double epslin = m->eplifac * NLSCOEF;
  N_VScale_Sts(1.0, m->y, m->z); // trivial predictor
  double crate = 1.0, delp = 0.0;
  m->cur_t     = ti;
  m->cur_i     = i;
  m->cur_gamma = gamma;
  m->cur_tol   = epslin;
  for (int it = 0;; ++it)
  {
    const int frc = rhs(m, ti, m->z, m->F[i]);
    if (frc < 0) return -1;
    if (frc > 0) return 2;
    { // right side of the correction: sdata + gamma F_i - z
      double cf[3]  = {1.0, gamma, -1.0};
      N_Vector X[3] = {m->sdata, m->F[i], m->z};
      N_VLinearCombination_Sts(3, cf, X, m->res);
    }
    if (it == 0 && m->psetup)
    {
      const bool need = m->force_setup || m->nsetups == 0 ||
                        m->nst >= m->nst_setup + (m->msbp > 0 ? m->msbp : MSBP_DEFAULT) ||
                        fabs(gamma / m->gamma_setup - 1.0) > DGMAX;
      if (need)
      {
        int jcur = 0;
        if (m->psetup(ti, m->z, m->F[i], m->force_setup ? 0 : 1, &jcur, gamma, prec_data(m))) return -1;
        m->npe++;
        m->nsetups++;
        m->gamma_setup = gamma;
        m->nst_setup   = m->nst;
        m->force_setup = false;
        crate          = 1.0;
      }
    }
    // linear solve (I - gamma J) del = res to ||r||_WRMS <= epslin
    const double bnrm = N_VWrmsNorm_Sts(m->res, m->ewt);
    if (bnrm <= epslin) N_VConst_Sts(0.0, m->del);
    else
    {
      STS_SUNLinSolSetATimes(m->LS, m, ark_atimes);
      STS_SUNLinSolSetPreconditioner(m->LS, m->psolve ? m : nullptr, m->psolve ? ark_psolve : nullptr);
      const int lrc = STS_SUNLinSolSolve(m->LS, m->del, m->res, epslin / bnrm);
      STS_SUNLinSolSetATimes(m->LS, nullptr, nullptr);
      STS_SUNLinSolSetPreconditioner(m->LS, nullptr, nullptr);
      m->nli += STS_SUNLinSolNumIters(m->LS);
      if (lrc < 0) return -1;
      if (lrc > 0) m->nlcf++; // not within maxl iterations: the iterate is used (residual reduced)
    }
    m->nni++;
    N_VLinearSum_Sts(1.0, m->z, 1.0, m->del, m->z);
    const double del = N_VWrmsNorm_Sts(m->del, m->ewt);
    if (m->linear) break;
    if (it > 0) crate = fmax(CRDOWN * crate, del / delp);
    const double dcon = del * fmin(1.0, crate) / NLSCOEF;
    if (dcon <= 1.0) break;
    if (it + 1 >= MAXCOR || (it >= 1 && del > RDIV * delp) || !(del == del)) return 1;
    delp = del;
  }
  const int frc = rhs(m, ti, m->z, m->F[i]);
  if (frc < 0) return -1;
  return frc > 0 ? 2 : 0;
}

// one step attempt of size h from (t, y); stage derivatives into F
static int attempt(ARKStepMem* m, double h)
{
  const Table& T = m->T;
  const int s    = T.s;
  std::vector<double> cf(s + 1);
  std::vector<N_Vector> X(s + 1);
  for (int i = 0; i < s; ++i)
  {
    const double ti  = m->t + T.c[i] * h;
    const double aii = T.A[i * s + i];
    if (i == 0 && aii == 0.0)
    { // explicit first stage: f(t_n, y_n), once per step start
      if (!m->fn_current)
      {
        const int frc = rhs(m, m->t, m->y, m->Fn);
        if (frc < 0) return -1;
        if (frc > 0) return 2;
        m->fn_current = true;
      }
      N_VScale_Sts(1.0, m->Fn, m->F[0]);
      continue;
    }
    // sdata = y + h sum_{j<i} A_ij F_j
    cf[0] = 1.0;
    X[0]  = m->y;
    for (int j = 0; j < i; ++j)
    {
      cf[j + 1] = h * T.A[i * s + j];
      X[j + 1]  = m->F[j];
    }
    N_VLinearCombination_Sts(i + 1, cf.data(), X.data(), m->sdata);
    if (aii == 0.0)
    { // explicit stage
      const int frc = rhs(m, ti, m->sdata, m->F[i]);
      if (frc < 0) return -1;
      if (frc > 0) return 2;
      continue;
    }
    const int rc = solve_stage(m, i, ti, h * aii);
    if (rc != 0) return rc;
  }
  return 0;
}

static double ark_controller(ARKStepMem* m, double h, double dsm, double hp)
{
  return sts_controller_estimate(m->controller, h, dsm, m->ep1, m->ep2, hp, m->nhist, (double)(m->T.p + 1));
}

// step loop: NORMAL mode until t >= tout, ONE_STEP mode one step; steps clipped only at `clip`
// (the stop time or +inf)
static int ark_evolve(ARKStepMem* m, double tout, double clip, int itask)
{
  const int s = m->T.s;
  if (!m->initialized)
  {
    m->hnext       = (m->hfixed > 0.0) ? m->hfixed : 0.0;
    m->initialized = true;
    m->fn_current  = false;
  }
  std::vector<double> cf(s + 1);
  std::vector<N_Vector> X(s + 1);
  long long nsteps_call = 0;
  int ret               = STS_SUCCESS;
  const double target   = tout < clip ? tout : clip; // initial-step distance
  while (m->t < clip && (itask == STS_ONE_STEP || m->t < tout))
  {
    if (nsteps_call >= (m->maxsteps > 0 ? m->maxsteps : 500))
    {
      ret = STS_TOO_MUCH_WORK;
      break;
    }
    compute_ewt(m, m->y);
    if (!(m->hnext > 0.0))
    { // initial step (Hairer, Norsett & Wanner II.4) from f(t_0, y_0), no stability cap
      if (!m->fn_current)
      {
        if (rhs(m, m->t, m->y, m->Fn) != 0)
        {
          sts_set_error("ARKStep: RHS failure at the initial state");
          return STS_RHSFUNC_FAIL;
        }
        m->fn_current = true;
      }
      const double tdist = target - m->t;
      const double d0    = N_VWrmsNorm_Sts(m->y, m->ewt);
      const double d1    = N_VWrmsNorm_Sts(m->Fn, m->ewt);
      double h0          = (d0 < 1.0e-5 || d1 < 1.0e-5) ? 1.0e-6 : 0.01 * (d0 / d1);
      if (h0 > tdist) h0 = tdist;
      N_VLinearSum_Sts(h0, m->Fn, 1.0, m->y, m->tmp2);
      if (rhs(m, m->t + h0, m->tmp2, m->tmp) != 0) return STS_RHSFUNC_FAIL;
      N_VLinearSum_Sts(1.0, m->tmp, -1.0, m->Fn, m->tmp);
      const double d2   = N_VWrmsNorm_Sts(m->tmp, m->ewt) / h0;
      const double dm   = d1 > d2 ? d1 : d2;
      const double ordv = (double)(m->T.p + 1);
      double h1         = (dm <= 1.0e-15) ? fmax(1.0e-6, h0 * 1.0e-3) : stsm::pow(0.01 / dm, 1.0 / ordv);
      if (!(h1 > 0.0) || !(h1 < INFINITY)) h1 = h0;
      double hh = (100.0 * h0 < h1) ? 100.0 * h0 : h1;
      if (hh > tdist) hh = tdist;
      if (!(hh > 0.0))
      {
        sts_set_error("ARKStep: no usable initial step (non-finite state)");
        return STS_ERR_FAILURE;
      }
      m->hnext = hh;
      m->h0u   = hh;
    }
    int nef = 0, ncf = 0;
    for (;;)
    {
      double h     = m->hnext;
      bool clipped = false;
      if (m->t + h >= clip)
      {
        h       = clip - m->t;
        clipped = true;
      }
      m->nst_att++;
      m->interp_ready = false; // the attempt overwrites F[0]
      const int rc    = attempt(m, h);
      if (rc < 0) return STS_ERR_FAILURE;
      if (rc == 1 || rc == 2)
      { // Newton failure or recoverable RHS failure: retry with a quarter step
        if (rc == 1)
        {
          m->ncfn++;
          m->nnf++;
        }
        if (m->hfixed > 0.0 || ++ncf > MAXNCF)
        {
          sts_set_error("ARKStep: %s at t = %g",
                        rc == 1 ? "the Newton iteration failed to converge" : "repeated recoverable RHS failures",
                        m->t);
          return rc == 1 ? STS_CONV_FAILURE : STS_RHSFUNC_FAIL;
        }
        m->hnext       = ETACF * h;
        m->after_fail  = true;
        m->force_setup = true;
        continue;
      }
      // error estimate h sum (b_i - d_i) F_i and the new state y + h sum b_i F_i
      for (int i = 0; i < s; ++i)
      {
        cf[i] = h * (m->T.b[i] - m->T.d[i]);
        X[i]  = m->F[i];
      }
      N_VLinearCombination_Sts(s, cf.data(), X.data(), m->tmp);
      const double dsm = N_VWrmsNorm_Sts(m->tmp, m->ewt);
      if (m->hfixed > 0.0 || dsm <= 1.0)
      {
        cf[0] = 1.0;
        X[0]  = m->y;
        for (int i = 0; i < s; ++i)
        {
          cf[i + 1] = h * m->T.b[i];
          X[i + 1]  = m->F[i];
        }
        N_VLinearCombination_Sts(s + 1, cf.data(), X.data(), m->ynew);
        std::swap(m->y, m->ynew); // y_{n+1}; y_n stays in ynew for the dense output
        m->interp_ready    = true;
        m->t               = clipped ? clip : m->t + h;
        m->fn_current      = false;
        const double hprev = m->hlast;
        m->hlast           = h;
        if (m->hfixed > 0.0) m->hnext = m->hfixed;
        else
        {
          double hn  = ark_controller(m, h, dsm, hprev);
          double eta = SAFETY * hn / h;
          double emx = (m->nst == 0) ? ETAMX1 : (m->after_fail ? 1.0 : GROWTH);
          if (eta > emx) eta = emx;
          if (eta >= LBOUND && eta <= UBOUND) eta = 1.0;
          m->hnext = h * eta;
          m->ep2   = m->ep1;
          m->ep1   = dsm;
          m->nhist++;
        }
        m->after_fail = false;
        m->nst++;
        nsteps_call++;
        break;
      }
      m->netf++;
      nef++;
      if (!(dsm == dsm) || nef > MAXNEF)
      {
        sts_set_error("ARKStep: error test failed %d times at t = %g", nef, m->t);
        return STS_ERR_FAILURE;
      }
      double hn  = ark_controller(m, h, dsm, m->hlast);
      double eta = SAFETY * hn / h;
      if (eta > 1.0) eta = 1.0;
      if (nef >= SMALL_NEF && eta > ETAMXF) eta = ETAMXF;
      if (eta < ETAMIN) eta = ETAMIN;
      m->hnext      = h * eta;
      m->after_fail = true;
    }
    if (itask == STS_ONE_STEP) break;
  }
  return ret;
}

// ---------------------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------------------
#define CHECK_ARK(mem)                                                   \
  do                                                                     \
  {                                                                      \
    if (!(mem) || sts_mem_kind(mem) != STS_MEM_ARKSTEP)                  \
    {                                                                    \
      sts_set_error("ARKStep: NULL or non-ARKStep integrator memory");   \
      return STS_MEM_NULL;                                               \
    }                                                                    \
  } while (0)

extern "C" void* STS_ARKStepCreate(STS_ARKRhsFn fe, STS_ARKRhsFn fi, double t0, N_Vector y0, STS_Context ctx)
{
  if (!y0 || !ctx || (!fe == !fi))
  {
    sts_set_error("ARKStepCreate: give exactly one of fe (explicit) and fi (implicit), a vector and a context");
    return nullptr;
  }
  ARKStepMem* m = new ARKStepMem();
  m->ctx        = ctx;
  m->implicit   = fi != nullptr;
  m->f          = fi ? fi : fe;
  m->order      = m->implicit ? 3 : 4; // ARKODE's default orders
  m->table_ok   = make_table(m->implicit, m->order, &m->T);
  m->t          = t0;
  m->n          = NVL(y0);
  m->y          = N_VClone_Sts(y0);
  N_VScale_Sts(1.0, y0, m->y);
  for (N_Vector* v : {&m->Fn, &m->sdata, &m->z, &m->res, &m->del, &m->ewt, &m->tmp, &m->tmp2, &m->ynew})
    *v = N_VClone_Sts(y0);
  return m;
}

extern "C" int STS_ARKodeSetOrder(void* mem, int order)
{
  CHECK_ARK(mem);
  ARKStepMem* m = AM(mem);
  Table T;
  if (!make_table(m->implicit, order, &T))
  {
    sts_set_error("ARKodeSetOrder: no %s table of order %d (implicit 2-3, explicit 2-4)",
                  m->implicit ? "implicit" : "explicit", order);
    return STS_ILL_INPUT;
  }
  m->order = order;
  m->T     = T;
  return 0;
}

extern "C" int STS_ARKodeSetLinearSolver(void* mem, void* LS, void* A)
{
  (void)A;
  CHECK_ARK(mem);
  AM(mem)->LS = LS;
  return LS ? 0 : STS_ILL_INPUT;
}

extern "C" int STS_ARKodeSetPreconditioner(void* mem, STS_ARKLsPrecSetupFn psetup, STS_ARKLsPrecSolveFn psolve)
{
  CHECK_ARK(mem);
  AM(mem)->psetup = psetup;
  AM(mem)->psolve = psolve;
  return 0;
}

extern "C" int STS_ARKStepSetPrecData(void* mem, void* pdata)
{
  CHECK_ARK(mem);
  AM(mem)->pdata = pdata;
  return 0;
}

extern "C" int STS_ARKodeSetLSetupFrequency(void* mem, int msbp)
{
  CHECK_ARK(mem);
  if (msbp < 0) return STS_ILL_INPUT;
  AM(mem)->msbp = msbp;
  return 0;
}

extern "C" int STS_ARKodeSetEpsLin(void* mem, double eplifac)
{
  CHECK_ARK(mem);
  if (eplifac < 0.0) return STS_ILL_INPUT;
  AM(mem)->eplifac = eplifac > 0.0 ? eplifac : 0.05;
  return 0;
}

extern "C" int STS_ARKodeSetLinear(void* mem, int timedepend)
{
  (void)timedepend;
  CHECK_ARK(mem);
  AM(mem)->linear = true;
  return 0;
}

extern "C" int STS_ARKodeSetNonlinear(void* mem)
{
  CHECK_ARK(mem);
  AM(mem)->linear = false;
  return 0;
}

extern "C" int STS_ARKStepGetStats(void* mem, STS_ARKStepStats* st)
{
  CHECK_ARK(mem);
  if (!st) return STS_ILL_INPUT;
  ARKStepMem* m    = AM(mem);
  st->nst          = m->nst;
  st->nst_attempts = m->nst_att;
  st->netf         = m->netf;
  st->ncfn         = m->ncfn;
  st->nfe          = m->nfe;
  st->nfi          = m->nfi;
  st->nfe_ls       = m->nfe_dq;
  st->nni          = m->nni;
  st->nnf          = m->nnf;
  st->nli          = m->nli;
  st->nlcf         = m->nlcf;
  st->npe          = m->npe;
  st->nps          = m->nps;
  st->njv          = m->njv;
  st->nsetups      = m->nsetups;
  st->t            = m->t;
  st->h0           = m->h0u;
  st->hlast        = m->hlast;
  st->hnext        = m->hnext;
  return 0;
}

// ---- the ARKode* calls of lsrk.cu dispatch here for an ARKStep memory ----
int arkstep_sstolerances(void* mem, double rtol, double atol)
{
  if (!(rtol >= 0.0) || !(atol >= 0.0)) return STS_ILL_INPUT;
  AM(mem)->rtol = rtol;
  AM(mem)->atol = atol;
  return 0;
}
int arkstep_set_user_data(void* mem, void* ud)
{
  AM(mem)->user_data = ud;
  return 0;
}
int arkstep_set_controller(void* mem, int c)
{
  if (c < STS_ADAPT_PID || c > STS_ADAPT_IMEX_GUS) return STS_ILL_INPUT;
  AM(mem)->controller = c;
  return 0;
}
int arkstep_set_fixed_step(void* mem, double h)
{
  AM(mem)->hfixed = h;
  if (h > 0.0) AM(mem)->hnext = h;
  return 0;
}
int arkstep_set_max_steps(void* mem, long long mx)
{
  AM(mem)->maxsteps = mx;
  return 0;
}
int arkstep_set_stop_time(void* mem, double ts)
{
  AM(mem)->tstop    = ts;
  AM(mem)->tstopset = true;
  return 0;
}

// dense output at tq on the last step (the Hermite rule of sts_hermite, degree min(q - 1, 5));
// f(t_n, y_n) is evaluated here when no step start has (counted like any RHS evaluation) and
// then serves the next step's explicit first stage
static int ark_output(ARKStepMem* m, N_Vector yout, double tq, bool interp)
{
  if (!interp || tq == m->t)
  {
    N_VScale_Sts(1.0, m->y, yout);
    return 0;
  }
  const double tfuzz = 100.0 * DBL_EPSILON * (fabs(m->t) + fabs(m->hlast));
  if (tq < m->t - m->hlast - tfuzz)
  {
    sts_set_error("ARKodeEvolve: tout = %g is behind the last step [%g, %g]", tq, m->t - m->hlast, m->t);
    return STS_ILL_INPUT;
  }
  const int deg = m->T.q - 1 < 5 ? m->T.q - 1 : 5;
  if (deg >= 2 && !m->fn_current)
  {
    const int frc = rhs(m, m->t, m->y, m->Fn);
    if (frc != 0)
    {
      sts_set_error("ARKStep: RHS failure in the dense output at t = %g", m->t);
      return STS_RHSFUNC_FAIL;
    }
    m->fn_current = true;
  }
  sts_hermite(m->ctx, m->n, deg, (tq - m->t) / m->hlast, m->hlast, NVD(m->ynew), NVD(m->y), NVD(m->F[0]),
              NVD(m->Fn), NVD(yout));
  return STS_CUDA_OK(cudaGetLastError()) ? 0 : STS_ERR_FAILURE;
}

int arkstep_evolve(void* mem, double tout, N_Vector yout, double* tret, int itask)
{
  ARKStepMem* m = AM(mem);
  if (!yout || NVL(yout) != m->n) return STS_ILL_INPUT;
  if (!m->table_ok)
  {
    sts_set_error("ARKStep: no method table");
    return STS_ILL_INPUT;
  }
  if (m->implicit && !m->LS)
  {
    sts_set_error("ARKStep: an implicit method needs a linear solver (ARKodeSetLinearSolver)");
    return STS_ILL_INPUT;
  }
  ctx_activate(m->ctx);
  while ((int)m->F.size() < m->T.s) m->F.push_back(N_VClone_Sts(m->y));
  auto finish = [&](int ret, double tr) {
    if (!STS_CUDA_OK(cudaStreamSynchronize(m->ctx->stream))) return (int)STS_ERR_FAILURE;
    if (tret) *tret = tr;
    m->tretlast = tr;
    return ret;
  };
  // the return rules of STS_ARKodeEvolve (lsrk.cu)
  if (m->interp_ready && itask != STS_ONE_STEP && m->t >= tout)
  {
    const int rc = ark_output(m, yout, tout, true);
    return rc ? rc : finish(STS_SUCCESS, tout);
  }
  if (m->interp_ready && itask == STS_ONE_STEP && m->t != m->tretlast)
  {
    ark_output(m, yout, m->t, false);
    return finish(STS_SUCCESS, m->t);
  }
  if (m->tstopset && m->t >= m->tstop)
  {
    m->tstopset = false;
    ark_output(m, yout, m->t, false);
    return finish(STS_TSTOP_RETURN, m->t);
  }
  int ret     = ark_evolve(m, tout, m->tstopset ? m->tstop : INFINITY, itask);
  double tr   = m->t;
  bool interp = false;
  if (m->tstopset && m->t >= m->tstop)
  {
    m->tstopset = false;
    if (ret == STS_SUCCESS) ret = STS_TSTOP_RETURN;
  }
  else if (ret == STS_SUCCESS && itask != STS_ONE_STEP && m->t >= tout)
  {
    interp = true;
    tr     = tout;
  }
  const int rc = ark_output(m, yout, tr, interp);
  if (rc) return rc;
  return finish(ret, tr);
}

int arkstep_reset(void* mem, double t, N_Vector y)
{
  ARKStepMem* m = AM(mem);
  if (!y || NVL(y) != m->n) return STS_ILL_INPUT;
  ctx_activate(m->ctx);
  m->t            = t;
  m->tretlast     = t;
  m->interp_ready = false;
  m->fn_current   = false;
  N_VScale_Sts(1.0, y, m->y);
  return 0;
}

int arkstep_get_stats(void* mem, STS_Stats* s)
{
  ARKStepMem* m      = AM(mem);
  s->nst             = m->nst;
  s->nst_attempts    = m->nst_att;
  s->netf            = m->netf;
  s->nfe             = m->nfe + m->nfi;
  s->nfe_dee         = 0;
  s->ndee            = 0;
  s->nst_exp         = 0;
  s->stage_max       = m->T.s;
  s->stages_total    = m->nst_att * (long long)m->T.s;
  s->t               = m->t;
  s->hlast           = m->hlast;
  s->hnext           = m->hnext;
  s->spectral_radius = 0.0;
  return 0;
}

// ARKodePrintAllStats in SUNDIALS' table format (the labels runtests-diffusion2d.py parses)
int arkstep_print_stats(void* mem, char* buf, int buflen)
{
  ARKStepMem* m    = AM(mem);
  const double nni = m->nni > 0 ? (double)m->nni : 1.0;
  const int w      = snprintf(buf, (size_t)buflen,
                              "Current time                  = %.17g\n"
                              "Steps                         = %lld\n"
                              "Step attempts                 = %lld\n"
                              "Stability limited steps       = 0\n"
                              "Accuracy limited steps        = %lld\n"
                              "Error test fails              = %lld\n"
                              "NLS step fails                = %lld\n"
                              "Inequality constraint fails   = 0\n"
                              "Initial step size             = %.17g\n"
                              "Last step size                = %.17g\n"
                              "Current step size             = %.17g\n"
                              "Explicit RHS fn evals         = %lld\n"
                              "Implicit RHS fn evals         = %lld\n"
                              "NLS iters                     = %lld\n"
                              "NLS fails                     = %lld\n"
                              "NLS iters per step            = %.17g\n"
                              "LS setups                     = %lld\n"
                              "Jac fn evals                  = 0\n"
                              "LS RHS fn evals               = %lld\n"
                              "Prec setup evals              = %lld\n"
                              "Prec solves                   = %lld\n"
                              "LS iters                      = %lld\n"
                              "LS fails                      = %lld\n"
                              "Jac-times setups              = 0\n"
                              "Jac-times evals               = %lld\n"
                              "LS iters per NLS iter         = %.17g\n"
                              "Jac evals per NLS iter        = 0\n"
                              "Prec evals per NLS iter       = %.17g\n",
                              m->t, m->nst, m->nst_att, m->nst_att, m->netf, m->ncfn, m->h0u, m->hlast, m->hnext,
                              m->nfe, m->nfi, m->nni, m->nnf, m->nst > 0 ? (double)m->nni / (double)m->nst : 0.0,
                              m->nsetups, m->nfe_dq, m->npe, m->nps, m->nli, m->nlcf, m->njv, (double)m->nli / nni,
                              (double)m->npe / nni);
  return (w < 0 || w >= buflen) ? -1 : 0;
}

void arkstep_free(void* mem)
{
  ARKStepMem* m = AM(mem);
  ctx_activate(m->ctx);
  cudaStreamSynchronize(m->ctx->stream);
  for (N_Vector v : {m->y, m->Fn, m->sdata, m->z, m->res, m->del, m->ewt, m->tmp, m->tmp2, m->ynew})
    if (v) N_VDestroy_Sts(v);
  for (N_Vector v : m->F) N_VDestroy_Sts(v);
  delete m;
}

// host helper: the method table an ARKStep of this kind and order uses
extern "C" int STS_ARKStepTable(int implicit, int order, int* s, int* q, int* p, double* A, double* b, double* d,
                                double* c)
{
  Table T;
  if (!s || !q || !p || !make_table(implicit != 0, order, &T)) return -1;
  *s = T.s;
  *q = T.q;
  *p = T.p;
  if (A) memcpy(A, T.A.data(), sizeof(double) * T.s * T.s);
  if (b) memcpy(b, T.b.data(), sizeof(double) * T.s);
  if (d) memcpy(d, T.d.data(), sizeof(double) * T.s);
  if (c) memcpy(c, T.c.data(), sizeof(double) * T.s);
  return 0;
}
