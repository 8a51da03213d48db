// LSRKStep super-time-stepping integrator (RKC2 / RKL2) with ARKODE-style step control.
//
// Replaces the SUNDIALS objects the reference driver builds in diffusion_2D/main.cpp:257-400
// and advances with ARKodeEvolve (main.cpp:442). Two execution paths:
//   fused   - RHS is STS_Diffusion on an STS_Problem: one fused stencil+stage kernel per
//             stage, a fused step-end kernel (F(y_{n+1}) + error estimate + exact WRMS), the
//             stage loop of each distinct stage count captured once in a CUDA graph;
//             optionally FP32 stage increments relative to the FP64 step start;
//   generic - any other ARKRhsFn: stages through the user callback and N_Vector ops.
// Step control runs on the host after one device sync per step (the WRMS lands in mapped
// pinned memory). Constants and formulas are restated from the RKC/RKL2 papers and the
// ARKODE documentation (SUNDIALS itself is an empty submodule in the reference tree):
//   stage count   RKC: s = max(2, 1 + floor(sqrt(1 + 1.54 h rho)))  (rkc.f)
//                 RKL: s = max(2, ceil((sqrt(9 + 8 h rho) - 1)/2))
//   stage cap     h <= 0.96 (smax^2-1)/(1.54 rho) (RKC), 0.96 (smax^2+smax-2)/(2 rho) (RKL)
//   controllers   PID (0.58, 0.21, 0.1), PI (0.8, 0.31), I (1.0), error bias 1.5, order 3
//   step limits   safety 0.96, growth 20 (10^4 on the first step, 1 after a failure),
//                 eta in [1, 1.5] -> 1, failures: eta <= 1, <= 0.3 after 2, >= 0.1
//   spectral radius = 1.01 |lambda|, refreshed every 25 accepted steps (0: computed once)
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <vector>

#include "kernels.cuh"
#include "stage_tma.cuh"
#include "portable_math.cuh"
#include "sts_internal.cuh"

void sts_f64_to_f32(STS_Context ctx, const double* a, float* b, long long n);

// ---------------------------------------------------------------------------------------
// coefficient and step-size rules (host)
// ---------------------------------------------------------------------------------------
extern "C" int STS_LSRKStageCoeffs(int method, int s, double* mu, double* nu, double* mus, double* ajm1,
                                   double* cjm1)
{
  if (s < 2) return -1;
  if (method == STS_LSRK_RKC_2)
  {
    const double sd    = (double)s;
    const double w0    = 1.0 + 2.0 / (13.0 * (sd * sd));
    const double temp1 = w0 * w0 - 1.0;
    const double temp2 = sqrt(temp1);
    const double arg   = sd * log(w0 + temp2);
    const double w1    = sinh(arg) * temp1 / (cosh(arg) * sd * temp2 - w0 * sinh(arg));
    double bjm1        = 1.0 / ((2.0 * w0) * (2.0 * w0));
    double bjm2        = bjm1;
    mu[1]              = 0.0;
    nu[1]              = 0.0;
    mus[1]             = w1 * bjm1;
    ajm1[1]            = 0.0;
    cjm1[1]            = 0.0;
    double thjm2 = 0.0, thjm1 = mus[1];
    double zjm1 = w0, zjm2 = 1.0, dzjm1 = 1.0, dzjm2 = 0.0, d2zjm1 = 0.0, d2zjm2 = 0.0;
    for (int j = 2; j <= s; ++j)
    {
      const double zj   = 2.0 * w0 * zjm1 - zjm2;
      const double dzj  = 2.0 * w0 * dzjm1 - dzjm2 + 2.0 * zjm1;
      const double d2zj = 2.0 * w0 * d2zjm1 - d2zjm2 + 4.0 * dzjm1;
      const double bj   = d2zj / (dzj * dzj);
      const double a    = 1.0 - zjm1 * bjm1;
      const double m    = 2.0 * w0 * bj / bjm1;
      const double n    = -bj / bjm2;
      const double ms   = m * w1 / w0;
      mu[j]             = m;
      nu[j]             = n;
      mus[j]            = ms;
      ajm1[j]           = a;
      cjm1[j]           = thjm1;
      const double thj  = m * thjm1 + n * thjm2 + ms * (1.0 - a);
      thjm2             = thjm1;
      thjm1             = thj;
      bjm2              = bjm1;
      bjm1              = bj;
      zjm2              = zjm1;
      zjm1              = zj;
      dzjm2             = dzjm1;
      dzjm1             = dzj;
      d2zjm2            = d2zjm1;
      d2zjm1            = d2zj;
    }
  }
  else if (method == STS_LSRK_RKL_2)
  {
    const double sd = (double)s;
    const double w1 = 4.0 / ((sd + 2.0) * (sd - 1.0));
    double bjm2 = 1.0 / 3.0, bjm1 = 1.0 / 3.0;
    mu[1]      = 0.0;
    nu[1]      = 0.0;
    mus[1]     = w1 * bjm1;
    ajm1[1]    = 0.0;
    cjm1[1]    = 0.0;
    double cj1 = mus[1];
    for (int j = 2; j <= s; ++j)
    {
      const double jd   = (double)j;
      const double temj = (jd + 2.0) * (jd - 1.0);
      const double cj   = temj * w1 / 4.0;
      const double bj   = temj / (2.0 * jd * (jd + 1.0));
      const double a    = 1.0 - bjm1;
      const double m    = (2.0 * jd - 1.0) / jd * (bj / bjm1);
      const double n    = -(jd - 1.0) / jd * (bj / bjm2);
      mu[j]             = m;
      nu[j]             = n;
      mus[j]            = w1 * m;
      ajm1[j]           = a;
      cjm1[j]           = cj1;
      cj1               = cj;
      bjm2              = bjm1;
      bjm1              = bj;
    }
  }
  else return -1;
  return 0;
}

extern "C" int STS_LSRKStagesNeeded(int method, double h, double rho, int smax, double* hmax)
{
  double ss;
  const double sm = (double)smax;
  if (method == STS_LSRK_RKC_2)
  {
    ss    = 1.0 + floor(sqrt(1.0 + 1.54 * h * rho));
    *hmax = (rho > 0.0) ? 0.96 * (sm * sm - 1.0) / (1.54 * rho) : INFINITY;
  }
  else
  {
    ss    = ceil((sqrt(9.0 + 8.0 * h * rho) - 1.0) / 2.0);
    *hmax = (rho > 0.0) ? 0.96 * (sm * sm + sm - 2.0) / (2.0 * rho) : INFINITY;
  }
  // a non-finite step (NaN state) gives the 2-stage minimum, as max(ss, 2) does
  if (!(ss >= 2.0)) ss = 2.0;
  if (ss > 1e9) ss = 1e9;
  return (int)ss;
}

static constexpr double ORD = 3.0, BIAS = 1.5, TINYE = 1.0e-10;
static double controller_estimate(int controller, double h, double dsm, double ep1, double ep2, double hp,
                                  long long nhist, double ORD);
double sts_controller_estimate(int controller, double h, double dsm, double ep1, double ep2, double hp,
                               long long nhist, double ord)
{
  return controller_estimate(controller, h, dsm, ep1, ep2, hp, nhist, ord);
}
extern "C" double STS_AdaptControllerEstimate(int controller, double h, double dsm, double ep1, double ep2,
                                              double hp, long long nhist)
{
  return controller_estimate(controller, h, dsm, ep1, ep2, hp, nhist, ORD);
}

// The controllers of diffusion_2D/main.cpp:366-376 for an error estimate of order ORD (3 for
// the STS methods' embedding); e = bias * dsm floored at 1e-10, hp = previous accepted step.
//   PID / PI / I: Soderlind-form exponents, leading terms only until enough history exists
//   ExpGus  (Gustafsson 1991): h e_n^(-k1/p) (e_n/e_{n-1})^(-k2/p), k1 0.367, k2 0.268
//   ImpGus  (Gustafsson 1994): h (h/h_{n-1}) e_n^(-k1/p) (e_n/e_{n-1})^(-k2/p), k1 0.98, k2 0.95
//   ImExGus: the smaller of the two; all three use h e_n^(-1/p) on the first step.
static double controller_estimate(int controller, double h, double dsm, double ep1, double ep2, double hp,
                                  long long nhist, double ORD)
{
  double e1 = BIAS * dsm;
  if (e1 < TINYE) e1 = TINYE;
  double e2 = BIAS * ep1;
  if (e2 < TINYE) e2 = TINYE;
  double e3 = BIAS * ep2;
  if (e3 < TINYE) e3 = TINYE;
  if (controller == STS_ADAPT_PID)
  {
    if (nhist < 1) return h * stsm::pow(e1, -0.58 / ORD);
    if (nhist < 2) return h * stsm::pow(e1, -0.58 / ORD) * stsm::pow(e2, 0.21 / ORD);
    return h * stsm::pow(e1, -0.58 / ORD) * stsm::pow(e2, 0.21 / ORD) * stsm::pow(e3, -0.1 / ORD);
  }
  if (controller == STS_ADAPT_PI)
  {
    if (nhist < 1) return h * stsm::pow(e1, -0.8 / ORD);
    return h * stsm::pow(e1, -0.8 / ORD) * stsm::pow(e2, 0.31 / ORD);
  }
  if (controller >= STS_ADAPT_EXP_GUS && controller <= STS_ADAPT_IMEX_GUS && nhist >= 1 && hp > 0.0)
  {
    const double r    = e1 / e2;
    const double hexp = h * stsm::pow(e1, -0.367 / ORD) * stsm::pow(r, -0.268 / ORD);
    if (controller == STS_ADAPT_EXP_GUS) return hexp;
    const double himp = h * (h / hp) * stsm::pow(e1, -0.98 / ORD) * stsm::pow(r, -0.95 / ORD);
    if (controller == STS_ADAPT_IMP_GUS) return himp;
    return hexp < himp ? hexp : himp;
  }
  return h * stsm::pow(e1, -1.0 / ORD);
}

static constexpr double SAFETY = 0.96, GROWTH = 20.0, ETAMX1 = 10000.0, ETAMXF = 0.3, ETAMIN = 0.1;
static constexpr double LBOUND = 1.0, UBOUND = 1.5;
static constexpr int SMALL_NEF = 2;

// ---------------------------------------------------------------------------------------
// integrator memory
// ---------------------------------------------------------------------------------------
struct GraphKey {
  int s, parity;
  bool operator<(const GraphKey& o) const { return s != o.s ? s < o.s : parity < o.parity; }
};

struct LSRKMem {
  uint32_t kind         = STS_MEM_LSRK; // first member: the ARKode* calls dispatch on it
  STS_Context ctx       = nullptr;
  STS_ARKRhsFn rhs      = nullptr;
  void* user_data       = nullptr;
  STS_ARKDomEigFn domeig = nullptr;
  bool power            = false;
  int dee_maxiters      = 100;
  int dee_init_warmups  = 0; // power iterations before the first estimate
  int dee_succ_warmups  = 0; // power iterations before each later estimate
  double dee_reltol     = 0.01;
  int method            = STS_LSRK_RKC_2;
  double ord            = 3.0; // order of the error estimate seen by the controller
  // SSP methods (LSRKStepCreateSSP): stage count and the error weights h (b_j - bhat_j)
  bool ssp              = false;
  int ssp_stages        = 10;
  bool use_fused_periodic = true; // reference mode: fused stage / step-end kernels (same bits)
  std::vector<double> ssp_w, ssp_c; // error weights b - bhat, stage times
  int controller        = STS_ADAPT_PID;
  int smax              = 200;
  double rtol = 1e-4, atol = 1e-9; // ARKODE defaults until SStolerances is called
  double hfixed         = 0.0;
  double eig_safety     = 1.01;
  long long dom_eig_freq = 25;
  long long maxsteps    = 500;
  double tstop          = INFINITY;
  bool tstopset         = false; // ARKodeSetStopTime: cleared when the stop time is returned
  bool mixed            = false;
  bool use_graphs       = true;
  int stage_variant     = 0; // 0: autotuned (TMA configurations + register kernel), 1: register marching
  TmaStage32 tma;
  int tma_variant       = -1; // chosen TMA configuration (-1: register-marching kernel)
  bool tuned            = false;
  double tune_ms[TMA_STAGE32_NVARIANTS + 1] = {};
  // fused stages: requested group size (0: autotuned, 1: off, 2..4) and tile configuration
  // (-1: autotuned); the chosen ones (fuse_ks 1: single-stage launches) and the time per
  // launch of each tile configuration at 4 stages
  int fuse_req = 0, fuse_tile_req = -1;
  int fuse_ks = 1, fuse_ti = -1;
  double fuse_ms[TMA_FUSED_NTILES] = {};
  long long n           = 0;

  // state (mirrors the oracle's orc_state)
  double t = 0, hnext = 0, hlast = 0, rho = 0, ep1 = 0, ep2 = 0;
  long long ncf = 0;
  long long nst = 0, nst_att = 0, netf = 0, nfe = 0, nfe_dee = 0, ndee = 0, nst_exp = 0, stage_max = 0,
            stages_total = 0, nhist = 0, steps_since_dee = -1;
  bool initialized = false, after_fail = false;
  int last_s = 0;
  // dense output: the last accepted step's y_old (and f_old) are still held (fused: the other
  // parity buffer; generic: g_yold / g_Fold); tretlast = the time last returned to the caller
  bool interp_ready = false;
  double tretlast   = 0.0;

  // device buffers
  double* yb[2] = {nullptr, nullptr}; // y_n / y_{n+1} (parity)
  double* Fb[2] = {nullptr, nullptr}; // F_n / F_{n+1}
  float* Ffb[2] = {nullptr, nullptr}; // FP32 copies (mixed)
  double* Y[3]  = {nullptr, nullptr, nullptr};
  float* D[4]   = {nullptr, nullptr, nullptr, nullptr}; // D[3]: fused stages only
  double* evec  = nullptr;
  float* per_faces = nullptr; // mixed reference mode: FP32 Dxw | Dxe | Dys | Dyn
  int par       = 0; // current parity: yb[par] = y_n
  N_Vector nv_y = nullptr, nv_F = nullptr, nv_tmp[3] = {nullptr, nullptr, nullptr};

  // stage parameters: [StepArgs][StageArgs x (smax+1)] on the device and pinned on the host
  void* d_par = nullptr;
  void* h_par = nullptr;
  size_t par_bytes = 0;
  std::map<GraphKey, cudaGraphExec_t> graphs;

  // generic path temporaries
  N_Vector g_Y[3] = {nullptr, nullptr, nullptr}, g_F = nullptr, g_Fnew = nullptr, g_err = nullptr,
           g_ewt = nullptr, g_y = nullptr, g_Fn = nullptr, g_yold = nullptr, g_Fold = nullptr;
};

static bool fused(const LSRKMem* m)
{
  return !m->ssp && m->rhs == STS_Diffusion && m->user_data != nullptr &&
         ((STS_Problem)m->user_data)->kind != STS_PROBLEM_PERIODIC;
}

// ---------------------------------------------------------------------------------------
// SSP methods of LSRKStepCreateSSP (diffusion_2D/main.cpp:250-294), restated from Ketcheson,
// "Highly efficient strong stability-preserving Runge-Kutta methods with low-storage
// implementations", SIAM J. Sci. Comput. 30 (2008):
//   SSP(s,2), s >= 2:       s-1 forward-Euler substeps of h/(s-1), then
//                           y+ = y/s + (s-1)/s (Y + h/(s-1) F(Y));
//   SSP(s,3), s = n^2 >= 4: Euler substeps of h/(n^2-n) with one convex combination
//                           (n/(2n-1)) q2 + ((n-1)/(2n-1)) (q1 + h/r F(q1)) at substep n(n+1)/2;
//   SSP(10,4):              5 substeps of h/6, q2 = q2/25 + 9 q1/25, q1 = 15 q2 - 5 q1,
//                           4 substeps, y+ = q2 + 3/5 q1 + h/10 F(q1).
// Embedded estimates (this implementation's choice; the SUNDIALS embeddings are not available
// here): SSP(s,2) the internal stage Y_s (first order: weights 1/(s-1) on the first s-1
// stage derivatives); SSP(s,3) and SSP(10,4) the weights nearest to a reference (uniform 1/s;
// for SSP(10,4), whose b is uniform, alternating 0.15 / 0.05) that satisfy the order
// conditions of order 2 (resp. 3) on the method's own stages. The error estimate is
// h sum_j (b_j - bhat_j) F_j; the controller uses order (embedding order + 1).
// ---------------------------------------------------------------------------------------
enum { SSP_S_2 = STS_LSRK_SSP_S_2, SSP_S_3 = STS_LSRK_SSP_S_3, SSP_10_4 = STS_LSRK_SSP_10_4 };

static bool ssp_stages_valid(int type, int s)
{
  if (type == SSP_S_2) return s >= 2 && s <= 1024;
  if (type == SSP_S_3)
  {
    const int n = (int)std::lround(std::sqrt((double)s));
    return n >= 2 && n * n == s && s <= 1024;
  }
  return type == SSP_10_4 && s == 10;
}

// Butcher weights of the SSP method (registers tracked as y coefficient + multiples of h F_j):
// A (s x s, row-major), b, c; and the error weights w = b - bhat
static void ssp_tableau(int type, int s, std::vector<double>& A, std::vector<double>& b, std::vector<double>& c,
                        std::vector<double>& w)
{
  struct Reg {
    double cy;
    std::vector<double> f;
  };
  // the stage matrix is only needed for the third-order conditions of SSP(10,4)
  A.assign(type == SSP_10_4 ? (size_t)s * s : 0, 0.0);
  c.assign(s, 0.0);
  int j = 0;
  auto stage = [&](const Reg& q) {
    double cj = 0.0;
    for (int k = 0; k < s; ++k)
    {
      if (type == SSP_10_4) A[(size_t)j * s + k] = q.f[k];
      cj += q.f[k];
    }
    c[j] = cj;
    return j++;
  };
  auto comb = [&](double a, const Reg& x, double bb, const Reg& y) {
    Reg r{a * x.cy + bb * y.cy, std::vector<double>(s)};
    for (int k = 0; k < s; ++k) r.f[k] = a * x.f[k] + bb * y.f[k];
    return r;
  };
  Reg q1{1.0, std::vector<double>(s, 0.0)}, q2 = q1, fin = q1;
  if (type == SSP_S_2)
  {
    const double r = s - 1.0;
    for (int i = 0; i < s - 1; ++i) q1.f[stage(q1)] += 1.0 / r;
    const int js = stage(q1);
    Reg t        = q1;
    t.f[js] += 1.0 / r;
    fin = comb(1.0 / s, Reg{1.0, std::vector<double>(s, 0.0)}, (s - 1.0) / s, t);
  }
  else if (type == SSP_S_3)
  {
    const int n    = (int)std::lround(std::sqrt((double)s));
    const double r = (double)(n * n - n);
    const int e1 = (n - 1) * (n - 2) / 2, e2 = n * (n + 1) / 2;
    for (int i = 1; i <= e1; ++i) q1.f[stage(q1)] += 1.0 / r;
    q2 = q1;
    for (int i = e1 + 1; i <= e2 - 1; ++i) q1.f[stage(q1)] += 1.0 / r;
    const int jc = stage(q1);
    Reg t        = q1;
    t.f[jc] += 1.0 / r;
    q1 = comb((double)n / (2 * n - 1), q2, (n - 1.0) / (2 * n - 1), t);
    for (int i = e2 + 1; i <= n * n; ++i) q1.f[stage(q1)] += 1.0 / r;
    fin = q1;
  }
  else
  {
    for (int i = 1; i <= 5; ++i) q1.f[stage(q1)] += 1.0 / 6.0;
    q2 = comb(1.0 / 25.0, q2, 9.0 / 25.0, q1);
    q1 = comb(15.0, q2, -5.0, q1);
    for (int i = 6; i <= 9; ++i) q1.f[stage(q1)] += 1.0 / 6.0;
    const int jl = stage(q1);
    Reg t        = q1;
    fin          = comb(1.0, q2, 3.0 / 5.0, t);
    fin.f[jl] += 1.0 / 10.0;
  }
  b = fin.f;
  std::vector<double> bh(s);
  if (type == SSP_S_2)
    for (int k = 0; k < s; ++k) bh[k] = (k < s - 1) ? 1.0 / (s - 1.0) : 0.0;
  else
  {
    // bhat = u - C^T (C C^T)^-1 (C u - d): nearest to uniform u under the order conditions
    std::vector<std::vector<double>> C;
    std::vector<double> d;
    C.push_back(std::vector<double>(s, 1.0));
    d.push_back(1.0);
    C.push_back(c);
    d.push_back(0.5);
    if (type == SSP_10_4)
    {
      std::vector<double> c2(s), Ac(s, 0.0);
      for (int k = 0; k < s; ++k)
      {
        c2[k] = c[k] * c[k];
        for (int l = 0; l < s; ++l) Ac[k] += A[(size_t)k * s + l] * c[l];
      }
      C.push_back(c2);
      d.push_back(1.0 / 3.0);
      C.push_back(Ac);
      d.push_back(1.0 / 6.0);
    }
    const int m = (int)C.size();
    // reference: uniform weights, except SSP(10,4) whose b is itself uniform: there
    // alternating 0.15 / 0.05 (its projection violates the fourth-order conditions)
    std::vector<double> u(s, 1.0 / s), res(m), G((size_t)m * m);
    if (type == SSP_10_4)
      for (int k = 0; k < s; ++k) u[k] = (k & 1) ? 0.05 : 0.15;
    for (int a = 0; a < m; ++a)
    {
      double v = 0.0;
      for (int k = 0; k < s; ++k) v += C[a][k] * u[k];
      res[a] = v - d[a];
      for (int e = 0; e < m; ++e)
      {
        double g = 0.0;
        for (int k = 0; k < s; ++k) g += C[a][k] * C[e][k];
        G[(size_t)a * m + e] = g;
      }
    }
    // solve G lam = res (Gaussian elimination with partial pivoting, m <= 4)
    std::vector<double> lam = res;
    for (int col = 0; col < m; ++col)
    {
      int pr = col;
      for (int rr = col + 1; rr < m; ++rr)
        if (std::fabs(G[(size_t)rr * m + col]) > std::fabs(G[(size_t)pr * m + col])) pr = rr;
      if (pr != col)
      {
        for (int e = 0; e < m; ++e) std::swap(G[(size_t)col * m + e], G[(size_t)pr * m + e]);
        std::swap(lam[col], lam[pr]);
      }
      for (int rr = col + 1; rr < m; ++rr)
      {
        const double f = G[(size_t)rr * m + col] / G[(size_t)col * m + col];
        for (int e = col; e < m; ++e) G[(size_t)rr * m + e] -= f * G[(size_t)col * m + e];
        lam[rr] -= f * lam[col];
      }
    }
    for (int col = m - 1; col >= 0; --col)
    {
      for (int e = col + 1; e < m; ++e) lam[col] -= G[(size_t)col * m + e] * lam[e];
      lam[col] /= G[(size_t)col * m + col];
    }
    for (int k = 0; k < s; ++k)
    {
      double v = u[k];
      for (int a = 0; a < m; ++a) v -= C[a][k] * lam[a];
      bh[k] = v;
    }
  }
  w.assign(s, 0.0);
  for (int k = 0; k < s; ++k) w[k] = b[k] - bh[k];
}

static void free_device(LSRKMem* m)
{
  for (auto& kv : m->graphs) cudaGraphExecDestroy(kv.second);
  m->graphs.clear();
  for (int b = 0; b < 2; ++b)
  {
    cudaFree(m->yb[b]);
    cudaFree(m->Fb[b]);
    cudaFree(m->Ffb[b]);
    m->yb[b] = m->Fb[b] = nullptr;
    m->Ffb[b]           = nullptr;
  }
  for (int b = 0; b < 3; ++b)
  {
    cudaFree(m->Y[b]);
    m->Y[b] = nullptr;
  }
  for (int b = 0; b < 4; ++b)
  {
    cudaFree(m->D[b]);
    m->D[b] = nullptr;
  }
  cudaFree(m->evec);
  m->evec = nullptr;
  cudaFree(m->per_faces);
  m->per_faces = nullptr;
  cudaFree(m->d_par);
  cudaFreeHost(m->h_par);
  m->d_par = m->h_par = nullptr;
  N_Vector* vs[] = {&m->nv_y, &m->nv_F, &m->nv_tmp[0], &m->nv_tmp[1], &m->nv_tmp[2], &m->g_Y[0], &m->g_Y[1],
                    &m->g_Y[2], &m->g_F, &m->g_Fnew, &m->g_err, &m->g_ewt, &m->g_y, &m->g_Fn,
                    &m->g_yold, &m->g_Fold};
  for (N_Vector* v : vs)
  {
    if (*v) N_VDestroy_Sts(*v);
    *v = nullptr;
  }
}

static StepArgs* hstep(LSRKMem* m) { return (StepArgs*)m->h_par; }
static StageArgs* hstage(LSRKMem* m) { return (StageArgs*)((char*)m->h_par + sizeof(StepArgs) + 8); }
static StepArgs* dstep(LSRKMem* m) { return (StepArgs*)m->d_par; }
static StageArgs* dstage(LSRKMem* m) { return (StageArgs*)((char*)m->d_par + sizeof(StepArgs) + 8); }

// allocate the fused-path buffers (y0 copied into yb[0])
static int alloc_fused(LSRKMem* m, const double* y0dev)
{
  const size_t n8 = m->n * sizeof(double), n4 = m->n * sizeof(float);
  cudaStream_t st = m->ctx->stream;
  for (int b = 0; b < 2; ++b)
  {
    if (!STS_CUDA_OK(cudaMalloc(&m->yb[b], n8)) || !STS_CUDA_OK(cudaMalloc(&m->Fb[b], n8)) ||
        !STS_CUDA_OK(cudaMalloc(&m->Ffb[b], n4)))
      return -1;
  }
  m->par_bytes = sizeof(StepArgs) + 8 + sizeof(StageArgs) * (size_t)(m->smax + 1);
  if (!STS_CUDA_OK(cudaMalloc(&m->d_par, m->par_bytes)) ||
      !STS_CUDA_OK(cudaHostAlloc(&m->h_par, m->par_bytes, cudaHostAllocDefault)))
    return -1;
  memset(m->h_par, 0, m->par_bytes);
  if (!STS_CUDA_OK(cudaMemcpyAsync(m->yb[0], y0dev, n8, cudaMemcpyDeviceToDevice, st))) return -1;
  m->par = 0;
  return 0;
}

static int ensure_stage_buffers(LSRKMem* m)
{
  const size_t n8 = m->n * sizeof(double), n4 = m->n * sizeof(float);
  for (int b = 0; b < 3; ++b)
  {
    if (!m->mixed && !m->Y[b] && !STS_CUDA_OK(cudaMalloc(&m->Y[b], n8))) return -1;
    if (m->mixed && !m->D[b] && !STS_CUDA_OK(cudaMalloc(&m->D[b], n4))) return -1;
  }
  // fused stages need a fourth buffer (a group reads two and writes two); the tensor maps of
  // the single-stage and the fused kernels cover every allocated buffer
  const bool want_fused = m->mixed && m->fuse_req != 1 && m->stage_variant != 1;
  if (m->mixed && m->stage_variant != 1 && (!m->tma.ok || (want_fused && !m->tma.fz_ok)))
  {
    STS_Problem p = (STS_Problem)m->user_data;
    if (tma_stage32_supported(p->nx, p->ny))
    {
      if (want_fused && !m->D[3] && !STS_CUDA_OK(cudaMalloc(&m->D[3], n4))) return -1;
      if (tma_stage32_prepare(&m->tma, m->D, m->Ffb, p->nx, p->ny) && want_fused)
        tma_fused_prepare(&m->tma, m->D, m->Ffb, p->nx, p->ny);
    }
  }
  return 0;
}

static int ensure_par(LSRKMem* m)
{
  size_t need = sizeof(StepArgs) + 8 + sizeof(StageArgs) * (size_t)(m->smax + 1);
  if (need <= m->par_bytes && m->d_par) return 0;
  for (auto& kv : m->graphs) cudaGraphExecDestroy(kv.second);
  m->graphs.clear();
  cudaFree(m->d_par);
  cudaFreeHost(m->h_par);
  m->par_bytes = need;
  if (!STS_CUDA_OK(cudaMalloc(&m->d_par, need)) || !STS_CUDA_OK(cudaHostAlloc(&m->h_par, need, cudaHostAllocDefault)))
    return -1;
  memset(m->h_par, 0, need);
  return 0;
}

// ---------------------------------------------------------------------------------------
// fused stage loop
// ---------------------------------------------------------------------------------------
// launch shapes: FP64 stage 64x4 threads, 2 columns x 8 rows per thread; FP32 stage 64x4
// threads, 4 columns x 8 rows per thread; scalar-column variants when nx is not a
// multiple of the vector width.
static constexpr int RY = 8;

template <typename F>
static void dispatch_forced(bool forced, F&& f)
{
  if (forced) f(std::true_type{});
  else f(std::false_type{});
}

static void launch_stage64(LSRKMem* m, STS_Problem p, const StageArgs* A, const double* ym1, const double* ym2,
                           const double* y0, const double* f0, double* yj)
{
  const bool forced = p->kind == STS_PROBLEM_MANUFACTURED;
  dim3 b(64, 4);
  if (p->nx % 2 == 0)
  {
    dim3 g((unsigned)((p->nx / 2 + b.x - 1) / b.x), (unsigned)((p->ny + b.y * RY - 1) / (b.y * RY)));
    dispatch_forced(forced, [&](auto F) {
      stage64_kernel<2, RY, decltype(F)::value><<<g, b, 0, m->ctx->stream>>>(p->dev, A, ym1, ym2, y0, f0, yj);
    });
  }
  else
  {
    dim3 g((unsigned)((p->nx + b.x - 1) / b.x), (unsigned)((p->ny + b.y * RY - 1) / (b.y * RY)));
    dispatch_forced(forced, [&](auto F) {
      stage64_kernel<1, RY, decltype(F)::value><<<g, b, 0, m->ctx->stream>>>(p->dev, A, ym1, ym2, y0, f0, yj);
    });
  }
}

static void launch_stage32(LSRKMem* m, STS_Problem p, const StageArgs* A, const float* dm1, const float* dm2,
                           const float* f0f, float* dj);

// mixed stage by buffer index (TMA path when prepared)
static void launch_stage32_idx(LSRKMem* m, STS_Problem p, const StageArgs* A, int im1, int im2, int par, int iout,
                               int variant)
{
  if (variant >= 0 && m->tma.ok &&
      tma_stage32_launch(&m->tma, variant, m->ctx->num_sms, p->dev, A, im1, im2, par, m->D[iout], m->ctx->d_err,
                         m->ctx->stream))
    return;
  launch_stage32(m, p, A, m->D[im1], im2 >= 0 ? m->D[im2] : nullptr, m->Ffb[par], m->D[iout]);
}

static void launch_stage32_idx(LSRKMem* m, STS_Problem p, const StageArgs* A, int im1, int im2, int par, int iout)
{
  const int v = m->stage_variant == 0 ? m->tma_variant : (m->stage_variant >= 2 ? m->stage_variant - 2 : -1);
  launch_stage32_idx(m, p, A, im1, im2, par, iout, v);
}

// Autotuner for the mixed stage kernel: times every TMA configuration and the register
// kernel on the integrator's own buffers (a realistic stage, CUDA events on the context
// stream, 2 warm + 5 timed launches each) and keeps the fastest for this problem.
static void autotune_stage32(LSRKMem* m, STS_Problem p)
{
  m->tuned       = true;
  m->tma_variant = -1;
  m->fuse_ks     = 1;
  m->fuse_ti     = -1;
  if (m->stage_variant != 0 || !m->tma.ok) return;
  cudaStream_t st = m->ctx->stream;
  // stage coefficients of a mid stage of a 100-stage RKL2 step (any finite values time alike)
  memset(m->h_par, 0, m->par_bytes);
  StageArgs* a = hstage(m) + 2;
  a->gsf = 0.01f;
  a->gxf = 0.2f;
  a->gyf = 0.05f;
  a->gmf = 0.9f;
  a->gFf = 1e-5f;
  cudaMemcpyAsync(m->d_par, m->h_par, m->par_bytes, cudaMemcpyHostToDevice, st);
  // scratch only: the stage buffers and the FP32 F of the other parity (the current one may
  // hold a restored or reset state)
  const int fpar = 1 - m->par;
  cudaMemsetAsync(m->D[0], 0, m->n * sizeof(float), st);
  cudaMemsetAsync(m->D[1], 0, m->n * sizeof(float), st);
  cudaMemsetAsync(m->Ffb[fpar], 0, m->n * sizeof(float), st);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  double best = 1e30;
  for (int v = -1; v < TMA_STAGE32_NVARIANTS; ++v)
  {
    for (int k = 0; k < 2; ++k) launch_stage32_idx(m, p, dstage(m) + 2, 0, 1, fpar, 2, v);
    cudaEventRecord(e0, st);
    for (int k = 0; k < 5; ++k) launch_stage32_idx(m, p, dstage(m) + 2, 0, 1, fpar, 2, v);
    cudaEventRecord(e1, st);
    if (cudaEventSynchronize(e1) != cudaSuccess) break;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    const double per = ms / 5.0;
    m->tune_ms[v + 1] = per;
    if (per < best)
    {
      best           = per;
      m->tma_variant = v;
    }
  }
  // fused groups of four stages, per tile configuration, against the best single stage
  m->fuse_ks = 1;
  m->fuse_ti = -1;
  if (m->tma.fz_ok && m->fuse_req != 1 && m->smax >= 5)
  {
    for (int k = 3; k <= 5; ++k) hstage(m)[k] = *a;
    cudaMemcpyAsync(m->d_par, m->h_par, m->par_bytes, cudaMemcpyHostToDevice, st);
    cudaMemsetAsync(m->D[2], 0, m->n * sizeof(float), st);
    double best_f = 1e30;
    for (int ti = 0; ti < TMA_FUSED_NTILES; ++ti)
    {
      if (m->fuse_tile_req >= 0 && ti != m->fuse_tile_req) continue;
      auto one = [&]() {
        return tma_fused_launch(&m->tma, ti, 4, m->ctx->num_sms, p->dev, dstage(m) + 2, 0, 1, fpar, m->D[2], m->D[3],
                                m->ctx->d_err, st);
      };
      bool ok = one() && one();
      cudaEventRecord(e0, st);
      for (int k = 0; k < 5 && ok; ++k) ok = one();
      cudaEventRecord(e1, st);
      if (!ok || cudaEventSynchronize(e1) != cudaSuccess) break;
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      m->fuse_ms[ti] = ms / 5.0;
      if (m->fuse_ms[ti] < best_f)
      {
        best_f     = m->fuse_ms[ti];
        m->fuse_ti = ti;
      }
    }
    if (m->fuse_ti >= 0)
    {
      if (m->fuse_req >= 2) m->fuse_ks = m->fuse_req;
      else if (best_f / 4.0 < best) m->fuse_ks = 4;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaGetLastError();
}

static void launch_stage32(LSRKMem* m, STS_Problem p, const StageArgs* A, const float* dm1, const float* dm2,
                           const float* f0f, float* dj)
{
  const bool forced = p->kind == STS_PROBLEM_MANUFACTURED;
  dim3 b(64, 4);
  auto go = [&](auto VECc) {
    constexpr int VEC = decltype(VECc)::value;
    dim3 g((unsigned)((p->nx / VEC + b.x - 1) / b.x), (unsigned)((p->ny + b.y * RY - 1) / (b.y * RY)));
    dispatch_forced(forced, [&](auto F) {
      if (dm2)
        stage32_kernel<VEC, RY, decltype(F)::value, true><<<g, b, 0, m->ctx->stream>>>(p->dev, A, dm1, dm2, f0f, dj);
      else
        stage32_kernel<VEC, RY, decltype(F)::value, false><<<g, b, 0, m->ctx->stream>>>(p->dev, A, dm1, dm2, f0f, dj);
    });
  };
  if (p->nx % 4 == 0) go(std::integral_constant<int, 4>{});
  else go(std::integral_constant<int, 1>{});
}

static void launch_stepend(LSRKMem* m, STS_Problem p, int par, const double* Ys, const float* ds)
{
  const bool forced = p->kind == STS_PROBLEM_MANUFACTURED;
  if (p->nx % 2 == 0)
  { // row-marching form: 64 x 4 threads, 2 columns x 16 rows each
    dim3 b(64, 4);
    dim3 g((unsigned)((p->nx / 2 + 63) / 64), (unsigned)((p->ny + 63) / 64));
    const int nxt = 1 - par;
    RedWork* w    = m->ctx->d_work;
    double* slot  = m->ctx->d_slots + SLOT_DSM;
    dispatch_forced(forced, [&](auto F) {
      if (m->mixed)
        stepend_march_kernel<true, decltype(F)::value><<<g, b, 0, m->ctx->stream>>>(
          p->dev, dstep(m), m->yb[par], nullptr, ds, m->Fb[par], m->yb[nxt], m->Fb[nxt], m->Ffb[nxt], w, slot);
      else
        stepend_march_kernel<false, decltype(F)::value><<<g, b, 0, m->ctx->stream>>>(
          p->dev, dstep(m), m->yb[par], Ys, nullptr, m->Fb[par], nullptr, m->Fb[nxt], nullptr, w, slot);
    });
    return;
  }
  dim3 b(256, 1);
  unsigned gx      = (unsigned)((p->nx + 255) / 256);
  long long gy_cap = std::max<long long>(1, (long long)m->ctx->num_sms * 8 / gx);
  unsigned gy      = (unsigned)std::min<long long>(p->ny, gy_cap);
  dim3 g(gx, gy);
  const int nxt = 1 - par;
  RedWork* w    = m->ctx->d_work;
  double* slot  = m->ctx->d_slots + SLOT_DSM;
  dispatch_forced(forced, [&](auto F) {
    if (m->mixed)
      stepend_kernel<true, decltype(F)::value><<<g, b, 0, m->ctx->stream>>>(
        p->dev, dstep(m), m->yb[par], nullptr, ds, m->Fb[par], m->yb[nxt], m->Fb[nxt], m->Ffb[nxt], w, slot);
    else
      stepend_kernel<false, decltype(F)::value><<<g, b, 0, m->ctx->stream>>>(
        p->dev, dstep(m), m->yb[par], Ys, nullptr, m->Fb[par], nullptr, m->Fb[nxt], nullptr, w, slot);
  });
}

// Record the whole step (parameter upload, s stages, step end) on the stream. Buffers
// rotate Y_{j-1} -> Y_j through three stage buffers; in the FP64 form the last stage
// writes into yb[1-par] so that acceptance only flips the parity.
static void record_step(LSRKMem* m, STS_Problem p, int s, int par)
{
  cudaStream_t st = m->ctx->stream;
  const long long n = m->n;
  const int nxt     = 1 - par;
  cudaMemcpyAsync(m->d_par, m->h_par, sizeof(StepArgs) + 8 + sizeof(StageArgs) * (size_t)(s + 1),
                  cudaMemcpyHostToDevice, st);
  const int eb = ew_blocks(m->ctx, n, 256 * 4);
  if (!m->mixed)
  {
    // stage 1 into Y[0]; stages j = 2..s rotate Y[1], Y[2], Y[0], ...; the final stage
    // writes yb[nxt]
    double* bufs[3] = {m->Y[0], m->Y[1], m->Y[2]};
    double* y1      = bufs[0];
    stage1_64_kernel<<<eb, 256, 0, st>>>(n, dstep(m), m->yb[par], m->Fb[par], y1);
    const double* ym2 = m->yb[par];
    const double* ym1 = y1;
    int bi            = 1;
    for (int j = 2; j <= s; ++j)
    {
      double* yj = (j == s) ? m->yb[nxt] : bufs[bi];
      bi         = (bi + 1) % 3;
      launch_stage64(m, p, dstage(m) + j, ym1, ym2, m->yb[par], m->Fb[par], yj);
      ym2 = ym1;
      ym1 = yj;
    }
    launch_stepend(m, p, par, m->yb[nxt], nullptr);
  }
  else
  {
    stage1_32_kernel<<<eb, 256, 0, st>>>(n, dstep(m), m->Ffb[par], m->D[0]);
    int im2 = -1, im1 = 0;
    const int nbuf = m->fuse_ks > 1 ? 4 : 3;
    auto free_buf = [&](int skip) { // a stage buffer that is neither input nor `skip`
      for (int b = 0; b < nbuf; ++b)
        if (b != im1 && b != im2 && b != skip) return b;
      return -1;
    };
    for (int j = 2; j <= s;)
    {
      const int ks = std::min(m->fuse_ks, s - j + 1);
      if (ks >= 2)
      {
        // stages j .. j+ks-1 in one launch; the group's last two stages land in the two
        // buffers that are not its inputs
        const int o2 = free_buf(-1), o1 = free_buf(o2);
        if (tma_fused_launch(&m->tma, m->fuse_ti, ks, m->ctx->num_sms, p->dev, dstage(m) + j, im1, im2, par,
                             m->D[o2], m->D[o1], m->ctx->d_err, st))
        {
          im2 = o2;
          im1 = o1;
          j += ks;
          continue;
        }
      }
      const int ij = free_buf(-1);
      launch_stage32_idx(m, p, dstage(m) + j, im1, im2, par, ij);
      im2 = im1;
      im1 = ij;
      ++j;
    }
    launch_stepend(m, p, par, nullptr, m->D[im1]);
  }
}

static int run_step_fused(LSRKMem* m, STS_Problem p, int s)
{
  cudaStream_t st = m->ctx->stream;
  if (m->use_graphs)
  {
    GraphKey key{s, m->par};
    auto it = m->graphs.find(key);
    if (it == m->graphs.end())
    {
      cudaGraph_t g;
      if (!STS_CUDA_OK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal))) return -1;
      record_step(m, p, s, m->par);
      if (!STS_CUDA_OK(cudaStreamEndCapture(st, &g))) return -1;
      cudaGraphExec_t ge;
      if (!STS_CUDA_OK(cudaGraphInstantiate(&ge, g, 0))) return -1;
      cudaGraphDestroy(g);
      it = m->graphs.emplace(key, ge).first;
    }
    if (!STS_CUDA_OK(cudaGraphLaunch(it->second, st))) return -1;
  }
  else record_step(m, p, s, m->par);
  return STS_CUDA_OK(cudaGetLastError()) ? 0 : -1;
}

// fill the host parameter block for a step of size h with s stages from t
static void fill_params(LSRKMem* m, STS_Problem p, double t, double h, int s, const std::vector<double>& mu,
                        const std::vector<double>& nu, const std::vector<double>& mus,
                        const std::vector<double>& ajm1, const std::vector<double>& cjm1)
{
  StepArgs* S = hstep(m);
  S->hm1      = h * mus[1];
  S->hm1f     = (float)(h * mus[1]);
  S->p4h      = 0.4 * h;
  S->rtol     = m->rtol;
  S->atol     = m->atol;
  {
    const double c = sts_c(t + h), cd = sts_cdot(t + h);
    S->al          = 1.0 * cd;
    S->be          = -(1.0 * c) * p->kx;
    S->ga          = -(1.0 * c) * p->ky;
  }
  const double c0 = sts_c(t), cd0 = sts_cdot(t);
  StageArgs* A    = hstage(m);
  for (int j = 2; j <= s; ++j)
  {
    StageArgs& a    = A[j];
    const double hm = h * mus[j];
    const double tj = t + h * cjm1[j];
    const double tm = hm * p->cc;
    a.gc            = mu[j] + tm;
    a.gx            = hm * p->cx;
    a.gy            = hm * p->cy;
    a.gn            = nu[j];
    a.g0            = (1.0 - mu[j]) - nu[j];
    a.gf            = -(hm * ajm1[j]);
    const double c = sts_c(tj), cd = sts_cdot(tj);
    a.al            = hm * cd;
    a.be            = -(hm * c) * p->kx;
    a.ga            = -(hm * c) * p->ky;
    a.gsf           = (float)(((mu[j] + nu[j]) - 1.0) + hm * ((p->cc + 2.0 * p->cx) + 2.0 * p->cy));
    a.gxf           = (float)a.gx;
    a.gyf           = (float)a.gy;
    a.gmf           = (float)(-nu[j]);
    a.gFf           = (float)(hm * (1.0 - ajm1[j]));
    const double dc  = c - c0;
    const double dcd = cd - cd0;
    a.alf           = (float)(hm * dcd);
    a.bef           = (float)(-(hm * dc) * p->kx);
    a.gaf           = (float)(-(hm * dc) * p->ky);
  }
}

// ---------------------------------------------------------------------------------------
// shared evolve logic
// ---------------------------------------------------------------------------------------
static int dee_update(LSRKMem* m, N_Vector ycur, N_Vector fcur)
{
  STS_MARK_REGION("DomEig");
  double lam = 0.0, lami = 0.0;
  if (m->power)
  {
    STS_Problem p = (STS_Problem)m->user_data;
    if (!m->evec)
    {
      if (!STS_CUDA_OK(cudaMalloc(&m->evec, m->n * sizeof(double)))) return -1;
      cudaMemcpyAsync(m->evec, N_VGetDeviceArrayPointer_Sts(ycur), m->n * sizeof(double), cudaMemcpyDeviceToDevice,
                      m->ctx->stream);
    }
    N_Vector ev = N_VMake_Sts(m->n, m->evec, m->ctx);
    int it      = 0, rc = 0;
    // warm-up ("preprocessing") iterations: v <- A v / |A v| without a convergence test
    const int warm = (m->ndee == 0) ? m->dee_init_warmups : m->dee_succ_warmups;
    if (warm > 0)
    {
      rc = STS_PowerIteration(p, ev, warm, 0.0, &lam, &it);
      m->nfe_dee += it;
    }
    if (rc == 0) rc = STS_PowerIteration(p, ev, m->dee_maxiters, m->dee_reltol, &lam, &it);
    N_VDestroy_Sts(ev);
    if (rc) return -1;
    m->nfe_dee += it;
  }
  else if (m->domeig)
  {
    if (!m->nv_tmp[0])
      for (int k = 0; k < 3; ++k) m->nv_tmp[k] = N_VClone_Sts(ycur);
    int rc = m->domeig(m->t, ycur, fcur, &lam, &lami, m->user_data, m->nv_tmp[0], m->nv_tmp[1], m->nv_tmp[2]);
    if (rc) return -1;
  }
  else
  {
    sts_set_error("LSRKStep: no dominant eigenvalue function or estimator");
    return -1;
  }
  m->rho = m->eig_safety * fabs(lam);
  m->ndee++;
  m->steps_since_dee = 0;
  return 0;
}

// Initial step (Hairer, Norsett & Wanner II.4) with the probe capped at 1/rho.
static double initial_step(LSRKMem* m, const double* y0, const double* F0, double tdist)
{
  STS_Context ctx = m->ctx;
  const long long n = m->n;
  double d0 = sts_wrms_ewt(ctx, y0, nullptr, y0, n, m->rtol, m->atol, SLOT_D0);
  double d1 = sts_wrms_ewt(ctx, F0, nullptr, y0, n, m->rtol, m->atol, SLOT_D1);
  double h0 = (d0 < 1.0e-5 || d1 < 1.0e-5) ? 1.0e-6 : 0.01 * (d0 / d1);
  if (m->rho > 0.0 && h0 * m->rho > 1.0) h0 = 1.0 / m->rho;
  if (h0 > tdist) h0 = tdist;
  double *y1 = nullptr, *F1 = nullptr;
  cudaMallocAsync(&y1, n * sizeof(double), ctx->stream);
  cudaMallocAsync(&F1, n * sizeof(double), ctx->stream);
  N_Vector vy1 = N_VMake_Sts(n, y1, ctx), vF1 = N_VMake_Sts(n, F1, ctx);
  N_Vector vy0 = N_VMake_Sts(n, (double*)y0, ctx), vF0 = N_VMake_Sts(n, (double*)F0, ctx);
  N_VLinearSum_Sts(h0, vF0, 1.0, vy0, vy1); // fma(h0, F0, 1*y0) = fma(h0, F0, y0)
  int rc = m->rhs(m->t + h0, vy1, vF1, m->user_data);
  m->nfe++;
  double d2 = sts_wrms_ewt(ctx, F1, F0, y0, n, m->rtol, m->atol, SLOT_D2) / h0;
  N_VDestroy_Sts(vy1);
  N_VDestroy_Sts(vF1);
  N_VDestroy_Sts(vy0);
  N_VDestroy_Sts(vF0);
  cudaFreeAsync(y1, ctx->stream);
  cudaFreeAsync(F1, ctx->stream);
  if (rc < 0) return -1.0;
  const double dm = d1 > d2 ? d1 : d2;
  double h1       = (dm <= 1.0e-15) ? fmax(1.0e-6, h0 * 1.0e-3) : stsm::pow(0.01 / dm, 1.0 / m->ord);
  if (!(h1 > 0.0) || !(h1 < INFINITY)) h1 = h0;
  double h = (100.0 * h0 < h1) ? 100.0 * h0 : h1;
  if (h > tdist) h = tdist;
  return h;
}

double sts_wrms_ewt(STS_Context ctx, const double* a, const double* b, const double* y, long long n, double rtol,
                    double atol, int slot)
{
  ctx_activate(ctx);
  const int g = ew_blocks(ctx, n, 256 * 4);
  if (b) wrms_ewt_kernel<1><<<g, 256, 0, ctx->stream>>>(n, a, b, y, rtol, atol, ctx->d_work, ctx->d_slots + slot);
  else wrms_ewt_kernel<0><<<g, 256, 0, ctx->stream>>>(n, a, b, y, rtol, atol, ctx->d_work, ctx->d_slots + slot);
  if (!STS_CUDA_OK(cudaStreamSynchronize(ctx->stream))) return NAN;
  return ((volatile double*)ctx->h_slots)[slot];
}

// controller update after an accepted step of size h with error dsm
static void accept_control(LSRKMem* m, double h, double dsm)
{
  m->interp_ready = true;
  const double hprev = m->hlast; // previous accepted step (implicit Gustafsson controller)
  m->hlast           = h;
  if (m->hfixed > 0.0)
  {
    m->hnext = m->hfixed;
  }
  else
  {
    double hn  = controller_estimate(m->controller, h, dsm, m->ep1, m->ep2, hprev, m->nhist, m->ord);
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
}

static void reject_control(LSRKMem* m, double h, double dsm, int nef)
{
  double hn  = controller_estimate(m->controller, h, dsm, m->ep1, m->ep2, m->hlast, m->nhist, m->ord);
  double eta = SAFETY * hn / h;
  if (eta > 1.0) eta = 1.0;
  if (nef >= SMALL_NEF && eta > ETAMXF) eta = ETAMXF;
  if (eta < ETAMIN) eta = ETAMIN;
  m->hnext      = h * eta;
  m->after_fail = true;
}

// one attempt's stage count and step size (returns -2 if a fixed step needs > smax stages)
static int choose_step(LSRKMem* m, double target, double* hout, int* sout, bool* clipped)
{
  double h = m->hnext, hmax;
  *clipped = false;
  int s    = STS_LSRKStagesNeeded(m->method, h, m->rho, m->smax, &hmax);
  if (s > m->smax)
  {
    if (m->hfixed > 0.0)
    {
      sts_set_error("LSRKStep: fixed step needs %d stages > max %d", s, m->smax);
      return -2;
    }
    h = hmax;
    m->nst_exp++;
  }
  if (m->t + h >= target)
  {
    h        = target - m->t;
    *clipped = true;
  }
  s     = STS_LSRKStagesNeeded(m->method, h, m->rho, m->smax, &hmax);
  *hout = h;
  *sout = s;
  return 0;
}

// ---------------------------------------------------------------------------------------
// fused evolve
// ---------------------------------------------------------------------------------------
// Step loop of ARKodeEvolve: NORMAL mode steps until t >= tout, ONE_STEP mode takes one step;
// steps are clipped only at `clip` (the stop time, or +inf), which they then end on exactly.
static int evolve_fused(LSRKMem* m, double tout, double clip, int itask)
{
  STS_Problem p   = (STS_Problem)m->user_data;
  cudaStream_t st = m->ctx->stream;
  const long long n = m->n;
  if (ensure_stage_buffers(m) || ensure_par(m)) return STS_ERR_FAILURE;
  if (m->mixed && !m->tuned) autotune_stage32(m, p);
  if (!m->nv_y) m->nv_y = N_VMake_Sts(n, nullptr, m->ctx);
  if (!m->nv_F) m->nv_F = N_VMake_Sts(n, nullptr, m->ctx);
  NVC(m->nv_y)->nx = p->nx;
  NVC(m->nv_y)->ny = p->ny;
  if (!m->initialized)
  {
    sts_rhs_launch(p, m->t, m->yb[m->par], m->Fb[m->par], true, st);
    m->nfe++;
    if (m->mixed) sts_f64_to_f32(m->ctx, m->Fb[m->par], m->Ffb[m->par], n);
    m->hnext           = (m->hfixed > 0.0) ? m->hfixed : 0.0;
    m->initialized     = true;
    m->steps_since_dee = -1;
  }
  std::vector<double> mu(m->smax + 1), nu(m->smax + 1), mus(m->smax + 1), ajm1(m->smax + 1), cjm1(m->smax + 1);
  long long nsteps_call = 0;
  int ret               = STS_SUCCESS;
  const double tdist_to = tout < clip ? tout : clip; // initial-step distance
  while (m->t < clip && (itask == STS_ONE_STEP || m->t < tout))
  {
    if (nsteps_call >= (m->maxsteps > 0 ? m->maxsteps : 500))
    {
      ret = STS_TOO_MUCH_WORK;
      break;
    }
    NVC(m->nv_y)->data = m->yb[m->par];
    NVC(m->nv_F)->data = m->Fb[m->par];
    const long long freq = m->dom_eig_freq; // <= 0: computed once
    if (m->steps_since_dee < 0 || (freq > 0 && m->steps_since_dee >= freq))
      if (dee_update(m, m->nv_y, m->nv_F)) return STS_ERR_FAILURE;
    if (!(m->hnext > 0.0))
    {
      double h0 = initial_step(m, m->yb[m->par], m->Fb[m->par], tdist_to - m->t);
      if (!(h0 > 0.0))
      {
        sts_set_error("LSRKStep: no usable initial step (RHS failure or non-finite state)");
        return STS_ERR_FAILURE;
      }
      m->hnext = h0;
    }
    int nef = 0;
    for (;;)
    {
      double h;
      int s;
      bool clipped;
      int rc = choose_step(m, clip, &h, &s, &clipped);
      if (rc) return STS_ILL_INPUT;
      STS_LSRKStageCoeffs(m->method, s, mu.data(), nu.data(), mus.data(), ajm1.data(), cjm1.data());
      m->nst_att++;
      fill_params(m, p, m->t, h, s, mu, nu, mus, ajm1, cjm1);
      if (run_step_fused(m, p, s)) return STS_ERR_FAILURE;
      m->interp_ready = false; // the attempt wrote y_{n+1} over the other parity buffer
      if (!STS_CUDA_OK(cudaStreamSynchronize(st))) return STS_ERR_FAILURE;
      if (const int ew = *(volatile int*)m->ctx->h_err)
      {
        *m->ctx->h_err = 0;
        sts_set_error("LSRKStep: %s in a stage kernel", sts_err_word_text(ew));
        return STS_ERR_FAILURE;
      }
      const double dsm = ((volatile double*)m->ctx->h_slots)[SLOT_DSM];
      m->nfe += s;
      m->stages_total += s;
      if (s > m->stage_max) m->stage_max = s;
      m->last_s = s;
      if (m->hfixed > 0.0 || dsm <= 1.0)
      {
        m->t     = clipped ? clip : m->t + h;
        m->par   = 1 - m->par;
        accept_control(m, h, dsm);
        m->nst++;
        m->steps_since_dee++;
        nsteps_call++;
        break;
      }
      m->netf++;
      nef++;
      if (!(dsm == dsm) || nef > 20) return STS_ERR_FAILURE;
      reject_control(m, h, dsm, nef);
    }
    if (itask == STS_ONE_STEP) break;
  }
  return ret;
}

// ---------------------------------------------------------------------------------------
// generic evolve (user RHS through N_Vector ops)
// ---------------------------------------------------------------------------------------
// One SSP step attempt of size h from (t, y, F = F(t, y)) with N_Vector operations: the new
// state into `yout`, the error estimate h sum_j w_j F_j into m->g_err. Registers: q1 = g_Y[0],
// q2 = g_Y[1], stage derivative G = g_F. Returns the RHS status (0 ok).
static int ssp_attempt(LSRKMem* m, double h, N_Vector y, N_Vector F, N_Vector yout)
{
  const int type = m->method, s = m->ssp_stages;
  const std::vector<double>& w = m->ssp_w;
  N_Vector q1 = m->g_Y[0], q2 = m->g_Y[1], G = m->g_F, E = m->g_err;
  const std::vector<double>& c = m->ssp_c;
  int j = 0;
  // stage j: G = F(t + c_j h, q) (stage 0 reuses F), E += h w_j G; returns the derivative
  auto stage = [&](N_Vector q) -> N_Vector {
    N_Vector g = F;
    if (j > 0)
    {
      const int rc = m->rhs(m->t + c[j] * h, q, G, m->user_data);
      if (rc != 0) return nullptr;
      g = G;
    }
    if (j == 0) N_VScale_Sts(h * w[0], g, E);
    else N_VLinearSum_Sts(h * w[j], g, 1.0, E, E);
    ++j;
    return g;
  };
  int frc = 0;
  auto euler = [&](double hr) { // q1 = q1 + hr F(q1)
    N_Vector g = stage(q1);
    if (!g) return false;
    N_VLinearSum_Sts(hr, g, 1.0, q1, q1);
    return true;
  };
  N_VScale_Sts(1.0, y, q1);
  if (type == SSP_S_2)
  {
    const double hr = h / (s - 1.0);
    for (int i = 0; i < s - 1; ++i)
      if (!euler(hr)) return 1;
    N_Vector g = stage(q1);
    if (!g) return 1;
    double cf[3]  = {1.0 / s, (s - 1.0) / s, (s - 1.0) / s * hr};
    N_Vector X[3] = {y, q1, g};
    N_VLinearCombination_Sts(3, cf, X, yout);
  }
  else if (type == SSP_S_3)
  {
    const int n     = (int)std::lround(std::sqrt((double)s));
    const double hr = h / (double)(n * n - n);
    const int e1 = (n - 1) * (n - 2) / 2, e2 = n * (n + 1) / 2;
    for (int i = 1; i <= e1; ++i)
      if (!euler(hr)) return 1;
    N_VScale_Sts(1.0, q1, q2);
    for (int i = e1 + 1; i <= e2 - 1; ++i)
      if (!euler(hr)) return 1;
    N_Vector g = stage(q1);
    if (!g) return 1;
    double cf[3]  = {(double)n / (2 * n - 1), (n - 1.0) / (2 * n - 1), (n - 1.0) / (2 * n - 1) * hr};
    N_Vector X[3] = {q2, q1, g};
    N_VLinearCombination_Sts(3, cf, X, q1);
    for (int i = e2 + 1; i <= n * n; ++i)
      if (!euler(hr)) return 1;
    N_VScale_Sts(1.0, q1, yout);
  }
  else
  {
    N_VScale_Sts(1.0, y, q2);
    for (int i = 1; i <= 5; ++i)
      if (!euler(h / 6.0)) return 1;
    {
      double cf[2]  = {1.0 / 25.0, 9.0 / 25.0};
      N_Vector X[2] = {q2, q1};
      N_VLinearCombination_Sts(2, cf, X, q2);
    }
    {
      double cf[2]  = {15.0, -5.0};
      N_Vector X[2] = {q2, q1};
      N_VLinearCombination_Sts(2, cf, X, q1);
    }
    for (int i = 6; i <= 9; ++i)
      if (!euler(h / 6.0)) return 1;
    N_Vector g = stage(q1);
    if (!g) return 1;
    double cf[3]  = {1.0, 3.0 / 5.0, h / 10.0};
    N_Vector X[3] = {q2, q1, g};
    N_VLinearCombination_Sts(3, cf, X, yout);
  }
  (void)frc;
  return 0;
}

// ---------------------------------------------------------------------------------------
// Reference mode (periodic wrap, per-face coefficients) through the generic path, fused: a
// stage is F_j = f(Y_{j-1}) evaluated in registers exactly as rhs_kernel does, then the
// N_VLinearCombination of (Y_{j-1}, Y_{j-2}, Y_0, F_j, F_0) in that kernel's order; the
// step end folds the error combination, ewt = N_VInv(N_VAddConst(N_VScale(rtol, |y|), atol))
// and the exact WRMS into one pass. Bit for bit the unfused sequence, with 40 instead of 64
// bytes per point and stage and one kernel instead of seven per step end.
// ---------------------------------------------------------------------------------------
__global__ void __launch_bounds__(256) periodic_stage_kernel(ProbDev P, double c0, double c1, double c2, double c3,
                                                             double c4, const double* __restrict__ ym1,
                                                             const double* __restrict__ ym2,
                                                             const double* __restrict__ y0,
                                                             const double* __restrict__ f0, double* __restrict__ yj)
{
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long j = (long long)blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= P.nx || j >= P.ny) return;
  const long long k = j * P.nx + i;
  const double fj   = periodic_point(P, ym1, i, j);
  double acc        = __dmul_rn(c0, ym1[k]);
  acc               = __fma_rn(c1, ym2[k], acc);
  acc               = __fma_rn(c2, y0[k], acc);
  acc               = __fma_rn(c3, fj, acc);
  acc               = __fma_rn(c4, f0[k], acc);
  yj[k]             = acc;
}

__global__ void __launch_bounds__(256) periodic_err_kernel(long long n, const double* __restrict__ y,
                                                           const double* __restrict__ ys,
                                                           const double* __restrict__ f0,
                                                           const double* __restrict__ fs, double p4h, double rtol,
                                                           double atol, RedWork* w, double* slot)
{
  xsum::Limbs acc;
  xsum::zero(acc);
  unsigned flags         = 0;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += stride)
  {
    const double yv = y[k];
    double e        = __dmul_rn(0.8, yv);
    e               = __fma_rn(-0.8, ys[k], e);
    e               = __fma_rn(p4h, f0[k], e);
    e               = __fma_rn(p4h, fs[k], e);
    const double wt = __drcp_rn(__dadd_rn(__dmul_rn(rtol, fabs(yv)), atol));
    const double x  = __dmul_rn(e, wt);
    xsum::add(acc, __dmul_rn(x, x), flags);
  }
  xsum_block_finish<256>(acc, flags, w, slot, 1, (double)n);
}

// Mixed reference mode: FP32 increments d_j = Y_j - Y_0 of the periodic problem in the
// difference form of the Dirichlet mixed stage (kernels.cuh): with A d = sum over the four faces
// D_face (d_nb - d_C) (exact: the diagonal is minus the sum of the faces),
//   d_j = d_C + inc, inc = gs d_C + hm A d + gm (d_C - d_{j-2}) + gF F_0,
//   gs = mu + nu - 1, gm = -nu, gF = hm (1 - a_{j-1}), FP32 face tables.
// The step end forms y_{n+1} = y_n + d_s in FP64; F(y_{n+1}), the error and the WRMS stay FP64.
__global__ void __launch_bounds__(256) periodic_stage32_kernel(ProbDev P, const float* __restrict__ faces, float gs,
                                                               float hmf, float gm, float gF,
                                                               const float* __restrict__ dm1,
                                                               const float* __restrict__ dm2,
                                                               const float* __restrict__ f0f, float* __restrict__ dj)
{
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long j = (long long)blockIdx.y * blockDim.y + threadIdx.y;
  const long long nx = P.nx, ny = P.ny;
  if (i >= nx || j >= ny) return;
  const float* Dxwf = faces;
  const float* Dxef = faces + nx;
  const float* Dysf = faces + 2 * nx;
  const float* Dynf = faces + 2 * nx + ny;
  const long long iw = (i == 0) ? nx - 1 : i - 1, ie = (i == nx - 1) ? 0 : i + 1;
  const long long js = (j == 0) ? ny - 1 : j - 1, jn = (j == ny - 1) ? 0 : j + 1;
  const long long k  = j * nx + i;
  const float dC = dm1[k], dW = dm1[j * nx + iw], dE = dm1[j * nx + ie], dS = dm1[js * nx + i],
              dN = dm1[jn * nx + i];
  const float m2 = dm2 ? dm2[k] : 0.0f;
  float a        = __fmul_rn(Dxwf[i], __fsub_rn(dW, dC));
  a              = __fmaf_rn(Dxef[i], __fsub_rn(dE, dC), a);
  a              = __fmaf_rn(Dysf[j], __fsub_rn(dS, dC), a);
  a              = __fmaf_rn(Dynf[j], __fsub_rn(dN, dC), a);
  float inc      = __fmul_rn(gs, dC);
  inc            = __fmaf_rn(hmf, a, inc);
  inc            = __fmaf_rn(gm, __fsub_rn(dC, m2), inc);
  inc            = __fmaf_rn(gF, f0f[k], inc);
  dj[k]          = __fadd_rn(dC, inc);
}

__global__ void __launch_bounds__(256) scale32_kernel(long long n, float c, const float* __restrict__ x,
                                                      float* __restrict__ z)
{
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += stride) z[k] = __fmul_rn(c, x[k]);
}

__global__ void __launch_bounds__(256) add_increment_kernel(long long n, const double* __restrict__ y,
                                                            const float* __restrict__ d, double* __restrict__ out)
{
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += stride)
    out[k] = __dadd_rn(y[k], (double)d[k]);
}

static bool periodic_fusable(const LSRKMem* m)
{
  return !m->ssp && m->rhs == STS_Diffusion && m->user_data != nullptr &&
         ((STS_Problem)m->user_data)->kind == STS_PROBLEM_PERIODIC && m->use_fused_periodic;
}

static int evolve_generic(LSRKMem* m, double tout, double clip, int itask)
{
  N_Vector y = m->g_y, F = m->g_Fn;
  if (!m->g_Y[0])
  {
    for (int k = 0; k < 3; ++k) m->g_Y[k] = N_VClone_Sts(y);
    m->g_F    = N_VClone_Sts(y);
    m->g_Fnew = N_VClone_Sts(y);
    m->g_err  = N_VClone_Sts(y);
    m->g_ewt  = N_VClone_Sts(y);
    m->g_yold = N_VClone_Sts(y);
    m->g_Fold = N_VClone_Sts(y);
  }
  if (!m->initialized)
  {
    if (m->rhs(m->t, y, F, m->user_data) != 0) return STS_RHSFUNC_FAIL;
    m->nfe++;
    m->hnext           = (m->hfixed > 0.0) ? m->hfixed : 0.0;
    m->initialized     = true;
    m->steps_since_dee = -1;
  }
  std::vector<double> mu(m->smax + 1), nu(m->smax + 1), mus(m->smax + 1), ajm1(m->smax + 1), cjm1(m->smax + 1);
  long long nsteps_call = 0;
  int ret               = STS_SUCCESS;
  const double tdist_to = tout < clip ? tout : clip;
  while (m->t < clip && (itask == STS_ONE_STEP || m->t < tout))
  {
    if (nsteps_call >= (m->maxsteps > 0 ? m->maxsteps : 500))
    {
      ret = STS_TOO_MUCH_WORK;
      break;
    }
    const long long freq = m->dom_eig_freq; // <= 0: computed once
    if (!m->ssp && (m->steps_since_dee < 0 || (freq > 0 && m->steps_since_dee >= freq)))
      if (dee_update(m, y, F)) return STS_ERR_FAILURE;
    if (!(m->hnext > 0.0))
    {
      double h0 = initial_step(m, NVD(y), NVD(F), tdist_to - m->t);
      if (!(h0 > 0.0))
      {
        sts_set_error("LSRKStep: no usable initial step (RHS failure or non-finite state)");
        return STS_ERR_FAILURE;
      }
      m->hnext = h0;
    }
    int nef = 0, ncf_step = 0;
    for (;;)
    {
      double h;
      int s;
      bool clipped;
      if (m->ssp)
      { // fixed stage count; the step only clipped at the stop time
        h       = m->hnext;
        clipped = false;
        if (m->t + h >= clip)
        {
          h       = clip - m->t;
          clipped = true;
        }
        s = m->ssp_stages;
        m->nst_att++;
        const int frc = ssp_attempt(m, h, y, F, m->g_Fnew); // new state into g_Fnew (scratch)
        m->nfe += s - 1;
        if (frc != 0)
        { // recoverable RHS failure: retry with h/4
          m->ncf++;
          if (++ncf_step > 10) return STS_RHSFUNC_FAIL;
          m->hnext      = 0.25 * h;
          m->after_fail = true;
          continue;
        }
        N_VAbs_Sts(y, m->g_ewt);
        N_VScale_Sts(m->rtol, m->g_ewt, m->g_ewt);
        N_VAddConst_Sts(m->g_ewt, m->atol, m->g_ewt);
        N_VInv_Sts(m->g_ewt, m->g_ewt);
        const double dsm = N_VWrmsNorm_Sts(m->g_err, m->g_ewt);
        m->stages_total += s;
        if (s > m->stage_max) m->stage_max = s;
        if (m->hfixed > 0.0 || dsm <= 1.0)
        {
          m->t = clipped ? clip : m->t + h;
          cudaMemcpyAsync(NVD(m->g_yold), NVD(y), m->n * sizeof(double), cudaMemcpyDeviceToDevice, m->ctx->stream);
          cudaMemcpyAsync(NVD(m->g_Fold), NVD(F), m->n * sizeof(double), cudaMemcpyDeviceToDevice, m->ctx->stream);
          cudaMemcpyAsync(NVD(y), NVD(m->g_Fnew), m->n * sizeof(double), cudaMemcpyDeviceToDevice, m->ctx->stream);
          if (m->rhs(m->t, y, F, m->user_data) != 0) return STS_RHSFUNC_FAIL; // F(y_{n+1}) for the next step
          m->nfe++;
          accept_control(m, h, dsm);
          m->nst++;
          nsteps_call++;
          break;
        }
        m->netf++;
        nef++;
        if (!(dsm == dsm) || nef > 20) return STS_ERR_FAILURE;
        reject_control(m, h, dsm, nef);
        continue;
      }
      if (choose_step(m, clip, &h, &s, &clipped)) return STS_ILL_INPUT;
      STS_LSRKStageCoeffs(m->method, s, mu.data(), nu.data(), mus.data(), ajm1.data(), cjm1.data());
      m->nst_att++;
      const bool pf = periodic_fusable(m);
      const bool pm = pf && m->mixed; // mixed reference mode
      N_Vector ym2 = y, ym1 = m->g_Y[0], yj = m->g_Y[0];
      int bi = 1, frc = 0;
      if (pm)
      {
        STS_Problem p   = (STS_Problem)m->user_data;
        STS_Context ctx = m->ctx;
        const long long n = m->n;
        if (!m->per_faces)
        {
          if (!STS_CUDA_OK(cudaMalloc(&m->per_faces, (2 * p->nx + 2 * p->ny) * sizeof(float)))) return STS_ERR_FAILURE;
          for (int b = 0; b < 3; ++b)
            if (!m->D[b] && !STS_CUDA_OK(cudaMalloc(&m->D[b], n * sizeof(float)))) return STS_ERR_FAILURE;
          if (!m->Ffb[0] && !STS_CUDA_OK(cudaMalloc(&m->Ffb[0], n * sizeof(float)))) return STS_ERR_FAILURE;
          sts_f64_to_f32(ctx, p->dev.Dxw, m->per_faces, p->nx);
          sts_f64_to_f32(ctx, p->dev.Dxe, m->per_faces + p->nx, p->nx);
          sts_f64_to_f32(ctx, p->dev.Dys, m->per_faces + 2 * p->nx, p->ny);
          sts_f64_to_f32(ctx, p->dev.Dyn, m->per_faces + 2 * p->nx + p->ny, p->ny);
        }
        sts_f64_to_f32(ctx, NVD(F), m->Ffb[0], n); // FP32 copy of F_n
        const int g1 = ew_blocks(ctx, n, 256 * 4);
        scale32_kernel<<<g1, 256, 0, ctx->stream>>>(n, (float)(h * mus[1]), m->Ffb[0], m->D[0]);
        const dim3 b(64, 4), g((unsigned)((p->nx + 63) / 64), (unsigned)((p->ny + 3) / 4));
        int im1 = 0, im2 = -1;
        for (int j = 2; j <= s; ++j)
        {
          const int io   = (im1 + 1) % 3;
          const double hm = h * mus[j];
          periodic_stage32_kernel<<<g, b, 0, ctx->stream>>>(
            p->dev, m->per_faces, (float)((mu[j] + nu[j]) - 1.0), (float)hm, (float)(-nu[j]),
            (float)(hm * (1.0 - ajm1[j])), m->D[im1], im2 >= 0 ? m->D[im2] : nullptr, m->Ffb[0], m->D[io]);
          im2 = im1;
          im1 = io;
        }
        add_increment_kernel<<<g1, 256, 0, ctx->stream>>>(n, NVD(y), m->D[im1], NVD(m->g_Y[0]));
        yj = m->g_Y[0];
      }
      else
        // Y_1 = y_n + h mus_1 F_n
        N_VLinearSum_Sts(h * mus[1], F, 1.0, y, m->g_Y[0]);
      for (int j = 2; j <= s && frc == 0 && !pm; ++j)
      {
        const double hm = h * mus[j];
        double c[5]    = {mu[j], nu[j], (1.0 - mu[j]) - nu[j], hm, -(hm * ajm1[j])};
        yj             = m->g_Y[bi];
        bi             = (bi + 1) % 3;
        if (pf)
        {
          STS_Problem p = (STS_Problem)m->user_data;
          const dim3 b(64, 4), g((unsigned)((p->nx + 63) / 64), (unsigned)((p->ny + 3) / 4));
          periodic_stage_kernel<<<g, b, 0, m->ctx->stream>>>(p->dev, c[0], c[1], c[2], c[3], c[4], NVD(ym1),
                                                             NVD(ym2), NVD(y), NVD(F), NVD(yj));
        }
        else
        {
          frc = m->rhs(m->t + h * cjm1[j], ym1, m->g_F, m->user_data);
          if (frc != 0) break;
          N_Vector X[5] = {ym1, ym2, y, m->g_F, F};
          N_VLinearCombination_Sts(5, c, X, yj);
        }
        ym2 = ym1;
        ym1 = yj;
      }
      if (frc == 0) frc = m->rhs(m->t + h, yj, m->g_Fnew, m->user_data);
      m->nfe += s;
      if (frc < 0) return STS_RHSFUNC_FAIL;
      if (frc > 0)
      { // recoverable RHS failure (diffusion_2D.cpp:900-933 convention): retry with h/4
        m->ncf++;
        if (++ncf_step > 10) return STS_RHSFUNC_FAIL;
        m->hnext      = 0.25 * h;
        m->after_fail = true;
        continue;
      }
      // err = 0.8 (y_n - y_{n+1}) + 0.4 h (F_n + F_{n+1}); ewt = 1/(rtol |y_n| + atol)
      double dsm;
      if (pf)
      {
        STS_Context ctx = m->ctx;
        periodic_err_kernel<<<ew_blocks(ctx, m->n, 256 * 4), 256, 0, ctx->stream>>>(
            m->n, NVD(y), NVD(yj), NVD(F), NVD(m->g_Fnew), 0.4 * h, m->rtol, m->atol, ctx->d_work,
            ctx->d_slots + SLOT_GENERIC);
        if (!STS_CUDA_OK(cudaStreamSynchronize(ctx->stream))) return STS_ERR_FAILURE;
        dsm = ((volatile double*)ctx->h_slots)[SLOT_GENERIC];
      }
      else
      {
        double c[4]   = {0.8, -0.8, 0.4 * h, 0.4 * h};
        N_Vector X[4] = {y, yj, F, m->g_Fnew};
        N_VLinearCombination_Sts(4, c, X, m->g_err);
        N_VAbs_Sts(y, m->g_ewt);
        N_VScale_Sts(m->rtol, m->g_ewt, m->g_ewt);
        N_VAddConst_Sts(m->g_ewt, m->atol, m->g_ewt);
        N_VInv_Sts(m->g_ewt, m->g_ewt);
        dsm = N_VWrmsNorm_Sts(m->g_err, m->g_ewt);
      }
      m->stages_total += s;
      if (s > m->stage_max) m->stage_max = s;
      if (m->hfixed > 0.0 || dsm <= 1.0)
      {
        m->t = clipped ? clip : m->t + h;
        cudaMemcpyAsync(NVD(m->g_yold), NVD(y), m->n * sizeof(double), cudaMemcpyDeviceToDevice, m->ctx->stream);
        cudaMemcpyAsync(NVD(y), NVD(yj), m->n * sizeof(double), cudaMemcpyDeviceToDevice, m->ctx->stream);
        cudaMemcpyAsync(NVD(F), NVD(m->g_Fnew), m->n * sizeof(double), cudaMemcpyDeviceToDevice, m->ctx->stream);
        accept_control(m, h, dsm);
        m->nst++;
        m->steps_since_dee++;
        nsteps_call++;
        break;
      }
      m->netf++;
      nef++;
      if (!(dsm == dsm) || nef > 20) return STS_ERR_FAILURE;
      reject_control(m, h, dsm, nef);
    }
    if (itask == STS_ONE_STEP) break;
  }
  return ret;
}

// ---------------------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------------------
#define MEM(v) ((LSRKMem*)(v))
#define CHECK_MEM(v)                                  \
  do                                                  \
  {                                                   \
    if (!(v))                                         \
    {                                                 \
      sts_set_error("LSRKStep: NULL integrator memory"); \
      return STS_MEM_NULL;                            \
    }                                                 \
  } while (0)

extern "C" void* STS_LSRKStepCreateSTS(STS_ARKRhsFn rhs, double t0, N_Vector y0, STS_Context ctx)
{
  if (!rhs || !y0 || !ctx)
  {
    sts_set_error("LSRKStepCreateSTS: NULL argument");
    return nullptr;
  }
  ctx_activate(ctx);
  LSRKMem* m = new LSRKMem();
  m->ctx     = ctx;
  m->rhs     = rhs;
  m->t       = t0;
  m->n       = NVL(y0);
  m->g_y     = N_VClone_Sts(y0);
  m->g_Fn    = N_VClone_Sts(y0);
  if (!m->g_y || !m->g_Fn)
  {
    delete m;
    return nullptr;
  }
  cudaMemcpyAsync(NVD(m->g_y), NVD(y0), m->n * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream);
  cudaStreamSynchronize(ctx->stream);
  return m;
}

extern "C" int STS_LSRKStepSetSTSMethod(void* mem, int method)
{
  CHECK_MEM(mem);
  if (MEM(mem)->ssp || (method != STS_LSRK_RKC_2 && method != STS_LSRK_RKL_2)) return STS_ILL_INPUT;
  MEM(mem)->method = method;
  return 0;
}

static void ssp_configure(LSRKMem* m)
{
  std::vector<double> A, b;
  ssp_tableau(m->method, m->ssp_stages, A, b, m->ssp_c, m->ssp_w);
  m->ord = (m->method == SSP_S_2) ? 2.0 : (m->method == SSP_S_3 ? 3.0 : 4.0); // embedding order + 1
}

// LSRKStepCreateSSP (diffusion_2D/main.cpp:251): SSP(s,2) with 10 stages until set otherwise
extern "C" void* STS_LSRKStepCreateSSP(STS_ARKRhsFn rhs, double t0, N_Vector y0, STS_Context ctx)
{
  void* mem = STS_LSRKStepCreateSTS(rhs, t0, y0, ctx);
  if (!mem) return nullptr;
  LSRKMem* m    = MEM(mem);
  m->ssp        = true;
  m->method     = SSP_S_2;
  m->ssp_stages = 10;
  ssp_configure(m);
  return mem;
}

// LSRKStepSetSSPMethod (main.cpp:289): ARKODE_LSRK_SSP_S_2 (10 stages), _S_3 (9), _10_4 (10)
extern "C" int STS_LSRKStepSetSSPMethod(void* mem, int type)
{
  CHECK_MEM(mem);
  LSRKMem* m = MEM(mem);
  if (!m->ssp || (type != SSP_S_2 && type != SSP_S_3 && type != SSP_10_4)) return STS_ILL_INPUT;
  m->method     = type;
  m->ssp_stages = (type == SSP_S_3) ? 9 : 10;
  ssp_configure(m);
  return 0;
}

// LSRKStepSetNumSSPStages (main.cpp:291): s >= 2 (S_2), s = n^2 >= 4 (S_3), s = 10 (10_4)
extern "C" int STS_LSRKStepSetNumSSPStages(void* mem, int s)
{
  CHECK_MEM(mem);
  LSRKMem* m = MEM(mem);
  if (!m->ssp || !ssp_stages_valid(m->method, s))
  {
    sts_set_error("LSRKStepSetNumSSPStages: %d stages are not valid for this SSP method", s);
    return STS_ILL_INPUT;
  }
  m->ssp_stages = s;
  ssp_configure(m);
  return 0;
}
extern "C" int STS_ARKodeSStolerances(void* mem, double rtol, double atol)
{
  CHECK_MEM(mem);
  if (sts_mem_kind(mem) == STS_MEM_ARKSTEP) return arkstep_sstolerances(mem, rtol, atol);
  if (rtol < 0 || atol < 0) return STS_ILL_INPUT;
  MEM(mem)->rtol = rtol;
  MEM(mem)->atol = atol;
  return 0;
}
extern "C" int STS_ARKodeSetUserData(void* mem, void* ud)
{
  CHECK_MEM(mem);
  if (sts_mem_kind(mem) == STS_MEM_ARKSTEP) return arkstep_set_user_data(mem, ud);
  MEM(mem)->user_data = ud;
  return 0;
}
extern "C" int STS_LSRKStepSetDomEigFn(void* mem, STS_ARKDomEigFn fn)
{
  CHECK_MEM(mem);
  MEM(mem)->domeig = fn;
  MEM(mem)->power  = false;
  return 0;
}
extern "C" int STS_LSRKStepSetDomEigEstimatorPower(void* mem, int maxiters, double reltol)
{
  CHECK_MEM(mem);
  MEM(mem)->power        = true;
  MEM(mem)->dee_maxiters = maxiters > 0 ? maxiters : 100;
  MEM(mem)->dee_reltol   = reltol > 0 ? reltol : 0.01;
  return 0;
}
extern "C" int STS_LSRKStepSetDomEigFrequency(void* mem, long long nsteps)
{
  CHECK_MEM(mem);
  MEM(mem)->dom_eig_freq = nsteps;
  return 0;
}
extern "C" int STS_LSRKStepSetMaxNumStages(void* mem, int smax)
{
  CHECK_MEM(mem);
  if (smax < 2) return STS_ILL_INPUT;
  MEM(mem)->smax = smax;
  return 0;
}
extern "C" int STS_LSRKStepSetDomEigSafetyFactor(void* mem, double safety)
{
  CHECK_MEM(mem);
  if (safety < 1.0) return STS_ILL_INPUT;
  MEM(mem)->eig_safety = safety;
  return 0;
}
extern "C" int STS_ARKodeSetAdaptController(void* mem, int controller)
{
  CHECK_MEM(mem);
  if (sts_mem_kind(mem) == STS_MEM_ARKSTEP) return arkstep_set_controller(mem, controller);
  if (controller < STS_ADAPT_PID || controller > STS_ADAPT_IMEX_GUS) return STS_ILL_INPUT;
  MEM(mem)->controller = controller;
  return 0;
}
extern "C" int STS_ARKodeSetFixedStep(void* mem, double h)
{
  CHECK_MEM(mem);
  if (sts_mem_kind(mem) == STS_MEM_ARKSTEP) return arkstep_set_fixed_step(mem, h);
  MEM(mem)->hfixed = h;
  if (h > 0.0) MEM(mem)->hnext = h;
  return 0;
}
extern "C" int STS_ARKodeSetMaxNumSteps(void* mem, long long mxsteps)
{
  CHECK_MEM(mem);
  if (sts_mem_kind(mem) == STS_MEM_ARKSTEP) return arkstep_set_max_steps(mem, mxsteps);
  MEM(mem)->maxsteps = mxsteps;
  return 0;
}
extern "C" int STS_ARKodeSetStopTime(void* mem, double tstop)
{
  CHECK_MEM(mem);
  if (sts_mem_kind(mem) == STS_MEM_ARKSTEP) return arkstep_set_stop_time(mem, tstop);
  MEM(mem)->tstop    = tstop;
  MEM(mem)->tstopset = true;
  return 0;
}
extern "C" int STS_LSRKStepSetMixedPrecision(void* mem, int on)
{
  CHECK_MEM(mem);
  if (MEM(mem)->initialized && MEM(mem)->mixed != (on != 0))
  {
    sts_set_error("LSRKStep: precision must be chosen before the first evolve");
    return STS_ILL_INPUT;
  }
  MEM(mem)->mixed = on != 0;
  return 0;
}
extern "C" int STS_LSRKStepSetStageKernel(void* mem, int variant)
{
  CHECK_MEM(mem);
  if (variant < 0 || variant > 1 + TMA_STAGE32_NVARIANTS) return STS_ILL_INPUT;
  LSRKMem* m = MEM(mem);
  if (m->stage_variant != variant)
  {
    for (auto& kv : m->graphs) cudaGraphExecDestroy(kv.second);
    m->graphs.clear();
  }
  m->stage_variant = variant;
  m->tuned         = false;
  return 0;
}

extern "C" int STS_LSRKStepGetStageKernelInfo(void* mem, int* variant, double* ms_per_launch, char* name, int namelen)
{
  CHECK_MEM(mem);
  LSRKMem* m = MEM(mem);
  const int v = m->stage_variant == 0 ? m->tma_variant : (m->stage_variant >= 2 ? m->stage_variant - 2 : -1);
  if (variant) *variant = v;
  if (ms_per_launch) *ms_per_launch = m->tuned ? m->tune_ms[m->tma_variant + 1] : 0.0;
  if (name && namelen > 0)
  {
    const char* nm = m->mixed ? tma_stage32_variant_name(v) : "fp64_register_marching";
    if (m->mixed && m->fuse_ks > 1)
      snprintf(name, namelen, "fused%d_%s (single stages: %s)", m->fuse_ks, tma_fused_config_name(m->fuse_ti), nm);
    else snprintf(name, namelen, "%s", nm);
  }
  return 0;
}

extern "C" int STS_LSRKStepSetStageFusion(void* mem, int ks, int config)
{
  CHECK_MEM(mem);
  if (ks < 0 || ks > 4 || config < 0 || config > TMA_FUSED_NTILES)
  {
    sts_set_error("LSRKStepSetStageFusion: stages per launch 0 (autotuned), 1 (off) or 2-4; tile configuration 0 "
                  "(autotuned) or 1-%d",
                  TMA_FUSED_NTILES);
    return STS_ILL_INPUT;
  }
  LSRKMem* m = MEM(mem);
  for (auto& kv : m->graphs) cudaGraphExecDestroy(kv.second);
  m->graphs.clear();
  m->fuse_req      = ks;
  m->fuse_tile_req = config - 1;
  m->tuned         = false;
  return 0;
}

extern "C" int STS_LSRKStepGetStageFusion(void* mem, int* ks, int* config, int* tile_rows, double* ms_per_launch)
{
  CHECK_MEM(mem);
  LSRKMem* m = MEM(mem);
  const bool on = m->mixed && m->fuse_ks > 1;
  if (ks) *ks = on ? m->fuse_ks : 1;
  if (config) *config = on ? m->fuse_ti + 1 : 0;
  if (tile_rows) *tile_rows = on ? tma_fused_tile_rows(m->fuse_ti) : 0;
  if (ms_per_launch) *ms_per_launch = on ? m->fuse_ms[m->fuse_ti] : 0.0;
  return 0;
}

extern "C" int STS_LSRKStepSetUseGraphs(void* mem, int on)
{
  CHECK_MEM(mem);
  MEM(mem)->use_graphs = on != 0;
  return 0;
}

extern "C" int STS_LSRKStepSetFusedPeriodic(void* mem, int on)
{
  CHECK_MEM(mem);
  MEM(mem)->use_fused_periodic = on != 0;
  return 0;
}

// ARKodeEvolve's return rules (ARKODE's documented behaviour, restated):
//  - a stop time (ARKodeSetStopTime) clips the step that would pass it; the call that ends on
//    it returns y_n with STS_TSTOP_RETURN and clears it;
//  - NORMAL mode steps until t_n >= tout and returns the dense output at tout (tret = tout;
//    a step ending exactly on tout returns y_n); a call whose tout the last step already passed
//    interpolates without stepping;
//  - ONE_STEP mode takes one step and returns y_n, t_n; a call that finds t_n not yet returned
//    (an earlier NORMAL call interpolated behind it) returns it without stepping.
static int lsrk_interp_degree(const LSRKMem* m)
{ // min(q - 1, 5): RKC2, RKL2 and SSP(s,2) 1, SSP(s,3) 2, SSP(10,4) 3
  if (m->ssp && m->method == SSP_S_3) return 2;
  if (m->ssp && m->method == SSP_10_4) return 3;
  return 1;
}

static int lsrk_output(LSRKMem* m, N_Vector yout, double tq, bool interp)
{
  const bool fz      = fused(m) && m->yb[0];
  const double* ycur = fz ? m->yb[m->par] : NVD(m->g_y);
  cudaStream_t st    = m->ctx->stream;
  if (!interp || tq == m->t)
    return STS_CUDA_OK(cudaMemcpyAsync(NVD(yout), ycur, m->n * sizeof(double), cudaMemcpyDeviceToDevice, st))
               ? 0
               : STS_ERR_FAILURE;
  const double tfuzz = 100.0 * DBL_EPSILON * (fabs(m->t) + fabs(m->hlast));
  if (tq < m->t - m->hlast - tfuzz)
  {
    sts_set_error("ARKodeEvolve: tout = %g is behind the last step [%g, %g]", tq, m->t - m->hlast, m->t);
    return STS_ILL_INPUT;
  }
  const double* yold = fz ? m->yb[1 - m->par] : NVD(m->g_yold);
  const double* fold = fz ? m->Fb[1 - m->par] : NVD(m->g_Fold);
  const double* fnew = fz ? m->Fb[m->par] : NVD(m->g_Fn);
  sts_hermite(m->ctx, m->n, lsrk_interp_degree(m), (tq - m->t) / m->hlast, m->hlast, yold, ycur, fold, fnew,
              NVD(yout));
  return STS_CUDA_OK(cudaGetLastError()) ? 0 : STS_ERR_FAILURE;
}

extern "C" int STS_ARKodeEvolve(void* mem, double tout, N_Vector yout, double* tret, int itask)
{
  STS_MARK_REGION("Evolve");
  CHECK_MEM(mem);
  if (itask != STS_NORMAL && itask != STS_ONE_STEP)
  {
    sts_set_error("ARKodeEvolve: itask must be STS_NORMAL or STS_ONE_STEP");
    return STS_ILL_INPUT;
  }
  if (sts_mem_kind(mem) == STS_MEM_ARKSTEP) return arkstep_evolve(mem, tout, yout, tret, itask);
  LSRKMem* m = MEM(mem);
  if (!yout || NVL(yout) != m->n)
  {
    sts_set_error("ARKodeEvolve: output vector length mismatch");
    return STS_ILL_INPUT;
  }
  ctx_activate(m->ctx);
  cudaStream_t st = m->ctx->stream;
  auto finish     = [&](int ret, double tr) {
    if (!STS_CUDA_OK(cudaStreamSynchronize(st))) return (int)STS_ERR_FAILURE;
    if (tret) *tret = tr;
    m->tretlast = tr;
    return ret;
  };
  // calls that return without stepping
  if (m->interp_ready && itask != STS_ONE_STEP && m->t >= tout)
  {
    const int rc = lsrk_output(m, yout, tout, true);
    return rc ? rc : finish(STS_SUCCESS, tout);
  }
  if (m->interp_ready && itask == STS_ONE_STEP && m->t != m->tretlast)
  {
    const int rc = lsrk_output(m, yout, m->t, false);
    return rc ? rc : finish(STS_SUCCESS, m->t);
  }
  if (m->tstopset && m->t >= m->tstop)
  {
    m->tstopset  = false;
    const int rc = lsrk_output(m, yout, m->t, false);
    return rc ? rc : finish(STS_TSTOP_RETURN, m->t);
  }
  // start every evolve from a clean reduction workspace (a failed launch could leave it dirty)
  cudaMemsetAsync(m->ctx->d_work, 0, sizeof(RedWork), st);
  const double clip = m->tstopset ? m->tstop : INFINITY;
  int ret;
  if (fused(m))
  {
    if (!m->yb[0])
    {
      if (m->mixed && ((STS_Problem)m->user_data)->kind == STS_PROBLEM_PERIODIC) return STS_ILL_INPUT;
      if (alloc_fused(m, NVD(m->g_y))) return STS_ERR_FAILURE;
    }
    ret = evolve_fused(m, tout, clip, itask);
  }
  else ret = evolve_generic(m, tout, clip, itask);
  double tr = m->t;
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
  const int rc = lsrk_output(m, yout, tr, interp);
  if (rc) return rc;
  return finish(ret, tr);
}

extern "C" int STS_ARKodeReset(void* mem, double t, N_Vector y)
{
  CHECK_MEM(mem);
  if (sts_mem_kind(mem) == STS_MEM_ARKSTEP) return arkstep_reset(mem, t, y);
  LSRKMem* m = MEM(mem);
  if (!y || NVL(y) != m->n) return STS_ILL_INPUT;
  ctx_activate(m->ctx);
  m->t            = t;
  m->tretlast     = t;
  m->interp_ready = false;
  if (fused(m) && m->yb[0])
  {
    if (!STS_CUDA_OK(cudaMemcpyAsync(m->yb[m->par], NVD(y), m->n * sizeof(double), cudaMemcpyDeviceToDevice,
                                     m->ctx->stream)))
      return STS_ERR_FAILURE;
  }
  else if (!STS_CUDA_OK(cudaMemcpyAsync(NVD(m->g_y), NVD(y), m->n * sizeof(double), cudaMemcpyDeviceToDevice,
                                        m->ctx->stream)))
    return STS_ERR_FAILURE;
  if (m->initialized)
  { // F(t, y) for the restarted state
    if (fused(m))
    {
      STS_Problem p = (STS_Problem)m->user_data;
      sts_rhs_launch(p, m->t, m->yb[m->par], m->Fb[m->par], true, m->ctx->stream);
      if (m->mixed) sts_f64_to_f32(m->ctx, m->Fb[m->par], m->Ffb[m->par], m->n);
    }
    else if (m->rhs(m->t, m->g_y, m->g_Fn, m->user_data) != 0)
      return STS_RHSFUNC_FAIL;
    m->nfe++;
  }
  return STS_CUDA_OK(cudaStreamSynchronize(m->ctx->stream)) ? 0 : STS_ERR_FAILURE;
}

extern "C" int STS_LSRKStepTimeStageKernel(void* mem, int nlaunch, double* ms_per_launch)
{
  CHECK_MEM(mem);
  LSRKMem* m = MEM(mem);
  if (!fused(m) || m->last_s < 2 || nlaunch < 1 || !ms_per_launch) return STS_ILL_INPUT;
  ctx_activate(m->ctx);
  STS_Problem p   = (STS_Problem)m->user_data;
  cudaStream_t st = m->ctx->stream;
  const int j     = m->last_s / 2 > 2 ? m->last_s / 2 : 2;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  // the parameter block of the last step is still on the device
  // fused stages: one launch of the step's stage groups (stages j .. j+ks-1)
  const int ks = (m->mixed && m->fuse_ks > 1 && m->last_s >= m->fuse_ks + 1) ? m->fuse_ks : 1;
  const int jf = (ks > 1 && j + ks - 1 > m->last_s) ? 2 : j;
  auto one = [&](int k) {
    if (ks > 1)
      tma_fused_launch(&m->tma, m->fuse_ti, ks, m->ctx->num_sms, p->dev, dstage(m) + jf, k % 4, (k + 1) % 4, m->par,
                       m->D[(k + 2) % 4], m->D[(k + 3) % 4], m->ctx->d_err, st);
    else if (m->mixed) launch_stage32_idx(m, p, dstage(m) + j, k % 3, (k + 1) % 3, m->par, (k + 2) % 3);
    else launch_stage64(m, p, dstage(m) + j, m->Y[k % 3], m->Y[(k + 1) % 3], m->yb[m->par], m->Fb[m->par], m->Y[(k + 2) % 3]);
  };
  one(0); // warm
  cudaEventRecord(e0, st);
  for (int k = 0; k < nlaunch; ++k) one(k);
  cudaEventRecord(e1, st);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *ms_per_launch = (double)ms / nlaunch;
  return STS_CUDA_OK(cudaGetLastError()) ? 0 : STS_ERR_FAILURE;
}

extern "C" int STS_ARKodeGetStats(void* mem, STS_Stats* s)
{
  CHECK_MEM(mem);
  if (sts_mem_kind(mem) == STS_MEM_ARKSTEP) return arkstep_get_stats(mem, s);
  LSRKMem* m        = MEM(mem);
  s->nst            = m->nst;
  s->nst_attempts   = m->nst_att;
  s->netf           = m->netf;
  s->nfe            = m->nfe;
  s->nfe_dee        = m->nfe_dee;
  s->ndee           = m->ndee;
  s->nst_exp        = m->nst_exp;
  s->stage_max      = m->stage_max;
  s->stages_total   = m->stages_total;
  s->t              = m->t;
  s->hlast          = m->hlast;
  s->hnext          = m->hnext;
  s->spectral_radius = m->rho;
  return 0;
}

// table format of ARKodePrintAllStats (main.cpp:486) for the counters this integrator keeps
extern "C" int STS_ARKodePrintAllStats(void* mem, char* buf, int buflen)
{
  CHECK_MEM(mem);
  if (sts_mem_kind(mem) == STS_MEM_ARKSTEP) return arkstep_print_stats(mem, buf, buflen);
  LSRKMem* m = MEM(mem);
  int k      = snprintf(buf, buflen,
                        "Current time                  = %.16g\n"
                        "Steps                         = %lld\n"
                        "Step attempts                 = %lld\n"
                        "Stability limited steps       = %lld\n"
                        "Error test fails              = %lld\n"
                        "RHS fn evals                  = %lld\n"
                        "Number of dom_eig updates     = %lld\n"
                        "Max. num. of stages used      = %lld\n"
                        "Last step size                = %.16g\n"
                        "Current step size             = %.16g\n",
                        m->t, m->nst, m->nst_att, m->nst_exp, m->netf, m->nfe + m->nfe_dee, m->ndee,
                        m->stage_max, m->hlast, m->hnext);
  return k < buflen ? 0 : -1;
}

extern "C" void STS_ARKodeFree(void** mem)
{
  if (!mem || !*mem) return;
  if (sts_mem_kind(*mem) == STS_MEM_ARKSTEP)
  {
    arkstep_free(*mem);
    *mem = nullptr;
    return;
  }
  LSRKMem* m = MEM(*mem);
  ctx_activate(m->ctx);
  cudaStreamSynchronize(m->ctx->stream);
  free_device(m);
  delete m;
  *mem = nullptr;
}

// ---------------------------------------------------------------------------------------
__global__ void f64_to_f32_kernel(long long n, const double* __restrict__ a, float* __restrict__ b)
{
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += stride) b[k] = (float)a[k];
}

void sts_f64_to_f32(STS_Context ctx, const double* a, float* b, long long n)
{
  f64_to_f32_kernel<<<ew_blocks(ctx, n, 256 * 4), 256, 0, ctx->stream>>>(n, a, b);
}

void sts_hermite_coeffs(int deg, double tau, double h, double a[4])
{
  const double tau2 = tau * tau, tau3 = tau * tau2;
  a[2] = a[3] = 0.0;
  if (deg == 1)
  {
    a[0] = -tau;
    a[1] = 1.0 + tau;
  }
  else if (deg == 2)
  {
    a[0] = tau2;
    a[1] = 1.0 - tau2;
    a[2] = h * (tau2 + tau);
  }
  else
  {
    a[0] = 3.0 * tau2 + 2.0 * tau3;
    a[1] = (1.0 - 3.0 * tau2) - 2.0 * tau3;
    a[2] = h * (tau2 + tau3);
    a[3] = h * ((tau + 2.0 * tau2) + tau3);
  }
}

__global__ void hermite_kernel(long long n, int deg, double a0, double a1, double a2, double a3,
                               const double* __restrict__ yold, const double* __restrict__ ynew,
                               const double* __restrict__ fold, const double* __restrict__ fnew,
                               double* __restrict__ out)
{
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += stride)
  {
    double v = __dmul_rn(a0, yold[k]);
    v        = __fma_rn(a1, ynew[k], v);
    if (deg == 2) v = __fma_rn(a2, fnew[k], v);
    else if (deg == 3)
    {
      v = __fma_rn(a2, fold[k], v);
      v = __fma_rn(a3, fnew[k], v);
    }
    out[k] = v;
  }
}

void sts_hermite(STS_Context ctx, long long n, int deg, double tau, double h, const double* yold,
                 const double* ynew, const double* fold, const double* fnew, double* out)
{
  double a[4];
  sts_hermite_coeffs(deg, tau, h, a);
  hermite_kernel<<<ew_blocks(ctx, n, 256 * 4), 256, 0, ctx->stream>>>(n, deg, a[0], a[1], a[2], a[3], yold, ynew,
                                                                     fold, fnew, out);
}

// ---------------------------------------------------------------------------------------
// checkpoint / restart: the complete integrator state (time, step-size history, controller
// memory, eigenvalue refresh counter and estimate, statistics, y_n, the FSAL F_n and, for the
// mixed path, its FP32 copy, and the power-iteration vector) in one binary file, so that a
// restarted run continues with the same step sequence and the same bits.
// Layout: CkptHeader, then y_n (n doubles), F_n (n doubles, if initialised), F_n FP32
// (n floats, mixed fused path), eigenvector (n doubles, if has_evec). Native endianness.
// ---------------------------------------------------------------------------------------
struct CkptHeader {
  char magic[8];
  int version, method, mixed, fused_path;
  long long n;
  double t, hnext, hlast, rho, ep1, ep2;
  long long ncf, nst, nst_att, netf, nfe, nfe_dee, ndee, nst_exp, stage_max, stages_total, nhist, steps_since_dee;
  int initialized, after_fail, has_evec, last_s;
};
static const char CKPT_MAGIC[8] = {'S', 'T', 'S', 'C', 'K', 'P', 'T', '1'};

static bool ckpt_io(FILE* f, void* host, const void* dev, void* dev_out, size_t bytes, bool write, cudaStream_t st)
{
  if (write)
  {
    if (!STS_CUDA_OK(cudaMemcpyAsync(host, dev, bytes, cudaMemcpyDeviceToHost, st)) ||
        !STS_CUDA_OK(cudaStreamSynchronize(st)))
      return false;
    return fwrite(host, 1, bytes, f) == bytes;
  }
  if (fread(host, 1, bytes, f) != bytes) return false;
  return STS_CUDA_OK(cudaMemcpyAsync(dev_out, host, bytes, cudaMemcpyHostToDevice, st)) &&
         STS_CUDA_OK(cudaStreamSynchronize(st));
}

extern "C" int STS_LSRKStepWriteCheckpoint(void* mem, const char* path)
{
  CHECK_MEM(mem);
  LSRKMem* m = MEM(mem);
  if (!path) return STS_ILL_INPUT;
  ctx_activate(m->ctx);
  cudaStream_t st = m->ctx->stream;
  if (!STS_CUDA_OK(cudaStreamSynchronize(st))) return STS_ERR_FAILURE;
  CkptHeader h;
  memset(&h, 0, sizeof(h));
  memcpy(h.magic, CKPT_MAGIC, 8);
  h.version         = 1;
  h.method          = m->method;
  h.mixed           = m->mixed;
  const bool fz     = fused(m) && m->yb[0] != nullptr;
  h.fused_path      = fz;
  h.n               = m->n;
  h.t               = m->t;
  h.hnext           = m->hnext;
  h.hlast           = m->hlast;
  h.rho             = m->rho;
  h.ep1             = m->ep1;
  h.ep2             = m->ep2;
  h.ncf             = m->ncf;
  h.nst             = m->nst;
  h.nst_att         = m->nst_att;
  h.netf            = m->netf;
  h.nfe             = m->nfe;
  h.nfe_dee         = m->nfe_dee;
  h.ndee            = m->ndee;
  h.nst_exp         = m->nst_exp;
  h.stage_max       = m->stage_max;
  h.stages_total    = m->stages_total;
  h.nhist           = m->nhist;
  h.steps_since_dee = m->steps_since_dee;
  h.initialized     = m->initialized;
  h.after_fail      = m->after_fail;
  h.has_evec        = m->evec != nullptr;
  h.last_s          = m->last_s;
  FILE* f = fopen(path, "wb");
  if (!f)
  {
    sts_set_error("STS_LSRKStepWriteCheckpoint: cannot open %s", path);
    return STS_ILL_INPUT;
  }
  std::vector<char> host((size_t)m->n * sizeof(double));
  bool ok = fwrite(&h, sizeof(h), 1, f) == 1;
  const double* y = fz ? m->yb[m->par] : NVD(m->g_y);
  const double* F = fz ? m->Fb[m->par] : NVD(m->g_Fn);
  ok = ok && ckpt_io(f, host.data(), y, nullptr, m->n * sizeof(double), true, st);
  if (m->initialized) ok = ok && ckpt_io(f, host.data(), F, nullptr, m->n * sizeof(double), true, st);
  if (m->initialized && fz && m->mixed)
    ok = ok && ckpt_io(f, host.data(), m->Ffb[m->par], nullptr, m->n * sizeof(float), true, st);
  if (h.has_evec) ok = ok && ckpt_io(f, host.data(), m->evec, nullptr, m->n * sizeof(double), true, st);
  ok = (fclose(f) == 0) && ok;
  if (!ok) sts_set_error("STS_LSRKStepWriteCheckpoint: write to %s failed", path);
  return ok ? STS_SUCCESS : STS_ERR_FAILURE;
}

extern "C" int STS_LSRKStepReadCheckpoint(void* mem, const char* path)
{
  CHECK_MEM(mem);
  LSRKMem* m = MEM(mem);
  if (!path) return STS_ILL_INPUT;
  ctx_activate(m->ctx);
  cudaStream_t st = m->ctx->stream;
  FILE* f         = fopen(path, "rb");
  if (!f)
  {
    sts_set_error("STS_LSRKStepReadCheckpoint: cannot open %s", path);
    return STS_ILL_INPUT;
  }
  CkptHeader h;
  bool ok = fread(&h, sizeof(h), 1, f) == 1 && memcmp(h.magic, CKPT_MAGIC, 8) == 0 && h.version == 1;
  if (!ok || h.n != m->n || h.method != m->method || h.mixed != (int)m->mixed)
  {
    fclose(f);
    sts_set_error("STS_LSRKStepReadCheckpoint: %s is not a checkpoint of this problem size, method and "
                  "precision",
                  path);
    return STS_ILL_INPUT;
  }
  const bool fz = fused(m);
  if (h.fused_path != (int)fz)
  {
    fclose(f);
    sts_set_error("STS_LSRKStepReadCheckpoint: checkpoint written by the %s path", h.fused_path ? "fused" : "generic");
    return STS_ILL_INPUT;
  }
  if (fz && !m->yb[0] && alloc_fused(m, NVD(m->g_y)))
  {
    fclose(f);
    return STS_ERR_FAILURE;
  }
  m->par       = 0;
  double* y    = fz ? m->yb[0] : NVD(m->g_y);
  double* F    = fz ? m->Fb[0] : NVD(m->g_Fn);
  std::vector<char> host((size_t)m->n * sizeof(double));
  ok = ckpt_io(f, host.data(), nullptr, y, m->n * sizeof(double), false, st);
  if (h.initialized) ok = ok && ckpt_io(f, host.data(), nullptr, F, m->n * sizeof(double), false, st);
  if (h.initialized && fz && h.mixed)
    ok = ok && ckpt_io(f, host.data(), nullptr, m->Ffb[0], m->n * sizeof(float), false, st);
  if (ok && h.has_evec)
  {
    if (!m->evec && !STS_CUDA_OK(cudaMalloc(&m->evec, m->n * sizeof(double)))) ok = false;
    ok = ok && ckpt_io(f, host.data(), nullptr, m->evec, m->n * sizeof(double), false, st);
  }
  fclose(f);
  if (!ok)
  {
    sts_set_error("STS_LSRKStepReadCheckpoint: %s is truncated or unreadable", path);
    return STS_ERR_FAILURE;
  }
  m->t               = h.t;
  m->hnext           = h.hnext;
  m->hlast           = h.hlast;
  m->rho             = h.rho;
  m->ep1             = h.ep1;
  m->ep2             = h.ep2;
  m->ncf             = h.ncf;
  m->nst             = h.nst;
  m->nst_att         = h.nst_att;
  m->netf            = h.netf;
  m->nfe             = h.nfe;
  m->nfe_dee         = h.nfe_dee;
  m->ndee            = h.ndee;
  m->nst_exp         = h.nst_exp;
  m->stage_max       = h.stage_max;
  m->stages_total    = h.stages_total;
  m->nhist           = h.nhist;
  m->steps_since_dee = h.steps_since_dee;
  m->initialized     = h.initialized != 0;
  m->after_fail      = h.after_fail != 0;
  m->last_s          = h.last_s;
  m->interp_ready    = false; // the checkpoint holds y_n only
  m->tretlast        = m->t;
  return STS_SUCCESS;
}

// LSRKStepSetNumDomEigEstInitPreprocessIters / LSRKStepSetNumDomEigEstPreprocessIters
// (gkeyll_diffusion/gk_diffusion_1x1v_p1.c:873-885): power iterations run before the first
// and before every later dominant-eigenvalue estimate
extern "C" int STS_LSRKStepSetNumDomEigEstInitPreprocessIters(void* mem, int iters)
{
  CHECK_MEM(mem);
  MEM(mem)->dee_init_warmups = iters > 0 ? iters : 0;
  return STS_SUCCESS;
}

extern "C" int STS_LSRKStepSetNumDomEigEstPreprocessIters(void* mem, int iters)
{
  CHECK_MEM(mem);
  MEM(mem)->dee_succ_warmups = iters > 0 ? iters : 0;
  return STS_SUCCESS;
}

// host helper: the SSP method's weights b, stage times c and error weights w = b - bhat
extern "C" int STS_LSRKSSPWeights(int type, int s, double* b, double* c, double* w)
{
  if ((type != SSP_S_2 && type != SSP_S_3 && type != SSP_10_4) || !ssp_stages_valid(type, s) || !b || !c || !w)
    return STS_ILL_INPUT;
  std::vector<double> A, bb, cc, ww;
  ssp_tableau(type, s, A, bb, cc, ww);
  for (int k = 0; k < s; ++k)
  {
    b[k] = bb[k];
    c[k] = cc[k];
    w[k] = ww[k];
  }
  return 0;
}
