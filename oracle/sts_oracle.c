/* CPU oracle for the diffusion_2D super-time-stepping path — TEST INFRASTRUCTURE ONLY.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load this file's
 * shared library; the CUDA product never calls it. See sts_oracle.h for the parity status
 * (SUNDIALS parity unpinned: deps/sundials is an empty submodule in the reference).
 *
 * Arithmetic contract. Every floating-point expression that the CUDA kernels also
 * evaluate is written here in the same order with explicit fma()/fmaf(), and the file is
 * compiled with -ffp-contract=off, so the GPU FP64 and mixed paths can be compared bit for
 * bit. Reductions use an exact fixed-point accumulator (every term truncated to a multiple
 * of 2^-160, summed exactly, rounded once), so their value does not depend on the order of
 * summation, the thread count or the GPU launch shape.
 */
#include "sts_oracle.h"

#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define PI 3.14159265358979323846

int orc_nthreads(void)
{
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* threads of the oracle's parallel loops from here on (1: the reference's serial run) */
void orc_set_nthreads(int n)
{
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

/* ------------------------------------------------------------------------------------
 * Exact accumulation. Replaces the MPI_Allreduce-backed sums of NVECTOR_PARALLEL and the
 * gkyl_array_reduce_range + gkyl_comm_allreduce pair of nvector_gkylzero.c:234-404.
 * ----------------------------------------------------------------------------------*/
#define XW 5 /* 320-bit accumulators: grid 2^-160, terms below 2^128 */
typedef struct {
  uint64_t p[XW], n[XW];
  int nan, ovf;
} xacc;

static void xacc_zero(xacc* a) { memset(a, 0, sizeof(*a)); }

static void add_at(uint64_t a[XW], int k, uint64_t lo, uint64_t hi)
{
  unsigned __int128 s = (unsigned __int128)a[k] + lo;
  a[k]                = (uint64_t)s;
  uint64_t carry      = (uint64_t)(s >> 64);
  for (int m = k + 1; m < XW; ++m)
  {
    uint64_t add = (m == k + 1) ? hi : 0;
    s            = (unsigned __int128)a[m] + add + carry;
    a[m]         = (uint64_t)s;
    carry        = (uint64_t)(s >> 64);
  }
}

static void xacc_add(xacc* a, double x)
{
  uint64_t b;
  memcpy(&b, &x, 8);
  int neg    = (int)(b >> 63);
  int e      = (int)((b >> 52) & 0x7ff);
  uint64_t m = b & ((1ULL << 52) - 1);
  int exp2;
  if (e == 0x7ff)
  {
    if (m) a->nan = 1;
    else a->ovf = 1;
    return;
  }
  if (e == 0)
  {
    if (m == 0) return;
    exp2 = -1074;
  }
  else
  {
    m |= (1ULL << 52);
    exp2 = e - 1075;
  }
  if (exp2 + 53 > 128)
  { /* |x| >= 2^128: outside the accumulator's range */
    a->ovf = 1;
    return;
  }
  int sh = exp2 + 160;
  uint64_t lo, hi;
  int k;
  if (sh < 0)
  {
    if (sh <= -64) return;
    lo = m >> (-sh);
    hi = 0;
    k  = 0;
  }
  else
  {
    k       = sh >> 6;
    int bsh = sh & 63;
    lo      = m << bsh;
    hi      = bsh ? (m >> (64 - bsh)) : 0;
  }
  add_at(neg ? a->n : a->p, k, lo, hi);
}

static void xacc_merge(xacc* a, const xacc* b)
{
  for (int k = 0; k < XW; ++k)
  {
    add_at(a->p, k, b->p[k], 0);
    add_at(a->n, k, b->n[k], 0);
  }
  a->nan |= b->nan;
  a->ovf |= b->ovf;
}

static double xacc_result(const xacc* a)
{
  if (a->nan) return NAN;
  if (a->ovf) return INFINITY;
  /* d = p - n in two's complement */
  uint64_t d[XW];
  unsigned __int128 borrow = 0;
  for (int k = 0; k < XW; ++k)
  {
    unsigned __int128 s = (unsigned __int128)a->p[k] - a->n[k] - borrow;
    d[k]                = (uint64_t)s;
    borrow              = (s >> 64) ? 1 : 0;
  }
  double sign = 1.0;
  if (d[XW - 1] >> 63)
  {
    sign = -1.0;
    unsigned __int128 c = 1;
    for (int k = 0; k < XW; ++k)
    {
      unsigned __int128 s = (unsigned __int128)(~d[k]) + c;
      d[k]                = (uint64_t)s;
      c                   = s >> 64;
    }
  }
  int top = -1;
  for (int k = XW - 1; k >= 0; --k)
    if (d[k])
    {
      top = k * 64 + 63 - __builtin_clzll(d[k]);
      break;
    }
  if (top < 0) return 0.0;
  if (top <= 52) return sign * ldexp((double)d[0], -160);
  int shift = top - 52;
  /* mantissa = bits [shift, top] */
  uint64_t mant;
  {
    int k = shift >> 6, bsh = shift & 63;
    mant = d[k] >> bsh;
    if (bsh && k + 1 < XW) mant |= d[k + 1] << (64 - bsh);
    mant &= ((1ULL << 53) - 1);
  }
  int rpos   = shift - 1;
  int rbit   = (int)((d[rpos >> 6] >> (rpos & 63)) & 1);
  int sticky = 0;
  for (int k = 0; k <= (rpos >> 6) && !sticky; ++k)
  {
    uint64_t w = d[k];
    if (k == (rpos >> 6)) w &= ((rpos & 63) ? ((1ULL << (rpos & 63)) - 1) : 0);
    if (w) sticky = 1;
  }
  if (rbit && (sticky || (mant & 1)))
  {
    mant++;
    if (mant == (1ULL << 53))
    {
      mant >>= 1;
      shift++;
    }
  }
  return sign * ldexp((double)mant, shift - 160);
}

/* Parallel exact reductions; the value is independent of the thread partition. */
#define XREDUCE(N, TERM)                                       \
  xacc tot;                                                    \
  xacc_zero(&tot);                                             \
  _Pragma("omp parallel")                                      \
  {                                                            \
    xacc loc;                                                  \
    xacc_zero(&loc);                                           \
    _Pragma("omp for schedule(static)") for (long i = 0; i < (N); ++i) \
    {                                                          \
      xacc_add(&loc, (TERM));                                  \
    }                                                          \
    _Pragma("omp critical") xacc_merge(&tot, &loc);            \
  }

double orc_xsum(const double* x, long n)
{
  XREDUCE(n, x[i]);
  return xacc_result(&tot);
}

/* N_VDotProd (nvector_gkylzero.c:349-404): sum_i x_i*y_i */
double orc_xdot(const double* x, const double* y, long n)
{
  XREDUCE(n, x[i] * y[i]);
  return xacc_result(&tot);
}

/* N_VWrmsNorm (nvector_gkylzero.c:234-290): sqrt(sum (x_i w_i)^2 / n) */
double orc_wrms(const double* x, const double* w, long n)
{
  double s;
  {
    XREDUCE(n, (x[i] * w[i]) * (x[i] * w[i]));
    s = xacc_result(&tot);
  }
  return sqrt(s / (double)n);
}

/* N_VMaxNorm (nvector_gkylzero.c:453-498) */
double orc_maxnorm(const double* x, long n)
{
  double m = 0.0;
  int nan  = 0;
  for (long i = 0; i < n; ++i)
  {
    double a = fabs(x[i]);
    if (a != a) nan = 1;
    if (a > m) m = a;
  }
  return nan ? NAN : m;
}

/* ------------------------------------------------------------------------------------
 * Problem definition.
 *   manufactured: u = S(x)S(y)c(t), S = sin^2(pi .), c = cos^2(2 pi t),
 *                 b = S S c' - c (kx S'' S + ky S S''), S'' = 2 pi^2 cos(2 pi .)
 *                 (form of diffusion_2D/README.md:13-34 with the cos^2(2 pi t) time factor)
 *   grid:         N interior nodes per direction on [0,1], d = 1/(N+1), x_i = (i+1) d
 *   periodic:     diffusion_2D.cpp:155-160 (d = (xu-xl)/(n-1)), initial.cpp:42-43,
 *                 Diffusion_Coeff_X/Y diffusion_2D.cpp:887-897
 * ----------------------------------------------------------------------------------*/
double orc_c(double t)
{
  double cs = cos(2.0 * PI * t);
  return cs * cs;
}

double orc_cdot(double t) { return -2.0 * PI * sin(4.0 * PI * t); }

static void manufactured_tables(int n, double d, double* S, double* Sdd)
{
  for (int i = 0; i < n; ++i)
  {
    double x = (i + 1) * d;
    double s = sin(PI * x);
    S[i]     = s * s;
    Sdd[i]   = 2.0 * PI * PI * cos(2.0 * PI * x);
  }
}

static double coeff(double k, double x, int inhom)
{
  return inhom ? (k * (1.0 + 0.99 * sin(x))) : k;
}

orc_prob* orc_prob_create(int kind, int nx, int ny, double kx, double ky, int inhomogeneous,
                          double xl, double xu, double yl, double yu)
{
  if (nx < 1 || ny < 1) return NULL;
  orc_prob* p = (orc_prob*)calloc(1, sizeof(orc_prob));
  p->nx = nx;
  p->ny = ny;
  p->kind = kind;
  p->kx   = kx;
  p->ky   = ky;
  p->inhomogeneous = (kind == ORC_PERIODIC) ? inhomogeneous : 0;
  if (kind == ORC_PERIODIC)
  {
    p->xl = xl;
    p->xu = xu;
    p->yl = yl;
    p->yu = yu;
    p->dx = (xu - xl) / (nx - 1);
    p->dy = (yu - yl) / (ny - 1);
  }
  else
  {
    p->xl = 0.0;
    p->xu = 1.0;
    p->yl = 0.0;
    p->yu = 1.0;
    p->dx = 1.0 / (nx + 1);
    p->dy = 1.0 / (ny + 1);
  }
  p->cx  = kx / (p->dx * p->dx);
  p->cy  = ky / (p->dy * p->dy);
  p->cc  = -2.0 * (p->cx + p->cy);
  p->Sx  = (double*)calloc(nx, sizeof(double));
  p->Sxx = (double*)calloc(nx, sizeof(double));
  p->Sy  = (double*)calloc(ny, sizeof(double));
  p->Syy = (double*)calloc(ny, sizeof(double));
  manufactured_tables(nx, p->dx, p->Sx, p->Sxx);
  manufactured_tables(ny, p->dy, p->Sy, p->Syy);
  p->Dxw = (double*)calloc(nx, sizeof(double));
  p->Dxe = (double*)calloc(nx, sizeof(double));
  p->Dys = (double*)calloc(ny, sizeof(double));
  p->Dyn = (double*)calloc(ny, sizeof(double));
  for (int i = 0; i < nx; ++i)
  { /* diffusion.cpp:43-46 (global index, is = 0) */
    double xlo = p->xl + (i - 0.5) * p->dx, xhi = p->xl + (i + 0.5) * p->dx;
    p->Dxw[i]  = coeff(kx, xlo, p->inhomogeneous) / (p->dx * p->dx);
    p->Dxe[i]  = coeff(kx, xhi, p->inhomogeneous) / (p->dx * p->dx);
  }
  for (int j = 0; j < ny; ++j)
  { /* diffusion.cpp:36-39 */
    double ylo = p->yl + (j - 0.5) * p->dy, yhi = p->yl + (j + 0.5) * p->dy;
    p->Dys[j]  = coeff(ky, ylo, p->inhomogeneous) / (p->dy * p->dy);
    p->Dyn[j]  = coeff(ky, yhi, p->inhomogeneous) / (p->dy * p->dy);
  }
  return p;
}

void orc_prob_free(orc_prob* p)
{
  if (!p) return;
  free(p->Sx);
  free(p->Sxx);
  free(p->Sy);
  free(p->Syy);
  free(p->Dxw);
  free(p->Dxe);
  free(p->Dys);
  free(p->Dyn);
  free(p);
}

void orc_initial(const orc_prob* p, double* u)
{
  long nx = p->nx;
  for (long j = 0; j < p->ny; ++j)
    for (long i = 0; i < nx; ++i)
    {
      if (p->kind == ORC_PERIODIC)
      { /* initial.cpp:39-43 */
        double x     = p->xl + i * p->dx;
        double y     = p->yl + j * p->dy;
        u[j * nx + i] = (1.0 + 0.3 * sin(2.0 * x)) / sqrt(5.5 * PI) * exp(-(y * y) / 5.5);
      }
      else u[j * nx + i] = p->Sx[i] * p->Sy[j];
    }
}

/* sum_k a_k sin(p_k pi x) sin(q_k pi y) (batched initial condition) */
void orc_initial_modes(const orc_prob* p, int nmodes, const int* pm, const int* qm,
                       const double* amp, double* u)
{
  long nx = p->nx;
  for (long j = 0; j < p->ny; ++j)
    for (long i = 0; i < nx; ++i)
    {
      double x = (i + 1) * p->dx, y = (j + 1) * p->dy, v = 0.0;
      for (int k = 0; k < nmodes; ++k) v += amp[k] * sin(pm[k] * PI * x) * sin(qm[k] * PI * y);
      u[j * nx + i] = v;
    }
}

void orc_exact(const orc_prob* p, double t, double* u)
{
  double c = orc_c(t);
  long nx  = p->nx;
  for (long j = 0; j < p->ny; ++j)
    for (long i = 0; i < nx; ++i) u[j * nx + i] = (p->Sx[i] * p->Sy[j]) * c;
}

/* Forcing tables for a scale hm at time t: b*hm at (i,j) = Sy_j P_i + Syy_j Q_i. */
static void forcing_scalars(const orc_prob* p, double hm, double t, double* al, double* be,
                            double* ga)
{
  double c  = orc_c(t);
  double cd = orc_cdot(t);
  *al       = hm * cd;
  *be       = -(hm * c) * p->kx;
  *ga       = -(hm * c) * p->ky;
}

/* Kernel-form RHS F(t,u) = A u + b(t) (the arithmetic of the CUDA RHS kernel). */
static inline double lap_point(const orc_prob* p, const double* u, long i, long j)
{
  long nx = p->nx, ny = p->ny;
  double uc = u[j * nx + i];
  double uw = (i > 0) ? u[j * nx + i - 1] : 0.0;
  double ue = (i < nx - 1) ? u[j * nx + i + 1] : 0.0;
  double us = (j > 0) ? u[(j - 1) * nx + i] : 0.0;
  double un = (j < ny - 1) ? u[(j + 1) * nx + i] : 0.0;
  double sx = uw + ue, sy = us + un;
  double acc = p->cc * uc;
  acc        = fma(p->cx, sx, acc);
  acc        = fma(p->cy, sy, acc);
  return acc;
}

void orc_rhs(const orc_prob* p, double t, const double* u, double* f)
{
  if (p->kind == ORC_PERIODIC)
  {
    orc_rhs_ref(p, t, u, f);
    return;
  }
  long nx = p->nx, ny = p->ny;
  double al, be, ga;
  forcing_scalars(p, 1.0, t, &al, &be, &ga);
  int forced = (p->kind == ORC_MANUFACTURED);
#pragma omp parallel for schedule(static)
  for (long j = 0; j < ny; ++j)
    for (long i = 0; i < nx; ++i)
    {
      double acc = lap_point(p, u, i, j);
      if (forced)
      {
        double P = fma(al, p->Sx[i], be * p->Sxx[i]);
        double Q = ga * p->Sx[i];
        acc      = fma(p->Sy[j], P, acc);
        acc      = fma(p->Syy[j], Q, acc);
      }
      f[j * nx + i] = acc;
    }
}

/* Literal restatement of laplacian() (diffusion.cpp:9-209): f = -((Dxw+Dxe)+(Dys+Dyn)) u
 * + Dxw uW + Dxe uE + Dys uS + Dyn uN, neighbours periodic (kind PERIODIC) or zero
 * (Dirichlet kinds), plus the manufactured forcing where present. */
void orc_rhs_ref(const orc_prob* p, double t, const double* u, double* f)
{
  long nx = p->nx, ny = p->ny;
  int per = (p->kind == ORC_PERIODIC);
#pragma omp parallel for schedule(static)
  for (long j = 0; j < ny; ++j)
    for (long i = 0; i < nx; ++i)
    {
      long iw = i - 1, ie = i + 1, js = j - 1, jn = j + 1;
      double uw, ue, us, un;
      if (per)
      {
        uw = u[j * nx + (iw < 0 ? nx - 1 : iw)];
        ue = u[j * nx + (ie >= nx ? 0 : ie)];
        us = u[(js < 0 ? ny - 1 : js) * nx + i];
        un = u[(jn >= ny ? 0 : jn) * nx + i];
      }
      else
      {
        uw = iw >= 0 ? u[j * nx + iw] : 0.0;
        ue = ie < nx ? u[j * nx + ie] : 0.0;
        us = js >= 0 ? u[js * nx + i] : 0.0;
        un = jn < ny ? u[jn * nx + i] : 0.0;
      }
      double Dxw = per ? p->Dxw[i] : p->cx, Dxe = per ? p->Dxe[i] : p->cx;
      double Dys = per ? p->Dys[j] : p->cy, Dyn = per ? p->Dyn[j] : p->cy;
      double v = -((Dxw + Dxe) + (Dys + Dyn)) * u[j * nx + i];
      v        = v + Dxw * uw;
      v        = v + Dxe * ue;
      v        = v + Dys * us;
      v        = v + Dyn * un;
      if (p->kind == ORC_MANUFACTURED)
      {
        double c = orc_c(t), cd = orc_cdot(t);
        v += p->Sx[i] * p->Sy[j] * cd - c * (p->kx * p->Sxx[i] * p->Sy[j] + p->ky * p->Sx[i] * p->Syy[j]);
      }
      f[j * nx + i] = v;
    }
}

/* Jacobian-vector product J v = A v (the RHS is affine in u). */
void orc_apply_A(const orc_prob* p, const double* v, double* w)
{
  long nx = p->nx, ny = p->ny;
  if (p->kind == ORC_PERIODIC)
  {
    orc_prob q = *p;
    q.kind     = ORC_PERIODIC;
    orc_rhs_ref(&q, 0.0, v, w);
    return;
  }
#pragma omp parallel for schedule(static)
  for (long j = 0; j < ny; ++j)
    for (long i = 0; i < nx; ++i) w[j * nx + i] = lap_point(p, v, i, j);
}

/* dom_eig (main.cpp:536-550): lambda = -8 max(kx/dx^2, ky/dy^2) */
double orc_dom_eig(const orc_prob* p)
{
  double a = p->kx / p->dx / p->dx, b = p->ky / p->dy / p->dy;
  return -8.0 * (a > b ? a : b);
}

/* Power iteration (SUNDomEigEstimator_Power(u, maxiters, reltol), main.cpp:344):
 * v <- v/||v||; repeat: w = A v; lambda = v.w; stop when |lambda - lambda_old| <
 * reltol |lambda|; v <- w / ||w||. Returns the number of iterations (A products). */
int orc_power_iteration(const orc_prob* p, double* v, int maxiters, double reltol, double* lambda)
{
  long n    = (long)p->nx * p->ny;
  double* w = (double*)malloc(n * sizeof(double));
  double nrm = sqrt(orc_xdot(v, v, n));
  if (!(nrm > 0.0))
  {
    for (long i = 0; i < n; ++i) v[i] = 1.0;
    nrm = sqrt(orc_xdot(v, v, n));
  }
  double inv = 1.0 / nrm;
  for (long i = 0; i < n; ++i) v[i] = inv * v[i];
  double lam = 0.0, lam_old = 0.0;
  int k;
  for (k = 1; k <= maxiters; ++k)
  {
    orc_apply_A(p, v, w);
    lam = orc_xdot(v, w, n);
    double wn = sqrt(orc_xdot(w, w, n));
    double wi = 1.0 / wn;
    for (long i = 0; i < n; ++i) v[i] = wi * w[i];
    if (k > 1 && fabs(lam - lam_old) < reltol * fabs(lam)) break;
    lam_old = lam;
  }
  if (k > maxiters) k = maxiters;
  free(w);
  *lambda = lam;
  return k;
}

/* ------------------------------------------------------------------------------------
 * LSRKStep STS methods, restated.
 *   RKC2: Sommeijer, Shampine & Verwer (1998), damping eps = 2/13; coefficient recurrence
 *         and stage count 1 + floor(sqrt(1 + 1.54 h rho)) as in the published rkc.f.
 *   RKL2: Meyer, Balsara & Aslam (2014). Stage count ceil((sqrt(9 + 8 h rho) - 1)/2).
 * Arrays are indexed by stage j = 1..s; entry 0 unused. cjm1[j] is the time fraction of
 * Y_{j-1} (where F is evaluated for stage j).
 * ----------------------------------------------------------------------------------*/
int orc_stage_coeffs(int method, int s, double* mu, double* nu, double* mus, double* ajm1,
                     double* cjm1)
{
  if (s < 2) return -1;
  if (method == 0)
  {
    double sd    = (double)s;
    double w0    = 1.0 + 2.0 / (13.0 * (sd * sd));
    double temp1 = w0 * w0 - 1.0;
    double temp2 = sqrt(temp1);
    double arg   = sd * log(w0 + temp2);
    double w1    = sinh(arg) * temp1 / (cosh(arg) * sd * temp2 - w0 * sinh(arg));
    double bjm1  = 1.0 / ((2.0 * w0) * (2.0 * w0));
    double bjm2  = bjm1;
    mu[1]   = 0.0;
    nu[1]   = 0.0;
    mus[1]  = w1 * bjm1;
    ajm1[1] = 0.0;
    cjm1[1] = 0.0;
    double thjm2 = 0.0, thjm1 = mus[1];
    double zjm1 = w0, zjm2 = 1.0, dzjm1 = 1.0, dzjm2 = 0.0, d2zjm1 = 0.0, d2zjm2 = 0.0;
    for (int j = 2; j <= s; ++j)
    {
      double zj   = 2.0 * w0 * zjm1 - zjm2;
      double dzj  = 2.0 * w0 * dzjm1 - dzjm2 + 2.0 * zjm1;
      double d2zj = 2.0 * w0 * d2zjm1 - d2zjm2 + 4.0 * dzjm1;
      double bj   = d2zj / (dzj * dzj);
      double a    = 1.0 - zjm1 * bjm1;
      double m    = 2.0 * w0 * bj / bjm1;
      double n    = -bj / bjm2;
      double ms   = m * w1 / w0;
      mu[j]   = m;
      nu[j]   = n;
      mus[j]  = ms;
      ajm1[j] = a;
      cjm1[j] = thjm1;
      double thj = m * thjm1 + n * thjm2 + ms * (1.0 - a);
      thjm2      = thjm1;
      thjm1      = thj;
      bjm2       = bjm1;
      bjm1       = bj;
      zjm2       = zjm1;
      zjm1       = zj;
      dzjm2      = dzjm1;
      dzjm1      = dzj;
      d2zjm2     = d2zjm1;
      d2zjm1     = d2zj;
    }
  }
  else
  {
    double sd   = (double)s;
    double w1   = 4.0 / ((sd + 2.0) * (sd - 1.0));
    double bjm2 = 1.0 / 3.0, bjm1 = 1.0 / 3.0;
    mu[1]   = 0.0;
    nu[1]   = 0.0;
    mus[1]  = w1 * bjm1;
    ajm1[1] = 0.0;
    cjm1[1] = 0.0;
    double cj1 = mus[1];
    for (int j = 2; j <= s; ++j)
    {
      double jd   = (double)j;
      double temj = (jd + 2.0) * (jd - 1.0);
      double cj   = temj * w1 / 4.0;
      double bj   = temj / (2.0 * jd * (jd + 1.0));
      double a    = 1.0 - bjm1;
      double m    = (2.0 * jd - 1.0) / jd * (bj / bjm1);
      double n    = -(jd - 1.0) / jd * (bj / bjm2);
      mu[j]   = m;
      nu[j]   = n;
      mus[j]  = w1 * m;
      ajm1[j] = a;
      cjm1[j] = cj1;
      cj1     = cj;
      bjm2    = bjm1;
      bjm1    = bj;
    }
  }
  return 0;
}

/* Stage count for h and spectral radius rho; *hmax = the largest h the stage limit admits
 * (0.96 * (smax^2-1)/(1.54 rho) for RKC, 0.96 * (smax^2+smax-2)/(2 rho) for RKL). */
int orc_stages_needed(int method, double h, double rho, int smax, double* hmax)
{
  double ss;
  double sm = (double)smax;
  if (method == 0)
  {
    ss    = 1.0 + floor(sqrt(1.0 + 1.54 * h * rho));
    *hmax = (rho > 0.0) ? 0.96 * (sm * sm - 1.0) / (1.54 * rho) : INFINITY;
  }
  else
  {
    ss    = ceil((sqrt(9.0 + 8.0 * h * rho) - 1.0) / 2.0);
    *hmax = (rho > 0.0) ? 0.96 * (sm * sm + sm - 2.0) / (2.0 * rho) : INFINITY;
  }
  /* a non-finite step (NaN state) gives the 2-stage minimum, as max(ss, 2) does */
  if (!(ss >= 2.0)) ss = 2.0;
  if (ss > 1e9) ss = 1e9;
  return (int)ss;
}

/* ARKODE-style controllers (SUNAdaptController PID/PI/I), error bias 1.5, method order
 * ord = p + 1 = 3 (the RKC/RKL embedding estimates an O(h^3) local error). The history
 * length nhist selects I -> PI -> PID forms on the first steps. */
#define ORD 3.0
#define BIAS 1.5
#define TINYE 1.0e-10
/* Deterministic pow for the controllers, restated from the product's portable math (the
 * same IEEE operation sequence runs in the device batch kernel): log x = k ln2 + 2 atanh(f),
 * x = m 2^k, m in [sqrt(1/2), sqrt(2)), f = (m-1)/(m+1), series to f^25; exp y = 2^k e^r,
 * k = rint(y / ln2), r = y - k ln2 (two-part ln2), Taylor series to r^17/17!. */
static const double ORC_LN2_HI = 0.6931471805599453094, ORC_LN2_LO = 2.3190468138462996e-17,
                    ORC_INV_LN2 = 1.4426950408889634074;

static double orc_log(double x)
{
  if (!(x > 0.0)) return x == 0.0 ? -HUGE_VAL : NAN;
  if (x == HUGE_VAL) return x;
  int k    = 0;
  double m = frexp(x, &k);
  if (m < 0.70710678118654752440)
  {
    m = m * 2.0;
    k = k - 1;
  }
  double f = (m - 1.0) / (m + 1.0), f2 = f * f, s = 1.0 / 25.0;
  for (int i = 11; i >= 0; --i) s = fma(s, f2, 1.0 / (double)(2 * i + 1));
  double lm = 2.0 * f * s, kd = (double)k;
  return fma(kd, ORC_LN2_HI, fma(kd, ORC_LN2_LO, lm));
}

static double orc_exp(double y)
{
  if (y != y) return y;
  if (y > 709.78) return HUGE_VAL;
  if (y < -745.2) return 0.0;
  double k = rint(y * ORC_INV_LN2);
  double r = fma(-k, ORC_LN2_HI, y);
  r        = fma(-k, ORC_LN2_LO, r);
  double c[18];
  c[0] = 1.0;
  for (int i = 1; i < 18; ++i) c[i] = c[i - 1] / (double)i;
  double s = c[17];
  for (int i = 16; i >= 0; --i) s = fma(s, r, c[i]);
  return ldexp(s, (int)k);
}

double orc_pow(double x, double y) { return orc_exp(y * orc_log(x)); }

static double controller_ord(int controller, double h, double dsm, double ep1, double ep2, double hp, long nhist,
                             double ORDV);

double orc_controller(int controller, double h, double dsm, double ep1, double ep2, double hp, long nhist)
{
  return controller_ord(controller, h, dsm, ep1, ep2, hp, nhist, ORD);
}

/* the controllers for an error estimate of order ORDV (3 for the STS embedding); hp is the
 * previous accepted step size (used by the implicit Gustafsson controller). ARKODE's
 * controller set, diffusion_2D/main.cpp:366-376: PID, PI, I (Soderlind-form exponents, the
 * leading terms only until enough history exists) and Gustafsson's explicit (1991), implicit
 * (1994) and combined controllers:
 *   ExpGus  h' = h e_n^(-k1/p) (e_n/e_{n-1})^(-k2/p),               k1 0.367, k2 0.268
 *   ImpGus  h' = h (h/h_{n-1}) e_n^(-k1/p) (e_n/e_{n-1})^(-k2/p),   k1 0.98,  k2 0.95
 *   ImExGus h' = min(ExpGus, ImpGus) with those two parameter pairs
 * with h' = h e_n^(-1/p) on the first step; e = bias * dsm, floored at 1e-10. */
static double controller_ord(int controller, double h, double dsm, double ep1, double ep2, double hp, long nhist,
                             double ORDV)
{
#undef ORD
#define ORD ORDV
  double e1 = BIAS * dsm;
  if (e1 < TINYE) e1 = TINYE;
  double e2 = BIAS * ep1;
  if (e2 < TINYE) e2 = TINYE;
  double e3 = BIAS * ep2;
  if (e3 < TINYE) e3 = TINYE;
  if (controller == 0)
  {
    if (nhist < 1) return h * orc_pow(e1, -0.58 / ORD);
    if (nhist < 2) return h * orc_pow(e1, -0.58 / ORD) * orc_pow(e2, 0.21 / ORD);
    return h * orc_pow(e1, -0.58 / ORD) * orc_pow(e2, 0.21 / ORD) * orc_pow(e3, -0.1 / ORD);
  }
  if (controller == 1)
  {
    if (nhist < 1) return h * orc_pow(e1, -0.8 / ORD);
    return h * orc_pow(e1, -0.8 / ORD) * orc_pow(e2, 0.31 / ORD);
  }
  if (controller >= 3 && controller <= 5 && nhist >= 1 && hp > 0.0)
  {
    const double r    = e1 / e2;
    const double hexp = h * orc_pow(e1, -0.367 / ORD) * orc_pow(r, -0.268 / ORD);
    if (controller == 3) return hexp;
    const double himp = h * (h / hp) * orc_pow(e1, -0.98 / ORD) * orc_pow(r, -0.95 / ORD);
    if (controller == 4) return himp;
    return hexp < himp ? hexp : himp;
  }
  return h * orc_pow(e1, -1.0 / ORD);
#undef ORD
#define ORD 3.0
}

#define SAFETY 0.96
#define GROWTH 20.0
#define ETAMX1 10000.0
#define ETAMXF 0.3
#define ETAMIN 0.1
#define SMALL_NEF 2
#define LBOUND 1.0
#define UBOUND 1.5

void orc_state_init(orc_state* st, double t0)
{
  memset(st, 0, sizeof(*st));
  st->t = t0;
}

void orc_state_free(orc_state* st)
{
  free(st->F);
  free(st->Ff);
  free(st->evec);
  free(st->d.ycur);
  free(st->d.yold);
  free(st->d.fold);
  st->F      = NULL;
  st->Ff     = NULL;
  st->evec   = NULL;
  st->d.ycur = st->d.yold = st->d.fold = NULL;
}

/* ---- stop time and dense output (csrc/lsrk.cu STS_ARKodeEvolve, sts_hermite) ---- */
void orc_hermite(long n, int deg, double tau, double h, const double* yold, const double* ynew,
                 const double* fold, const double* fnew, double* out)
{
  const double tau2 = tau * tau, tau3 = tau * tau2;
  double a0, a1, a2 = 0.0, a3 = 0.0;
  if (deg == 1)
  {
    a0 = -tau;
    a1 = 1.0 + tau;
  }
  else if (deg == 2)
  {
    a0 = tau2;
    a1 = 1.0 - tau2;
    a2 = h * (tau2 + tau);
  }
  else
  {
    a0 = 3.0 * tau2 + 2.0 * tau3;
    a1 = (1.0 - 3.0 * tau2) - 2.0 * tau3;
    a2 = h * (tau2 + tau3);
    a3 = h * ((tau + 2.0 * tau2) + tau3);
  }
  for (long k = 0; k < n; ++k)
  {
    double v = a0 * yold[k];
    v        = fma(a1, ynew[k], v);
    if (deg == 2) v = fma(a2, fnew[k], v);
    else if (deg == 3)
    {
      v = fma(a2, fold[k], v);
      v = fma(a3, fnew[k], v);
    }
    out[k] = v;
  }
}

/* the value returned at tq: y_n itself, or the dense output on the last step [t - h, t]
 * (need_fnew, when given, makes f(t_n, y_n) current first); -22 when tq is behind the step */
typedef int (*dense_fnew_fn)(void* ctx, const double** fnew);
static int dense_out(orc_dense* d, long n, double t, double h, int deg, dense_fnew_fn need_fnew, void* ctx,
                     double tq, int interp, double* yout)
{
  if (!interp || tq == t)
  {
    memcpy(yout, d->ycur, n * sizeof(double));
    return 0;
  }
  const double tfuzz = 100.0 * DBL_EPSILON * (fabs(t) + fabs(h));
  if (tq < t - h - tfuzz) return -22;
  const double* fnew = NULL;
  if (deg >= 2 && need_fnew(ctx, &fnew)) return -8; /* RHS failure */
  orc_hermite(n, deg, (tq - t) / h, h, d->yold, d->ycur, d->fold, fnew, yout);
  return 0;
}

/* calls that return without stepping: 1 (with *ret) when this one does */
static int dense_entry(orc_dense* d, long n, double t, double h, int deg, dense_fnew_fn need_fnew, void* ctx,
                       int onestep, double tout, double* yout, int* ret)
{
  if (d->interp_ready && !onestep && t >= tout)
  {
    *ret        = dense_out(d, n, t, h, deg, need_fnew, ctx, tout, 1, yout);
    d->tretlast = tout;
    return 1;
  }
  if (d->interp_ready && onestep && t != d->tretlast)
  {
    *ret        = dense_out(d, n, t, h, deg, need_fnew, ctx, t, 0, yout);
    d->tretlast = t;
    return 1;
  }
  if (d->tstopset && t >= d->tstop)
  {
    d->tstopset = 0;
    dense_out(d, n, t, h, deg, need_fnew, ctx, t, 0, yout);
    d->tretlast = t;
    *ret        = 1; /* ARK_TSTOP_RETURN */
    return 1;
  }
  return 0;
}

/* after the step loop (return code ret): the stop time first, then NORMAL mode's tout */
static int dense_finish(orc_dense* d, long n, double t, double h, int deg, dense_fnew_fn need_fnew, void* ctx,
                        int onestep, double tout, double* yout, int ret)
{
  double tr  = t;
  int interp = 0;
  if (d->tstopset && t >= d->tstop)
  {
    d->tstopset = 0;
    if (ret == 0) ret = 1;
  }
  else if (ret == 0 && !onestep && t >= tout)
  {
    interp = 1;
    tr     = tout;
  }
  const int rc = dense_out(d, n, t, h, deg, need_fnew, ctx, tr, interp, yout);
  if (rc) return rc;
  d->tretlast = tr;
  return ret;
}

/* ---- stage arithmetic (mirrors the CUDA stage kernels) ---- */
typedef struct {
  double gc, gx, gy, gn, g0, gf, al, be, ga;
  /* mixed (difference) form: gsf = mu + nu - 1 + hm (cc + 2 cx + 2 cy), gmf = -nu */
  float gsf, gxf, gyf, gmf, gFf, alf, bef, gaf;
} stage_c;

static void stage_coeffs_j(const orc_prob* p, double t, double h, const double* mu, const double* nu,
                           const double* mus, const double* ajm1, const double* cjm1, int j,
                           stage_c* c)
{
  double hm = h * mus[j];
  double tj = t + h * cjm1[j];
  double tm = hm * p->cc;
  c->gc     = mu[j] + tm;
  c->gx     = hm * p->cx;
  c->gy     = hm * p->cy;
  c->gn     = nu[j];
  c->g0     = (1.0 - mu[j]) - nu[j];
  c->gf     = -(hm * ajm1[j]);
  forcing_scalars(p, hm, tj, &c->al, &c->be, &c->ga);
  /* mixed (increment) form */
  c->gsf    = (float)(((mu[j] + nu[j]) - 1.0) + hm * ((p->cc + 2.0 * p->cx) + 2.0 * p->cy));
  c->gxf    = (float)c->gx;
  c->gyf    = (float)c->gy;
  c->gmf    = (float)(-nu[j]);
  c->gFf    = (float)(hm * (1.0 - ajm1[j]));
  double dc  = orc_c(tj) - orc_c(t);
  double dcd = orc_cdot(tj) - orc_cdot(t);
  c->alf     = (float)(hm * dcd);
  c->bef     = (float)(-(hm * dc) * p->kx);
  c->gaf     = (float)(-(hm * dc) * p->ky);
}

static void stage64(const orc_prob* p, const stage_c* c, const double* ym1, const double* ym2,
                    const double* y0, const double* f0, double* yj)
{
  long nx = p->nx, ny = p->ny;
  int forced = (p->kind == ORC_MANUFACTURED);
#pragma omp parallel for schedule(static)
  for (long j = 0; j < ny; ++j)
    for (long i = 0; i < nx; ++i)
    {
      long k     = j * nx + i;
      double uw  = (i > 0) ? ym1[k - 1] : 0.0;
      double ue  = (i < nx - 1) ? ym1[k + 1] : 0.0;
      double us  = (j > 0) ? ym1[k - nx] : 0.0;
      double un  = (j < ny - 1) ? ym1[k + nx] : 0.0;
      double sx  = uw + ue, sy = us + un;
      double acc = c->gc * ym1[k];
      acc        = fma(c->gx, sx, acc);
      acc        = fma(c->gy, sy, acc);
      acc        = fma(c->gn, ym2[k], acc);
      acc        = fma(c->g0, y0[k], acc);
      acc        = fma(c->gf, f0[k], acc);
      if (forced)
      {
        double P = fma(c->al, p->Sx[i], c->be * p->Sxx[i]);
        double Q = c->ga * p->Sx[i];
        acc      = fma(p->Sy[j], P, acc);
        acc      = fma(p->Syy[j], Q, acc);
      }
      yj[k] = acc;
    }
}

/* Mixed stage in difference form: d_j = d_C + inc, where every FP32 operation of inc rounds a
 * quantity of the size of the stage-to-stage increment (neighbour differences, d_C - d_{j-2},
 * the F_0 and forcing terms) and d_C + inc is the only rounding at the scale of d. This is the
 * product's FP32 arithmetic operation for operation (mixed_point in the CUDA stage kernels). */
static void stage32(const orc_prob* p, const stage_c* c, const float* dm1, const float* dm2,
                    const float* f0f, const float* Sxf, const float* Sxxf, const float* Syf,
                    const float* Syyf, float* dj)
{
  long nx = p->nx, ny = p->ny;
  int forced = (p->kind == ORC_MANUFACTURED);
#pragma omp parallel for schedule(static)
  for (long j = 0; j < ny; ++j)
    for (long i = 0; i < nx; ++i)
    {
      long k    = j * nx + i;
      float dc  = dm1[k];
      float dw  = (i > 0) ? dm1[k - 1] : 0.0f;
      float de  = (i < nx - 1) ? dm1[k + 1] : 0.0f;
      float ds  = (j > 0) ? dm1[k - nx] : 0.0f;
      float dn  = (j < ny - 1) ? dm1[k + nx] : 0.0f;
      float m2  = dm2 ? dm2[k] : 0.0f;
      float lx  = (dw - dc) + (de - dc), ly = (ds - dc) + (dn - dc);
      float inc = c->gsf * dc;
      inc       = fmaf(c->gxf, lx, inc);
      inc       = fmaf(c->gyf, ly, inc);
      inc       = fmaf(c->gmf, dc - m2, inc);
      inc       = fmaf(c->gFf, f0f[k], inc);
      if (forced)
      {
        float P = fmaf(c->alf, Sxf[i], c->bef * Sxxf[i]);
        float Q = c->gaf * Sxf[i];
        inc     = fmaf(Syf[j], P, inc);
        inc     = fmaf(Syyf[j], Q, inc);
      }
      dj[k] = dc + inc;
    }
}

/* Error weight of the mixed step end: den = fma(rtol, |y|, atol); the correctly rounded FP32
 * reciprocal of (float)den, one Newton step in FP64; outside [2^-120, 2^120] the division. */
static double mixed_weight(double rtol, double atol, double y)
{
  double den = fma(rtol, fabs(y), atol);
  if (den >= 0x1p-120 && den <= 0x1p120)
  {
    float df  = (float)den;
    float rf  = 1.0f / df;
    double r0 = (double)rf;
    double e1 = fma(-den, r0, 1.0);
    return fma(r0, e1, r0);
  }
  return 1.0 / den;
}

/* Step end: Fnew = F(t+h, ynew), err = 0.8 (yn - ynew) + 0.4 h (Fn + Fnew),
 * dsm = ||err||_WRMS with ewt = 1/(rtol |yn| + atol). For the mixed form ynew = yn + ds,
 * yn - ynew is taken as -ds and ewt comes from mixed_weight. */
static double step_end(const orc_prob* p, const orc_opts* o, double t, double h, const double* yn,
                       const double* Fn, double* ynew, const float* ds, double* Fnew, float* Fnewf)
{
  long nx = p->nx, ny = p->ny, n = nx * ny;
  if (ds)
  {
#pragma omp parallel for schedule(static)
    for (long k = 0; k < n; ++k) ynew[k] = yn[k] + (double)ds[k];
  }
  orc_rhs(p, t + h, ynew, Fnew);
  if (Fnewf)
  {
#pragma omp parallel for schedule(static)
    for (long k = 0; k < n; ++k) Fnewf[k] = (float)Fnew[k];
  }
  double p4h = 0.4 * h;
  double s;
  if (ds)
  { /* mixed form: y_n - y_{n+1} as -d_s, the fast weight (mixed_weight in csrc/kernels.cuh) */
    XREDUCE(n, ({
              double d = -(double)ds[i];
              double e = 0.8 * d;
              e        = fma(p4h, Fn[i], e);
              e        = fma(p4h, Fnew[i], e);
              double w = mixed_weight(o->rtol, o->atol, yn[i]);
              double x = e * w;
              x * x;
            }));
    s = xacc_result(&tot);
  }
  else
  {
    XREDUCE(n, ({
              double d = yn[i] - ynew[i];
              double e = 0.8 * d;
              e        = fma(p4h, Fn[i], e);
              e        = fma(p4h, Fnew[i], e);
              double w = 1.0 / (o->rtol * fabs(yn[i]) + o->atol);
              double x = e * w;
              x * x;
            }));
    s = xacc_result(&tot);
  }
  return sqrt(s / (double)n);
}

/* WRMS of v with ewt(y) (used by the initial step estimate) */
static double wrms_ewt(const orc_opts* o, const double* v, const double* y, long n)
{
  XREDUCE(n, ({
            double w = 1.0 / (o->rtol * fabs(y[i]) + o->atol);
            double x = v[i] * w;
            x * x;
          }));
  return sqrt(xacc_result(&tot) / (double)n);
}

static double wrms_diff_ewt(const orc_opts* o, const double* a, const double* b, const double* y, long n)
{
  XREDUCE(n, ({
            double w = 1.0 / (o->rtol * fabs(y[i]) + o->atol);
            double x = (a[i] - b[i]) * w;
            x * x;
          }));
  return sqrt(xacc_result(&tot) / (double)n);
}

/* Initial step (Hairer, Norsett & Wanner, "Solving ODEs I", II.4), WRMS norms on ewt(y0),
 * order ORD; the explicit-Euler probe step is capped at 1/rho so that it stays stable, a
 * non-finite second-derivative estimate falls back to the probe step, and the result is
 * capped at tdist. */
static double initial_step_ord(const orc_prob* p, const orc_opts* o, double t0, const double* y0,
                               const double* F0, double tdist, double rho, long* nfe, double ordv);
static double initial_step(const orc_prob* p, const orc_opts* o, double t0, const double* y0,
                           const double* F0, double tdist, double rho, long* nfe)
{
  return initial_step_ord(p, o, t0, y0, F0, tdist, rho, nfe, ORD);
}

static double initial_step_ord(const orc_prob* p, const orc_opts* o, double t0, const double* y0,
                               const double* F0, double tdist, double rho, long* nfe, double ordv)
{
  long n = (long)p->nx * p->ny;
  double d0 = wrms_ewt(o, y0, y0, n);
  double d1 = wrms_ewt(o, F0, y0, n);
  double h0 = (d0 < 1.0e-5 || d1 < 1.0e-5) ? 1.0e-6 : 0.01 * (d0 / d1);
  if (rho > 0.0 && h0 * rho > 1.0) h0 = 1.0 / rho;
  if (h0 > tdist) h0 = tdist;
  double* y1 = (double*)malloc(n * sizeof(double));
  double* F1 = (double*)malloc(n * sizeof(double));
  for (long k = 0; k < n; ++k) y1[k] = fma(h0, F0[k], y0[k]);
  orc_rhs(p, t0 + h0, y1, F1);
  (*nfe)++;
  double d2  = wrms_diff_ewt(o, F1, F0, y0, n) / h0;
  double dm  = d1 > d2 ? d1 : d2;
  double h1  = (dm <= 1.0e-15) ? fmax(1.0e-6, h0 * 1.0e-3) : orc_pow(0.01 / dm, 1.0 / ordv);
  if (!(h1 > 0.0) || !(h1 < INFINITY)) h1 = h0;
  double h   = (100.0 * h0 < h1) ? 100.0 * h0 : h1;
  if (h > tdist) h = tdist;
  free(y1);
  free(F1);
  return h;
}

/* step loop: until t >= tout; steps clipped only at `clip` (the stop time or +inf) */
static int lsrk_steps(const orc_prob* p, const orc_opts* o, orc_state* st, double tout, double clip, double* y)
{
  long n    = (long)p->nx * p->ny;
  int smax  = o->smax > 1 ? o->smax : 200;
  long maxs = o->maxsteps > 0 ? o->maxsteps : 500;
  double* mu   = (double*)malloc((smax + 1) * sizeof(double));
  double* nu   = (double*)malloc((smax + 1) * sizeof(double));
  double* mus  = (double*)malloc((smax + 1) * sizeof(double));
  double* ajm1 = (double*)malloc((smax + 1) * sizeof(double));
  double* cjm1 = (double*)malloc((smax + 1) * sizeof(double));
  double *Ya = NULL, *Yb = NULL, *Yc = NULL, *ynew = NULL, *Fnew = NULL;
  float *da = NULL, *db = NULL, *dc = NULL, *Fnewf = NULL, *Sxf = NULL, *Sxxf = NULL, *Syf = NULL,
        *Syyf = NULL;
  int ret = 0;
  ynew = (double*)malloc(n * sizeof(double));
  Fnew = (double*)malloc(n * sizeof(double));
  if (o->mixed)
  {
    da    = (float*)malloc(n * sizeof(float));
    db    = (float*)malloc(n * sizeof(float));
    dc    = (float*)malloc(n * sizeof(float));
    Fnewf = (float*)malloc(n * sizeof(float));
    Sxf   = (float*)malloc(p->nx * sizeof(float));
    Sxxf  = (float*)malloc(p->nx * sizeof(float));
    Syf   = (float*)malloc(p->ny * sizeof(float));
    Syyf  = (float*)malloc(p->ny * sizeof(float));
    for (int i = 0; i < p->nx; ++i)
    {
      Sxf[i]  = (float)p->Sx[i];
      Sxxf[i] = (float)p->Sxx[i];
    }
    for (int j = 0; j < p->ny; ++j)
    {
      Syf[j]  = (float)p->Sy[j];
      Syyf[j] = (float)p->Syy[j];
    }
  }
  else
  {
    Ya = (double*)malloc(n * sizeof(double));
    Yb = (double*)malloc(n * sizeof(double));
    Yc = (double*)malloc(n * sizeof(double));
  }

  if (!st->initialized)
  {
    st->F  = (double*)malloc(n * sizeof(double));
    st->Ff = (float*)malloc(n * sizeof(float));
    orc_rhs(p, st->t, y, st->F);
    st->nfe++;
    for (long k = 0; k < n; ++k) st->Ff[k] = (float)st->F[k];
    st->hnext           = (o->hfixed > 0.0) ? o->hfixed : 0.0;
    st->initialized     = 1;
    st->steps_since_dee = -1;
  }

  long nsteps_call = 0;
  while (st->t < clip && st->t < tout)
  {
    if (nsteps_call >= maxs)
    {
      ret = -1; /* ARK_TOO_MUCH_WORK */
      break;
    }
    /* dominant eigenvalue: first step, then every dom_eig_freq accepted steps */
    /* dom_eig_freq <= 0: the eigenvalue is computed once (LSRKStepSetDomEigFrequency(0)) */
    int freq = o->dom_eig_freq;
    if (st->steps_since_dee < 0 || (freq > 0 && st->steps_since_dee >= freq))
    {
      double lam;
      if (o->internaleig)
      {
        if (!st->evec)
        {
          st->evec = (double*)malloc(n * sizeof(double));
          memcpy(st->evec, y, n * sizeof(double));
        }
        /* warm-up iterations (LSRKStepSetNumDomEigEst[Init]PreprocessIters): no convergence test */
        int warm = (st->ndee == 0) ? o->dee_init_warmups : o->dee_succ_warmups;
        if (warm > 0) st->nfe_dee += orc_power_iteration(p, st->evec, warm, 0.0, &lam);
        int it = orc_power_iteration(p, st->evec, o->dee_maxiters > 0 ? o->dee_maxiters : 100,
                                     o->dee_reltol > 0.0 ? o->dee_reltol : 0.01, &lam);
        st->nfe_dee += it;
      }
      else lam = orc_dom_eig(p);
      double saf          = o->eig_safety > 0.0 ? o->eig_safety : 1.01;
      st->spectral_radius = saf * fabs(lam);
      st->ndee++;
      st->steps_since_dee = 0;
    }
    if (!(st->hnext > 0.0))
    {
      st->hnext = initial_step(p, o, st->t, y, st->F, (tout < clip ? tout : clip) - st->t, st->spectral_radius,
                               &st->nfe);
      if (!(st->hnext > 0.0))
      {
        /* a non-finite state (NaN / Inf) gives no usable step: the call fails before any
         * attempt, as an unrecoverable failure */
        ret = -3;
        goto done;
      }
    }

    int nef = 0;
    for (;;)
    {
      double h = st->hnext, hmax;
      int clipped = 0;
      int s       = orc_stages_needed(o->method, h, st->spectral_radius, smax, &hmax);
      if (s > smax)
      {
        if (o->hfixed > 0.0)
        {
          ret = -2;
          goto done;
        }
        h = hmax;
        st->nst_exp++;
      }
      if (st->t + h >= clip)
      {
        h       = clip - st->t;
        clipped = 1;
      }
      s = orc_stages_needed(o->method, h, st->spectral_radius, smax, &hmax);
      orc_stage_coeffs(o->method, s, mu, nu, mus, ajm1, cjm1);
      st->nst_attempts++;
      st->d.interp_ready = 0;
      double dsm;
      if (p->kind == ORC_PERIODIC)
      {
        /* reference mode (periodic wrap, per-face coefficients): the product's generic
         * N_Vector path, stage by stage F_j = f(t + c_{j-1} h, Y_{j-1}) and
         * Y_j = mu Y_{j-1} + nu Y_{j-2} + (1 - mu - nu) Y_0 + h mus F_j - h mus a_{j-1} F_0
         * (N_VLinearCombination order); error 0.8 Y_0 - 0.8 Y_s + 0.4 h F_0 + 0.4 h F_s and
         * ewt = 1 / (rtol |y| + atol) as N_VScale, N_VAddConst, N_VInv */
        if (o->mixed)
        { /* mixed reference mode (the product's periodic_stage32_kernel): FP32 increments in the
           * difference form with FP32 face tables, y_{n+1} = y_n + d_s in FP64 */
          long nx = p->nx, ny = p->ny;
          float* fc = (float*)malloc((2 * nx + 2 * ny) * sizeof(float));
          for (long i = 0; i < nx; ++i)
          {
            fc[i]      = (float)p->Dxw[i];
            fc[nx + i] = (float)p->Dxe[i];
          }
          for (long j = 0; j < ny; ++j)
          {
            fc[2 * nx + j]      = (float)p->Dys[j];
            fc[2 * nx + ny + j] = (float)p->Dyn[j];
          }
          float* Ff32 = (float*)malloc(n * sizeof(float));
          for (long k = 0; k < n; ++k) Ff32[k] = (float)st->F[k];
          float hm1f = (float)(h * mus[1]);
          for (long k = 0; k < n; ++k) da[k] = hm1f * Ff32[k];
          float* dbufs[3] = {da, db, dc};
          int im1 = 0, im2 = -1;
          for (int j = 2; j <= s; ++j)
          {
            int io    = (im1 + 1) % 3;
            double hm = h * mus[j];
            float gs = (float)((mu[j] + nu[j]) - 1.0), hmf = (float)hm, gm = (float)(-nu[j]);
            float gF = (float)(hm * (1.0 - ajm1[j]));
            const float* dm1 = dbufs[im1];
            const float* dm2 = im2 >= 0 ? dbufs[im2] : NULL;
            float* out       = dbufs[io];
#pragma omp parallel for schedule(static)
            for (long jj = 0; jj < ny; ++jj)
              for (long ii = 0; ii < nx; ++ii)
              {
                long iw = (ii == 0) ? nx - 1 : ii - 1, ie = (ii == nx - 1) ? 0 : ii + 1;
                long js = (jj == 0) ? ny - 1 : jj - 1, jn = (jj == ny - 1) ? 0 : jj + 1;
                long k  = jj * nx + ii;
                float dC = dm1[k], dW = dm1[jj * nx + iw], dE = dm1[jj * nx + ie], dS = dm1[js * nx + ii],
                      dN = dm1[jn * nx + ii];
                float m2  = dm2 ? dm2[k] : 0.0f;
                float a   = fc[ii] * (dW - dC);
                a         = fmaf(fc[nx + ii], dE - dC, a);
                a         = fmaf(fc[2 * nx + jj], dS - dC, a);
                a         = fmaf(fc[2 * nx + ny + jj], dN - dC, a);
                float inc = gs * dC;
                inc       = fmaf(hmf, a, inc);
                inc       = fmaf(gm, dC - m2, inc);
                inc       = fmaf(gF, Ff32[k], inc);
                out[k]    = dC + inc;
              }
            im2 = im1;
            im1 = io;
          }
          for (long k = 0; k < n; ++k) ynew[k] = y[k] + (double)dbufs[im1][k];
          free(fc);
          free(Ff32);
          st->nfe += s;
        }
        else
        {
        double hm1 = h * mus[1];
        for (long k = 0; k < n; ++k) Ya[k] = fma(hm1, st->F[k], y[k]);
        const double *ym2 = y, *ym1 = Ya;
        double* bufs[3] = {Yb, Yc, Ya};
        int bi          = 0;
        double* yj      = Ya;
        for (int j = 2; j <= s; ++j)
        {
          orc_rhs(p, st->t + h * cjm1[j], ym1, Fnew);
          yj = bufs[bi];
          bi = (bi + 1) % 3;
          const double hm = h * mus[j];
          const double c0 = mu[j], c1 = nu[j], c2 = (1.0 - mu[j]) - nu[j], c3 = hm, c4 = -(hm * ajm1[j]);
          for (long k = 0; k < n; ++k)
          {
            double acc = c0 * ym1[k];
            acc        = fma(c1, ym2[k], acc);
            acc        = fma(c2, y[k], acc);
            acc        = fma(c3, Fnew[k], acc);
            acc        = fma(c4, st->F[k], acc);
            yj[k]      = acc;
          }
          ym2 = ym1;
          ym1 = yj;
        }
        st->nfe += s;
        memcpy(ynew, yj, n * sizeof(double));
        }
        orc_rhs(p, st->t + h, ynew, Fnew);
        if (o->mixed)
          for (long k = 0; k < n; ++k) Fnewf[k] = (float)Fnew[k];
        const double p4h = 0.4 * h;
        XREDUCE(n, ({
                  double e = 0.8 * y[i];
                  e        = fma(-0.8, ynew[i], e);
                  e        = fma(p4h, st->F[i], e);
                  e        = fma(p4h, Fnew[i], e);
                  double w = 1.0 / (o->rtol * fabs(y[i]) + o->atol);
                  double x = e * w;
                  x * x;
                }));
        dsm = sqrt(xacc_result(&tot) / (double)n);
      }
      else if (!o->mixed)
      {
        /* Y_1 = Y_0 + h mus_1 F_0 ; Y_j from Y_{j-1}, Y_{j-2} (Y_{-1} := Y_0) */
        double hm1 = h * mus[1];
        for (long k = 0; k < n; ++k) Ya[k] = fma(hm1, st->F[k], y[k]);
        const double *ym2 = y, *ym1 = Ya;
        double* bufs[3] = {Yb, Yc, Ya};
        int bi          = 0;
        double* yj      = Ya;
        for (int j = 2; j <= s; ++j)
        {
          stage_c c;
          stage_coeffs_j(p, st->t, h, mu, nu, mus, ajm1, cjm1, j, &c);
          yj = bufs[bi];
          bi = (bi + 1) % 3;
          stage64(p, &c, ym1, ym2, y, st->F, yj);
          ym2 = ym1;
          ym1 = yj;
        }
        st->nfe += s; /* F_0 reused (FSAL); s - 1 stage RHS + 1 step-end RHS */
        memcpy(ynew, yj, n * sizeof(double));
        dsm = step_end(p, o, st->t, h, y, st->F, ynew, NULL, Fnew, NULL);
      }
      else
      {
        float hm1 = (float)(h * mus[1]);
        for (long k = 0; k < n; ++k) da[k] = hm1 * st->Ff[k];
        const float *dm2 = NULL, *dm1 = da;
        float* bufs[3] = {db, dc, da};
        int bi         = 0;
        float* dj      = da;
        for (int j = 2; j <= s; ++j)
        {
          stage_c c;
          stage_coeffs_j(p, st->t, h, mu, nu, mus, ajm1, cjm1, j, &c);
          dj = bufs[bi];
          bi = (bi + 1) % 3;
          stage32(p, &c, dm1, dm2, st->Ff, Sxf, Sxxf, Syf, Syyf, dj);
          dm2 = dm1;
          dm1 = dj;
        }
        st->nfe += s;
        dsm = step_end(p, o, st->t, h, y, st->F, ynew, dj, Fnew, Fnewf);
      }
      st->stages_total += s;
      if (s > st->stage_max) st->stage_max = s;

      if (o->hfixed > 0.0 || dsm <= 1.0)
      {
        /* accept */
        st->t = clipped ? clip : st->t + h;
        memcpy(st->d.yold, y, n * sizeof(double));
        memcpy(y, ynew, n * sizeof(double));
        st->d.interp_ready = 1;
        memcpy(st->F, Fnew, n * sizeof(double));
        if (o->mixed) memcpy(st->Ff, Fnewf, n * sizeof(float));
        else
          for (long k = 0; k < n; ++k) st->Ff[k] = (float)Fnew[k];
        const double hprev = st->hlast;
        st->hlast          = h;
        if (o->hfixed > 0.0) st->hnext = o->hfixed;
        else
        {
          double hn  = orc_controller(o->controller, h, dsm, st->ep1, st->ep2, hprev, st->nhist);
          double eta = SAFETY * hn / h;
          double emx = (st->nst == 0) ? ETAMX1 : (st->after_fail ? 1.0 : GROWTH);
          if (eta > emx) eta = emx;
          if (eta >= LBOUND && eta <= UBOUND) eta = 1.0;
          st->hnext = h * eta;
          st->ep2   = st->ep1;
          st->ep1   = dsm;
          st->nhist++;
        }
        st->after_fail = 0;
        st->nst++;
        st->steps_since_dee++;
        nsteps_call++;
        break;
      }
      /* reject */
      st->netf++;
      nef++;
      if (!(dsm == dsm) || nef > 20)
      {
        ret = -3; /* ARK_ERR_FAILURE */
        goto done;
      }
      double hn  = orc_controller(o->controller, h, dsm, st->ep1, st->ep2, st->hlast, st->nhist);
      double eta = SAFETY * hn / h;
      if (eta > 1.0) eta = 1.0;
      if (nef >= SMALL_NEF && eta > ETAMXF) eta = ETAMXF;
      if (eta < ETAMIN) eta = ETAMIN;
      st->hnext      = h * eta;
      st->after_fail = 1;
    }
  }
done:
  free(mu);
  free(nu);
  free(mus);
  free(ajm1);
  free(cjm1);
  free(Ya);
  free(Yb);
  free(Yc);
  free(ynew);
  free(Fnew);
  free(da);
  free(db);
  free(dc);
  free(Fnewf);
  free(Sxf);
  free(Sxxf);
  free(Syf);
  free(Syyf);
  return ret;
}

static void dense_alloc(orc_dense* d, long n, int with_fold, const double* y0)
{
  if (d->ycur) return;
  d->ycur = (double*)malloc(n * sizeof(double));
  d->yold = (double*)malloc(n * sizeof(double));
  d->fold = with_fold ? (double*)malloc(n * sizeof(double)) : NULL;
  memcpy(d->ycur, y0, n * sizeof(double));
}

int orc_lsrk_evolve(const orc_prob* p, const orc_opts* o, orc_state* st, double tout, double* y)
{
  long n = (long)p->nx * p->ny;
  int ret;
  dense_alloc(&st->d, n, 0, y);
  if (dense_entry(&st->d, n, st->t, st->hlast, 1, NULL, NULL, 0, tout, y, &ret)) return ret;
  ret = lsrk_steps(p, o, st, tout, st->d.tstopset ? st->d.tstop : INFINITY, st->d.ycur);
  return dense_finish(&st->d, n, st->t, st->hlast, 1, NULL, NULL, 0, tout, y, ret);
}

/* ------------------------------------------------------------------------------------
 * Implicit comparator: (I - gamma A) x = b by preconditioned CG with the Jacobi
 * preconditioner of preconditioner_jacobi.cpp:21-40 (D = 1/(1 - gamma diag),
 * diag = -((Dxw+Dxe)+(Dys+Dyn)) = cc) and PSolve z = D r (preconditioner_jacobi.cpp:58).
 * x starts at zero; stop when ||r||_2 <= tol ||b||_2. Arithmetic mirrors the fused CUDA
 * kernels: K1 forms p = beta p + D r, q = M p, p.q; K2 updates x, r and r.r, r.(D r).
 * ----------------------------------------------------------------------------------*/
/* q = (I - gamma A) v with the coefficients folded: c0 v_C + c1 (v_W + v_E) + c2 (v_S + v_N),
 * c0 = 1 - gamma cc, c1 = -gamma cx, c2 = -gamma cy (the fused kernels pcg_q / fcg_q) */
static void apply_M_folded(const orc_prob* p, double gamma, const double* v, double* w)
{
  long nx = p->nx, ny = p->ny;
  const double c0 = 1.0 - gamma * p->cc, c1 = -gamma * p->cx, c2 = -gamma * p->cy;
#pragma omp parallel for schedule(static)
  for (long j = 0; j < ny; ++j)
    for (long i = 0; i < nx; ++i)
    {
      long k   = j * nx + i;
      double w_ = (i > 0) ? v[k - 1] : 0.0, e = (i < nx - 1) ? v[k + 1] : 0.0;
      double s_ = (j > 0) ? v[k - nx] : 0.0, nn = (j < ny - 1) ? v[k + nx] : 0.0;
      double sx = w_ + e, sy = s_ + nn;
      w[k]      = fma(c1, sx, fma(c2, sy, c0 * v[k]));
    }
}

/* The fused Jacobi-PCG (csrc/pcg.cu): SUNLinSol_PCG with the constant Jacobi scaling D of
 * preconditioner_jacobi.cpp:9-61 for constant coefficients, so r.z = D (r.r) (one exact sum
 * per iteration, rounded once, times D) */
int orc_pcg(const orc_prob* p, double gamma, int jacobi, const double* b, double* x,
            double tol, int maxit, double* relres)
{
  long n    = (long)p->nx * p->ny;
  double D  = jacobi ? 1.0 / (1.0 - gamma * p->cc) : 1.0;
  double* r  = (double*)malloc(n * sizeof(double));
  double* pv = (double*)calloc(n, sizeof(double));
  double* q  = (double*)malloc(n * sizeof(double));
  for (long k = 0; k < n; ++k)
  {
    x[k] = 0.0;
    r[k] = b[k];
  }
  const double bb = orc_xdot(b, b, n);
  double bnorm    = sqrt(bb);
  if (!(bnorm > 0.0))
  {
    *relres = 0.0;
    free(r);
    free(pv);
    free(q);
    return 0;
  }
  double rz = D * bb;
  double beta = 0.0, rr = 0.0;
  int it;
  for (it = 1; it <= maxit; ++it)
  {
    for (long k = 0; k < n; ++k) pv[k] = fma(beta, pv[k], D * r[k]);
    apply_M_folded(p, gamma, pv, q);
    double pq    = orc_xdot(pv, q, n);
    double alpha = rz / pq;
    for (long k = 0; k < n; ++k)
    {
      x[k] = fma(alpha, pv[k], x[k]);
      r[k] = fma(-alpha, q[k], r[k]);
    }
    {
      XREDUCE(n, r[i] * r[i]);
      rr = xacc_result(&tot);
    }
    const double rzn = D * rr;
    if (sqrt(rr) <= tol * bnorm) break;
    beta = rzn / rz;
    rz   = rzn;
  }
  if (it > maxit) it = maxit;
  *relres = sqrt(rr) / bnorm;
  free(r);
  free(pv);
  free(q);
  return it;
}

/* Fixed-step SDIRK2 (Alexander; gamma = 1 - 1/sqrt(2), stiffly accurate) with each stage's
 * linear Newton correction solved by Jacobi-PCG (ARKStep DIRK + SUNLinSol_PCG,
 * main.cpp:199-231,242,302-329; the RHS is linear so one Newton iteration is exact). */
int orc_sdirk2(const orc_prob* p, double t0, double h, int nsteps, double tol, int maxit,
               double* y, long* total_iters)
{
  long n     = (long)p->nx * p->ny;
  double g   = 1.0 - sqrt(0.5);
  double* f  = (double*)malloc(n * sizeof(double));
  double* f1 = (double*)malloc(n * sizeof(double));
  double* rhs = (double*)malloc(n * sizeof(double));
  double* d   = (double*)malloc(n * sizeof(double));
  double* Y1  = (double*)malloc(n * sizeof(double));
  double relres;
  long iters = 0;
  double t   = t0;
  for (int s = 0; s < nsteps; ++s)
  {
    double hg = h * g;
    /* stage 1: (I - hg A) d1 = hg f(t + g h, y_n), Y1 = y_n + d1 */
    orc_rhs(p, t + g * h, y, f);
    for (long k = 0; k < n; ++k) rhs[k] = hg * f[k];
    iters += orc_pcg(p, hg, 1, rhs, d, tol, maxit, &relres);
    for (long k = 0; k < n; ++k) Y1[k] = y[k] + d[k];
    orc_rhs(p, t + g * h, Y1, f1);
    /* stage 2: (I - hg A) d2 = h(1-g) F1 + hg f(t+h, y_n), y_{n+1} = y_n + d2 */
    orc_rhs(p, t + h, y, f);
    double h1g = h * (1.0 - g);
    for (long k = 0; k < n; ++k) rhs[k] = fma(h1g, f1[k], hg * f[k]);
    iters += orc_pcg(p, hg, 1, rhs, d, tol, maxit, &relres);
    for (long k = 0; k < n; ++k) y[k] = y[k] + d[k];
    t = t0 + (s + 1) * h;
  }
  *total_iters = iters;
  free(f);
  free(f1);
  free(rhs);
  free(d);
  free(Y1);
  return 0;
}

static void v_linsum(long n, double a, const double* x, double b, const double* y, double* z)
{
  for (long k = 0; k < n; ++k) z[k] = fma(a, x[k], b * y[k]);
}
static void v_scale(long n, double c, const double* x, double* z)
{
  for (long k = 0; k < n; ++k) z[k] = c * x[k];
}
static void v_lincomb(long n, int nv, const double* cf, const double** X, double* z)
{
  for (long k = 0; k < n; ++k)
  {
    double acc = cf[0] * X[0][k];
    for (int v = 1; v < nv; ++v) acc = fma(cf[v], X[v][k], acc);
    z[k] = acc;
  }
}

/* ------------------------------------------------------------------------------------
 * Generic Krylov solvers of the SUNLinSol_PCG / SUNLinSol_SPGMR interface
 * (diffusion_2D/main.cpp:209-218) on (I - gamma A) x = b with the Jacobi preconditioner,
 * restated in the exact operation sequence of the product's callback path: ATimes
 * z = fma(1, v, (-gamma) (A v)) (N_VLinearSum after J*v), PSolve z = D r, LinearSum
 * z = fma(a, x, b y), Scale z = c x, LinearCombination acc = c0 x0 then fma(c_k, x_k, acc),
 * exact dot products; small dense algebra in plain double arithmetic. Dirichlet kinds only.
 * ----------------------------------------------------------------------------------*/
typedef struct orc_pfmg orc_pfmg;
static void pfmg_apply(orc_pfmg* mg, const double* r, double* z);

typedef struct {
  const orc_prob* p;
  double gamma, D;
  int jacobi;     /* 1: Jacobi PSolve, 2: the PFMG V-cycle below */
  double* tmp;
  orc_pfmg* mg;
} gen_op;

/* calls of the callbacks (the ARKStep restatement reports them as Jac-times evals / Prec solves) */
static long g_gen_atimes_calls = 0, g_gen_psolve_calls = 0;

static void gen_atimes(const gen_op* o, const double* v, double* z)
{
  long n = (long)o->p->nx * o->p->ny;
  g_gen_atimes_calls++;
  orc_apply_A(o->p, v, o->tmp);
  v_linsum(n, 1.0, v, -o->gamma, o->tmp, z);
}

/* z = P^-1 r (Jacobi) or z = r when unpreconditioned (PCG copies with LinearSum(1, r, 0, r)) */
static void gen_psolve(const gen_op* o, const double* r, double* z, int copy_form)
{
  long n = (long)o->p->nx * o->p->ny;
  if (o->jacobi) g_gen_psolve_calls++;
  if (o->jacobi == 2) pfmg_apply(o->mg, r, z);
  else if (o->jacobi && o->p->kind == ORC_PERIODIC)
  { /* per-point diagonal of the periodic operator: -((Dxw + Dxe) + (Dys + Dyn)) */
    const orc_prob* p = o->p;
    for (long j = 0; j < p->ny; ++j)
      for (long i = 0; i < p->nx; ++i)
      {
        double diag      = -((p->Dxw[i] + p->Dxe[i]) + (p->Dys[j] + p->Dyn[j]));
        double D         = 1.0 / (1.0 - o->gamma * diag);
        z[j * p->nx + i] = D * r[j * p->nx + i];
      }
  }
  else if (o->jacobi)
    for (long k = 0; k < n; ++k) z[k] = o->D * r[k];
  else if (copy_form) v_linsum(n, 1.0, r, 0.0, r, z);
  else memcpy(z, r, n * sizeof(double));
}

/* SUNLinSol_PCG through callbacks, x0 = 0, stop when ||r|| <= tol ||b|| (0 / 1 = converged /
 * not within maxl iterations) */
/* SUNLinSol_PCG over the operator / preconditioner of `o` (the product's pcg_solve) */
static int gen_pcg(gen_op* o, const double* b, double* x, double tol, int maxl, int* iters, double* relres)
{
  long n     = (long)o->p->nx * o->p->ny;
  double* r  = (double*)malloc(n * sizeof(double));
  double* z  = (double*)malloc(n * sizeof(double));
  double* pv = (double*)malloc(n * sizeof(double));
  double* Ap = (double*)malloc(n * sizeof(double));
  int ret = 1;
  *iters  = 0;
  *relres = 0.0;
  for (long k = 0; k < n; ++k) x[k] = 0.0;
  v_linsum(n, 1.0, b, 0.0, b, r);
  double bnorm = sqrt(orc_xdot(b, b, n));
  if (!(bnorm > 0.0))
  {
    ret = 0;
    goto out;
  }
  gen_psolve(o, r, z, 1);
  double rz = orc_xdot(r, z, n);
  v_linsum(n, 1.0, z, 0.0, z, pv);
  for (int it = 1; it <= maxl; ++it)
  {
    gen_atimes(o, pv, Ap);
    double pq    = orc_xdot(pv, Ap, n);
    double alpha = rz / pq;
    v_linsum(n, alpha, pv, 1.0, x, x);
    v_linsum(n, -alpha, Ap, 1.0, r, r);
    double rr = orc_xdot(r, r, n);
    *iters    = it;
    *relres   = sqrt(rr) / bnorm;
    if (sqrt(rr) <= tol * bnorm)
    {
      ret = 0;
      goto out;
    }
    gen_psolve(o, r, z, 1);
    double rzn  = orc_xdot(r, z, n);
    double beta = rzn / rz;
    rz          = rzn;
    v_linsum(n, 1.0, z, beta, pv, pv);
  }
out:
  free(r);
  free(z);
  free(pv);
  free(Ap);
  return ret;
}

int orc_pcg_generic(const orc_prob* p, double gamma, int jacobi, const double* b, double* x, double tol,
                    int maxl, int* iters, double* relres)
{
  long n   = (long)p->nx * p->ny;
  gen_op o = {p, gamma, 1.0 / (1.0 - gamma * p->cc), jacobi, (double*)malloc(n * sizeof(double)), NULL};
  int ret  = gen_pcg(&o, b, x, tol, maxl, iters, relres);
  free(o.tmp);
  return ret;
}

static void orc_givens(double a, double b, double* c, double* s)
{
  if (b == 0.0)
  {
    *c = 1.0;
    *s = 0.0;
  }
  else if (fabs(b) > fabs(a))
  {
    double t = a / b;
    *s       = 1.0 / sqrt(1.0 + t * t);
    *c       = *s * t;
  }
  else
  {
    double t = b / a;
    *c       = 1.0 / sqrt(1.0 + t * t);
    *s       = *c * t;
  }
}

/* SUNLinSol_SPGMR: restarted GMRES(maxl) with right preconditioning (Saad & Schultz 1986),
 * x0 = 0, Arnoldi by modified Gram-Schmidt (gstype 1) or classical Gram-Schmidt with one
 * re-orthogonalisation pass (gstype 2), Givens rotations; stop when the residual estimate
 * |g_{j+1}| <= tol ||b||; restart from the true residual. Returns 0 / 1 as orc_pcg_generic. */
static int spgmr_op(gen_op* op, const double* b, double* x, double tol, int maxl, int max_restarts, int gstype,
                    int flexible, int* iters, double* relres)
{
  gen_op o         = *op;
  const int jacobi = o.jacobi;
  long n           = (long)o.p->nx * o.p->ny;
  int m            = maxl;
  double** V = (double**)malloc((m + 1) * sizeof(double*));
  for (int k = 0; k <= m; ++k) V[k] = (double*)malloc(n * sizeof(double));
  /* flexible GMRES keeps the preconditioned basis Z (Saad 1993) */
  const int flex = flexible && jacobi;
  double** Z     = (double**)malloc((m > 0 ? m : 1) * sizeof(double*));
  for (int k = 0; k < m; ++k) Z[k] = flex ? (double*)malloc(n * sizeof(double)) : NULL;
  double* r  = (double*)malloc(n * sizeof(double));
  double* z  = (double*)malloc(n * sizeof(double));
  double* u  = (double*)malloc(n * sizeof(double));
  double* H  = (double*)calloc((size_t)(m + 1) * m, sizeof(double));
  double* cs = (double*)malloc(m * sizeof(double));
  double* sn = (double*)malloc(m * sizeof(double));
  double* g  = (double*)malloc((m + 1) * sizeof(double));
  double* y  = (double*)malloc(m * sizeof(double));
  double* h1 = (double*)malloc((m + 1) * sizeof(double));
  double* h2 = (double*)malloc((m + 1) * sizeof(double));
  double* cf = (double*)malloc((m + 2) * sizeof(double));
  const double** X = (const double**)malloc((m + 2) * sizeof(double*));
#define HH(i, j) H[(size_t)(i) * m + (j)]
  int ret = 1;
  *iters  = 0;
  *relres = 0.0;
  for (long k = 0; k < n; ++k) x[k] = 0.0;
  v_linsum(n, 1.0, b, 0.0, b, r);
  double bnorm = sqrt(orc_xdot(b, b, n));
  if (!(bnorm > 0.0))
  {
    ret = 0;
    goto out;
  }
  double beta = bnorm;
  for (int cycle = 0; cycle <= max_restarts; ++cycle)
  {
    v_scale(n, 1.0 / beta, r, V[0]);
    for (int k = 0; k <= m; ++k) g[k] = 0.0;
    g[0]          = beta;
    int kc        = 0;
    int converged = 0;
    for (int j = 0; j < m; ++j)
    {
      double* w = V[j + 1];
      if (jacobi)
      {
        double* zj = flex ? Z[j] : z;
        gen_psolve(&o, V[j], zj, 0);
        gen_atimes(&o, zj, w);
      }
      else gen_atimes(&o, V[j], w);
      if (gstype == 1)
        for (int i = 0; i <= j; ++i)
        {
          HH(i, j) = orc_xdot(w, V[i], n);
          v_linsum(n, -HH(i, j), V[i], 1.0, w, w);
        }
      else
      {
        for (int pass = 0; pass < 2; ++pass)
        {
          double* hp = pass ? h2 : h1;
          for (int i = 0; i <= j; ++i) hp[i] = orc_xdot(w, V[i], n);
          cf[0] = 1.0;
          X[0]  = w;
          for (int i = 0; i <= j; ++i)
          {
            cf[i + 1] = -hp[i];
            X[i + 1]  = V[i];
          }
          v_lincomb(n, j + 2, cf, X, w);
        }
        for (int i = 0; i <= j; ++i) HH(i, j) = h1[i] + h2[i];
      }
      double hn    = sqrt(orc_xdot(w, w, n));
      HH(j + 1, j) = hn;
      for (int i = 0; i < j; ++i)
      {
        double a = HH(i, j), bb = HH(i + 1, j);
        HH(i, j)     = cs[i] * a + sn[i] * bb;
        HH(i + 1, j) = cs[i] * bb - sn[i] * a;
      }
      orc_givens(HH(j, j), HH(j + 1, j), &cs[j], &sn[j]);
      HH(j, j)     = cs[j] * HH(j, j) + sn[j] * HH(j + 1, j);
      HH(j + 1, j) = 0.0;
      g[j + 1]     = -sn[j] * g[j];
      g[j]         = cs[j] * g[j];
      kc           = j + 1;
      (*iters)++;
      *relres = fabs(g[j + 1]) / bnorm;
      if (hn > 0.0) v_scale(n, 1.0 / hn, w, w);
      if (fabs(g[j + 1]) <= tol * bnorm || !(hn > 0.0))
      {
        converged = fabs(g[j + 1]) <= tol * bnorm;
        break;
      }
    }
    for (int i = kc - 1; i >= 0; --i)
    {
      double sacc = g[i];
      for (int q = i + 1; q < kc; ++q) sacc = sacc - HH(i, q) * y[q];
      y[i] = sacc / HH(i, i);
    }
    if (flex)
    {
      for (int i = 0; i < kc; ++i) X[i] = Z[i];
      v_lincomb(n, kc, y, X, u);
      v_linsum(n, 1.0, x, 1.0, u, x);
    }
    else
    {
      for (int i = 0; i < kc; ++i) X[i] = V[i];
      v_lincomb(n, kc, y, X, u);
      if (jacobi)
      {
        gen_psolve(&o, u, z, 0);
        v_linsum(n, 1.0, x, 1.0, z, x);
      }
      else v_linsum(n, 1.0, x, 1.0, u, x);
    }
    if (converged)
    {
      ret = 0;
      goto out;
    }
    if (cycle == max_restarts) break;
    gen_atimes(&o, x, u);
    v_linsum(n, 1.0, b, -1.0, u, r);
    beta    = sqrt(orc_xdot(r, r, n));
    *relres = beta / bnorm;
    if (beta <= tol * bnorm)
    {
      ret = 0;
      goto out;
    }
  }
#undef HH
out:
  for (int k = 0; k <= m; ++k) free(V[k]);
  free(V);
  for (int k = 0; k < m; ++k) free(Z[k]);
  free(Z);
  free(r);
  free(z);
  free(u);
  free(H);
  free(cs);
  free(sn);
  free(g);
  free(y);
  free(h1);
  free(h2);
  free(cf);
  free(X);
  return ret;
}

static int spgmr_impl(const orc_prob* p, double gamma, int jacobi, const double* b, double* x, double tol, int maxl,
                      int max_restarts, int gstype, int flexible, int* iters, double* relres)
{
  long n   = (long)p->nx * p->ny;
  gen_op o = {p, gamma, 1.0 / (1.0 - gamma * p->cc), jacobi, (double*)malloc(n * sizeof(double)), NULL};
  int ret  = spgmr_op(&o, b, x, tol, maxl, max_restarts, gstype, flexible, iters, relres);
  free(o.tmp);
  return ret;
}

int orc_spgmr(const orc_prob* p, double gamma, int jacobi, const double* b, double* x, double tol, int maxl,
              int max_restarts, int gstype, int* iters, double* relres)
{
  return spgmr_impl(p, gamma, jacobi, b, x, tol, maxl, max_restarts, gstype, 0, iters, relres);
}

/* SUNLinSol_SPFGMR restated: the preconditioned vectors z_j = P^-1 v_j are kept and the cycle
 * ends with x += Z y; without a preconditioner it is GMRES itself. */
int orc_spfgmr(const orc_prob* p, double gamma, int jacobi, const double* b, double* x, double tol, int maxl,
               int max_restarts, int gstype, int* iters, double* relres)
{
  return spgmr_impl(p, gamma, jacobi, b, x, tol, maxl, max_restarts, gstype, 1, iters, relres);
}

/* ------------------------------------------------------------------------------------
 * Structured multigrid V-cycle in the role of hypre PFMG (diffusion_2D/preconditioner_hypre.cpp
 * :13-180): semicoarsening in the direction of the larger coupling (coarse point I = fine
 * 2I + 1, coupling / 4), non-Galerkin coarse operators d = 1 + 2 (a_x + a_y), linear
 * interpolation, full-weighting restriction, weighted Jacobi (omega 0.8), symmetric or
 * nonsymmetric red/black Gauss-Seidel relaxation, 8 sweeps on the coarsest level (at most 2 x 2);
 * on the periodic problem per-face couplings (coarse faces: two fine faces in series, 0.5 a1 a2 /
 * (a1 + a2)), wrapped neighbours and sweeps from one buffer into the other; the product's
 * operation order (csrc/pfmg.cu).
 * ----------------------------------------------------------------------------------*/
typedef struct {
  long nx, ny;
  double ax, ay, d, dinv, wd;
  int dir;
  double *f, *u, *t;
  double *axf, *ayf; /* periodic: coupling of each x / y face (i + 1/2, wrapping) */
} pfmg_level;

struct orc_pfmg {
  int relax, nrelax, nl, periodic;
  pfmg_level L[64];
};

/* ---- periodic levels (csrc/pfmg.cu per_* kernels): M u = d u - (w uW + e uE + s uS + n uN) */
static long pwrap(long i, long n) { return i < 0 ? i + n : (i >= n ? i - n : i); }

typedef struct {
  double w, e, s, n, d, uW, uE, uS, uN;
} per_pt;

static per_pt per_point(const double* u, const pfmg_level* l, long i, long j)
{
  per_pt q;
  long iw = pwrap(i - 1, l->nx), ie = pwrap(i + 1, l->nx), js = pwrap(j - 1, l->ny), jn = pwrap(j + 1, l->ny);
  q.w  = l->axf[iw];
  q.e  = l->axf[i];
  q.s  = l->ayf[js];
  q.n  = l->ayf[j];
  q.d  = 1.0 + ((q.w + q.e) + (q.s + q.n));
  q.uW = u[j * l->nx + iw];
  q.uE = u[j * l->nx + ie];
  q.uS = u[js * l->nx + i];
  q.uN = u[jn * l->nx + i];
  return q;
}

static double per_m(const per_pt* q, double uc)
{
  double m = q->d * uc;
  m        = fma(-q->w, q->uW, m);
  m        = fma(-q->e, q->uE, m);
  m        = fma(-q->s, q->uS, m);
  m        = fma(-q->n, q->uN, m);
  return m;
}

static double series_coupling(double a1, double a2)
{
  double s = a1 + a2;
  if (!(s > 0.0)) return 0.0;
  double t = a1 * a2;
  return 0.5 * (t / s);
}

static void per_smooth(orc_pfmg* mg, pfmg_level* l, int sweeps, int post)
{
  long n = l->nx * l->ny;
  int nw = 0;
  for (int s = 0; s < sweeps; ++s)
  {
    int halves = mg->relax == 1 ? 1 : 2;
    for (int h = 0; h < halves; ++h)
    {
      const double* in = (nw & 1) ? l->t : l->u;
      double* out      = (nw & 1) ? l->u : l->t;
      int color        = (post && mg->relax == 2) ? 1 - h : h;
      for (long j = 0; j < l->ny; ++j)
        for (long i = 0; i < l->nx; ++i)
        {
          long k = j * l->nx + i;
          if (mg->relax == 1)
          {
            per_pt q  = per_point(in, l, i, j);
            double wd = 0.8 * (1.0 / q.d);
            out[k]    = fma(wd, l->f[k] - per_m(&q, in[k]), in[k]);
          }
          else if (((i + j) & 1) != color) out[k] = in[k];
          else
          {
            per_pt q = per_point(in, l, i, j);
            double v = fma(q.w, q.uW, l->f[k]);
            v        = fma(q.e, q.uE, v);
            v        = fma(q.s, q.uS, v);
            v        = fma(q.n, q.uN, v);
            out[k]   = v / q.d;
          }
        }
      ++nw;
    }
  }
  if (nw & 1) memcpy(l->u, l->t, n * sizeof(double));
}

static orc_pfmg* pfmg_create_periodic(const orc_prob* p, double gamma, int relax, int nrelax)
{
  orc_pfmg* mg = (orc_pfmg*)calloc(1, sizeof(orc_pfmg));
  mg->relax    = relax;
  mg->nrelax   = nrelax;
  mg->periodic = 1;
  for (int lev = 0; lev < 64; ++lev)
  {
    pfmg_level l;
    memset(&l, 0, sizeof(l));
    if (lev == 0)
    {
      l.nx  = p->nx;
      l.ny  = p->ny;
      l.axf = (double*)malloc(l.nx * sizeof(double));
      l.ayf = (double*)malloc(l.ny * sizeof(double));
      for (long i = 0; i < l.nx; ++i) l.axf[i] = gamma * p->Dxe[i];
      for (long j = 0; j < l.ny; ++j) l.ayf[j] = gamma * p->Dyn[j];
    }
    else
    {
      const pfmg_level* f = &mg->L[lev - 1];
      l.nx  = f->dir == 0 ? f->nx / 2 : f->nx;
      l.ny  = f->dir == 1 ? f->ny / 2 : f->ny;
      l.axf = (double*)malloc(l.nx * sizeof(double));
      l.ayf = (double*)malloc(l.ny * sizeof(double));
      for (long I = 0; I < l.nx; ++I)
        l.axf[I] = f->dir == 0 ? series_coupling(f->axf[2 * I + 1], f->axf[(2 * I + 2) % f->nx]) : f->axf[I];
      for (long J = 0; J < l.ny; ++J)
        l.ayf[J] = f->dir == 1 ? series_coupling(f->ayf[2 * J + 1], f->ayf[(2 * J + 2) % f->ny]) : f->ayf[J];
    }
    double axm = 0.0, aym = 0.0;
    for (long i = 0; i < l.nx; ++i) axm = l.axf[i] > axm ? l.axf[i] : axm;
    for (long j = 0; j < l.ny; ++j) aym = l.ayf[j] > aym ? l.ayf[j] : aym;
    int cx = l.nx > 2 && l.nx % 2 == 0, cy = l.ny > 2 && l.ny % 2 == 0;
    if (cx && (axm >= aym || !cy)) l.dir = 0;
    else if (cy) l.dir = 1;
    else l.dir = -1;
    long n = l.nx * l.ny;
    l.f    = (double*)calloc(n, sizeof(double));
    l.u    = (double*)calloc(n, sizeof(double));
    l.t    = (double*)calloc(n, sizeof(double));
    mg->L[lev] = l;
    mg->nl     = lev + 1;
    if (l.dir < 0) break;
  }
  return mg;
}

static void per_apply(orc_pfmg* mg, const double* r, double* z)
{
  pfmg_level* L = mg->L;
  memcpy(L[0].f, r, (size_t)(L[0].nx * L[0].ny) * sizeof(double));
  for (int lev = 0; lev < mg->nl; ++lev)
  {
    pfmg_level* l = &L[lev];
    memset(l->u, 0, (size_t)(l->nx * l->ny) * sizeof(double));
    if (l->dir < 0)
    {
      per_smooth(mg, l, 8, 0);
      break;
    }
    per_smooth(mg, l, mg->nrelax, 0);
    for (long j = 0; j < l->ny; ++j)
      for (long i = 0; i < l->nx; ++i)
      {
        per_pt q               = per_point(l->u, l, i, j);
        l->t[j * l->nx + i] = l->f[j * l->nx + i] - per_m(&q, l->u[j * l->nx + i]);
      }
    pfmg_level* c = &L[lev + 1];
    for (long J = 0; J < c->ny; ++J)
      for (long I = 0; I < c->nx; ++I)
      {
        double a, b, cc;
        if (l->dir == 0)
        {
          a  = l->t[J * l->nx + 2 * I];
          b  = l->t[J * l->nx + 2 * I + 1];
          cc = l->t[J * l->nx + pwrap(2 * I + 2, l->nx)];
        }
        else
        {
          a  = l->t[(2 * J) * l->nx + I];
          b  = l->t[(2 * J + 1) * l->nx + I];
          cc = l->t[pwrap(2 * J + 2, l->ny) * l->nx + I];
        }
        c->f[J * c->nx + I] = fma(0.5, b, 0.25 * (a + cc));
      }
  }
  for (int lev = mg->nl - 2; lev >= 0; --lev)
  {
    pfmg_level* l = &L[lev];
    pfmg_level* c = &L[lev + 1];
    for (long j = 0; j < l->ny; ++j)
      for (long i = 0; i < l->nx; ++i)
      {
        long q = l->dir == 0 ? i : j, Q = q >> 1;
        double e;
        if (q & 1) e = l->dir == 0 ? c->u[j * c->nx + Q] : c->u[Q * c->nx + i];
        else
        {
          long Qm   = pwrap(Q - 1, l->dir == 0 ? c->nx : c->ny);
          double lo = l->dir == 0 ? c->u[j * c->nx + Qm] : c->u[Qm * c->nx + i];
          double hi = l->dir == 0 ? c->u[j * c->nx + Q] : c->u[Q * c->nx + i];
          e         = 0.5 * (lo + hi);
        }
        l->u[j * l->nx + i] += e;
      }
    per_smooth(mg, l, mg->nrelax, 1);
  }
  memcpy(z, L[0].u, (size_t)(L[0].nx * L[0].ny) * sizeof(double));
}

static double pat(const double* u, long nx, long ny, long i, long j)
{
  return (i >= 0 && i < nx && j >= 0 && j < ny) ? u[j * nx + i] : 0.0;
}

static double pfmg_m(const double* u, const pfmg_level* l, long i, long j)
{
  double sx = pat(u, l->nx, l->ny, i - 1, j) + pat(u, l->nx, l->ny, i + 1, j);
  double sy = pat(u, l->nx, l->ny, i, j - 1) + pat(u, l->nx, l->ny, i, j + 1);
  double m  = l->d * u[j * l->nx + i];
  m         = fma(-l->ax, sx, m);
  m         = fma(-l->ay, sy, m);
  return m;
}

static void pfmg_smooth(orc_pfmg* mg, pfmg_level* l, int sweeps, int post)
{
  long n = l->nx * l->ny;
  if (mg->relax == 1)
  {
    for (int s = 0; s < sweeps; ++s)
    {
      const double* in = (s & 1) ? l->t : l->u;
      double* out      = (s & 1) ? l->u : l->t;
      for (long j = 0; j < l->ny; ++j)
        for (long i = 0; i < l->nx; ++i)
        {
          long k = j * l->nx + i;
          out[k] = fma(l->wd, l->f[k] - pfmg_m(in, l, i, j), in[k]);
        }
    }
    if (sweeps & 1) memcpy(l->u, l->t, n * sizeof(double));
  }
  else
  {
    for (int s = 0; s < sweeps; ++s)
      for (int h = 0; h < 2; ++h)
      {
        int color = (post && mg->relax == 2) ? 1 - h : h; /* relax 3: red, black also after */
        for (long j = 0; j < l->ny; ++j)
          for (long i = (j + color) & 1; i < l->nx; i += 2)
          {
            double sx = pat(l->u, l->nx, l->ny, i - 1, j) + pat(l->u, l->nx, l->ny, i + 1, j);
            double sy = pat(l->u, l->nx, l->ny, i, j - 1) + pat(l->u, l->nx, l->ny, i, j + 1);
            double v  = fma(l->ax, sx, l->f[j * l->nx + i]);
            v         = fma(l->ay, sy, v);
            l->u[j * l->nx + i] = l->dinv * v;
          }
      }
  }
}

static orc_pfmg* pfmg_create(const orc_prob* p, double gamma, int relax, int nrelax)
{
  if (p->kind == ORC_PERIODIC) return pfmg_create_periodic(p, gamma, relax, nrelax);
  orc_pfmg* mg = (orc_pfmg*)calloc(1, sizeof(orc_pfmg));
  mg->relax    = relax;
  mg->nrelax   = nrelax;
  for (int lev = 0; lev < 64; ++lev)
  {
    pfmg_level l;
    memset(&l, 0, sizeof(l));
    if (lev == 0)
    {
      l.nx = p->nx;
      l.ny = p->ny;
      l.ax = gamma * p->cx;
      l.ay = gamma * p->cy;
      l.d  = 1.0 - gamma * p->cc;
    }
    else
    {
      l = mg->L[lev - 1];
      if (l.dir == 0)
      {
        l.nx = l.nx / 2;
        l.ax = l.ax * 0.25;
      }
      else
      {
        l.ny = l.ny / 2;
        l.ay = l.ay * 0.25;
      }
      l.d = 1.0 + 2.0 * (l.ax + l.ay);
    }
    l.dinv = 1.0 / l.d;
    l.wd   = 0.8 * l.dinv;
    if (l.nx > 2 && (l.ax >= l.ay || l.ny <= 2)) l.dir = 0;
    else if (l.ny > 2) l.dir = 1;
    else l.dir = -1;
    long n = l.nx * l.ny;
    l.f    = (double*)calloc(n, sizeof(double));
    l.u    = (double*)calloc(n, sizeof(double));
    l.t    = (double*)calloc(n, sizeof(double));
    mg->L[lev] = l;
    mg->nl     = lev + 1;
    if (l.dir < 0) break;
  }
  return mg;
}

static void pfmg_destroy(orc_pfmg* mg)
{
  for (int k = 0; k < mg->nl; ++k)
  {
    free(mg->L[k].f);
    free(mg->L[k].u);
    free(mg->L[k].t);
    free(mg->L[k].axf);
    free(mg->L[k].ayf);
  }
  free(mg);
}

static void pfmg_apply(orc_pfmg* mg, const double* r, double* z)
{
  if (mg->periodic)
  {
    per_apply(mg, r, z);
    return;
  }
  pfmg_level* L = mg->L;
  memcpy(L[0].f, r, (size_t)(L[0].nx * L[0].ny) * sizeof(double));
  for (int lev = 0; lev < mg->nl; ++lev)
  {
    pfmg_level* l = &L[lev];
    memset(l->u, 0, (size_t)(l->nx * l->ny) * sizeof(double));
    if (l->dir < 0)
    {
      pfmg_smooth(mg, l, 8, 0);
      break;
    }
    pfmg_smooth(mg, l, mg->nrelax, 0);
    for (long j = 0; j < l->ny; ++j)
      for (long i = 0; i < l->nx; ++i) l->t[j * l->nx + i] = l->f[j * l->nx + i] - pfmg_m(l->u, l, i, j);
    pfmg_level* c = &L[lev + 1];
    for (long J = 0; J < c->ny; ++J)
      for (long I = 0; I < c->nx; ++I)
      {
        double a, b, cc;
        if (l->dir == 0)
        {
          a  = pat(l->t, l->nx, l->ny, 2 * I, J);
          b  = pat(l->t, l->nx, l->ny, 2 * I + 1, J);
          cc = pat(l->t, l->nx, l->ny, 2 * I + 2, J);
        }
        else
        {
          a  = pat(l->t, l->nx, l->ny, I, 2 * J);
          b  = pat(l->t, l->nx, l->ny, I, 2 * J + 1);
          cc = pat(l->t, l->nx, l->ny, I, 2 * J + 2);
        }
        c->f[J * c->nx + I] = fma(0.5, b, 0.25 * (a + cc));
      }
  }
  for (int lev = mg->nl - 2; lev >= 0; --lev)
  {
    pfmg_level* l = &L[lev];
    pfmg_level* c = &L[lev + 1];
    for (long j = 0; j < l->ny; ++j)
      for (long i = 0; i < l->nx; ++i)
      {
        long q = l->dir == 0 ? i : j;
        double e;
        if (q & 1)
          e = l->dir == 0 ? pat(c->u, c->nx, c->ny, q >> 1, j) : pat(c->u, c->nx, c->ny, i, q >> 1);
        else
        {
          long Q    = q >> 1;
          double lo = l->dir == 0 ? pat(c->u, c->nx, c->ny, Q - 1, j) : pat(c->u, c->nx, c->ny, i, Q - 1);
          double hi = l->dir == 0 ? pat(c->u, c->nx, c->ny, Q, j) : pat(c->u, c->nx, c->ny, i, Q);
          e         = 0.5 * (lo + hi);
        }
        l->u[j * l->nx + i] += e;
      }
    pfmg_smooth(mg, l, mg->nrelax, 1);
  }
  memcpy(z, L[0].u, (size_t)(L[0].nx * L[0].ny) * sizeof(double));
}

int orc_pfmg_vcycle(const orc_prob* p, double gamma, int relax, int nrelax, const double* r, double* z, int* nlevels)
{
  orc_pfmg* mg = pfmg_create(p, gamma, relax, nrelax);
  pfmg_apply(mg, r, z);
  if (nlevels) *nlevels = mg->nl;
  pfmg_destroy(mg);
  return 0;
}

/* CG with the PFMG preconditioner, the operation sequence of orc_pcg_generic */
int orc_pcg_pfmg(const orc_prob* p, double gamma, int relax, int nrelax, const double* b, double* x, double tol,
                 int maxl, int* iters, double* relres)
{
  long n   = (long)p->nx * p->ny;
  gen_op o = {p, gamma, 0.0, 2, (double*)malloc(n * sizeof(double)), pfmg_create(p, gamma, relax, nrelax)};
  int ret  = gen_pcg(&o, b, x, tol, maxl, iters, relres);
  pfmg_destroy(o.mg);
  free(o.tmp);
  return ret;
}

/* SDIRK2 (orc_sdirk2's stages) with CG + the PFMG-role V-cycle (STS_SDIRK2EvolvePFMG) */
int orc_sdirk2_pfmg(const orc_prob* p, double t0, double h, int nsteps, double tol, int maxl, int relax, int nrelax,
                    double* y, long* total_iters)
{
  long n      = (long)p->nx * p->ny;
  double g    = 1.0 - sqrt(0.5);
  double* f   = (double*)malloc(n * sizeof(double));
  double* f1  = (double*)malloc(n * sizeof(double));
  double* rhs = (double*)malloc(n * sizeof(double));
  double* d   = (double*)malloc(n * sizeof(double));
  double* Y1  = (double*)malloc(n * sizeof(double));
  double relres;
  long iters = 0;
  double t   = t0;
  int it;
  for (int s = 0; s < nsteps; ++s)
  {
    double hg = h * g;
    orc_rhs(p, t + g * h, y, f);
    v_scale(n, hg, f, rhs);
    orc_pcg_pfmg(p, hg, relax, nrelax, rhs, d, tol, maxl, &it, &relres);
    iters += it;
    v_linsum(n, 1.0, y, 1.0, d, Y1);
    orc_rhs(p, t + g * h, Y1, f1);
    orc_rhs(p, t + h, y, f);
    double h1g = h * (1.0 - g);
    v_linsum(n, h1g, f1, hg, f, rhs);
    orc_pcg_pfmg(p, hg, relax, nrelax, rhs, d, tol, maxl, &it, &relres);
    iters += it;
    v_linsum(n, 1.0, y, 1.0, d, y);
    t = t0 + (s + 1) * h;
  }
  *total_iters = iters;
  free(f);
  free(f1);
  free(rhs);
  free(d);
  free(Y1);
  return 0;
}

/* SDIRK2 (orc_sdirk2's stages) with a generic solver: ls 0 = PCG, 1 = SPGMR */
int orc_sdirk2_ls(const orc_prob* p, double t0, double h, int nsteps, double tol, int ls, int maxl,
                  int max_restarts, int gstype, int jacobi, double* y, long* total_iters)
{
  long n     = (long)p->nx * p->ny;
  double g   = 1.0 - sqrt(0.5);
  double* f  = (double*)malloc(n * sizeof(double));
  double* f1 = (double*)malloc(n * sizeof(double));
  double* rhs = (double*)malloc(n * sizeof(double));
  double* d   = (double*)malloc(n * sizeof(double));
  double* Y1  = (double*)malloc(n * sizeof(double));
  double relres;
  long iters = 0;
  double t   = t0;
  int it;
  for (int s = 0; s < nsteps; ++s)
  {
    double hg = h * g;
    orc_rhs(p, t + g * h, y, f);
    v_scale(n, hg, f, rhs);
    if (ls == 0) orc_pcg_generic(p, hg, jacobi, rhs, d, tol, maxl, &it, &relres);
    else orc_spgmr(p, hg, jacobi, rhs, d, tol, maxl, max_restarts, gstype, &it, &relres);
    iters += it;
    v_linsum(n, 1.0, y, 1.0, d, Y1);
    orc_rhs(p, t + g * h, Y1, f1);
    orc_rhs(p, t + h, y, f);
    double h1g = h * (1.0 - g);
    v_linsum(n, h1g, f1, hg, f, rhs);
    if (ls == 0) orc_pcg_generic(p, hg, jacobi, rhs, d, tol, maxl, &it, &relres);
    else orc_spgmr(p, hg, jacobi, rhs, d, tol, maxl, max_restarts, gstype, &it, &relres);
    iters += it;
    v_linsum(n, 1.0, y, 1.0, d, y);
    t = t0 + (s + 1) * h;
  }
  *total_iters = iters;
  free(f);
  free(f1);
  free(rhs);
  free(d);
  free(Y1);
  return 0;
}

/* ------------------------------------------------------------------------------------
 * SSP methods of LSRKStepCreateSSP (diffusion_2D/main.cpp:250-294), restated from Ketcheson
 * (SIAM J. Sci. Comput. 30, 2008) with this project's embedded estimates, in the exact
 * operation sequence of the product's generic path (N_Vector ops: LinearSum z = fma(a, x, b y),
 * Scale z = c x, LinearCombination acc = c0 x0 then fma(c_k, x_k, acc)).
 * ----------------------------------------------------------------------------------*/
static int ssp_valid(int type, int s)
{
  if (type == 2) return s >= 2 && s <= 1024;
  if (type == 3)
  {
    int n = (int)lround(sqrt((double)s));
    return n >= 2 && n * n == s && s <= 1024;
  }
  return type == 4 && s == 10;
}

/* b, c and the error weights w = b - bhat of the SSP method (as the product computes them) */
int orc_ssp_weights(int type, int s, double* b, double* c, double* w)
{
  if (!ssp_valid(type, s)) return -1;
  /* registers: y coefficient + multiples of h F_j */
  double* q1 = (double*)calloc(s, sizeof(double));
  double* q2 = (double*)calloc(s, sizeof(double));
  double* fin = (double*)calloc(s, sizeof(double));
  double* A = (type == 4) ? (double*)calloc((size_t)s * s, sizeof(double)) : NULL;
  double q1y = 1.0, q2y = 1.0, finy = 1.0;
  int j = 0;
#define STAGE(q)                                                                                        \
  do                                                                                                    \
  {                                                                                                     \
    double cj = 0.0;                                                                                    \
    for (int k = 0; k < s; ++k)                                                                         \
    {                                                                                                   \
      if (A) A[(size_t)j * s + k] = (q)[k];                                                             \
      cj += (q)[k];                                                                                     \
    }                                                                                                   \
    c[j] = cj;                                                                                          \
    ++j;                                                                                                \
  } while (0)
  if (type == 2)
  {
    double r = s - 1.0;
    for (int i = 0; i < s - 1; ++i)
    {
      STAGE(q1);
      q1[j - 1] += 1.0 / r;
    }
    STAGE(q1);
    q1[j - 1] += 1.0 / r; /* t = q1 + (1/r) e_{s-1} (q1 is not used again) */
    for (int k = 0; k < s; ++k) fin[k] = (1.0 / s) * 0.0 + ((s - 1.0) / s) * q1[k];
    finy = (1.0 / s) * 1.0 + ((s - 1.0) / s) * q1y;
  }
  else if (type == 3)
  {
    int n = (int)lround(sqrt((double)s));
    double r = (double)(n * n - n);
    int e1 = (n - 1) * (n - 2) / 2, e2 = n * (n + 1) / 2;
    for (int i = 1; i <= e1; ++i)
    {
      STAGE(q1);
      q1[j - 1] += 1.0 / r;
    }
    memcpy(q2, q1, s * sizeof(double));
    q2y = q1y;
    for (int i = e1 + 1; i <= e2 - 1; ++i)
    {
      STAGE(q1);
      q1[j - 1] += 1.0 / r;
    }
    STAGE(q1);
    q1[j - 1] += 1.0 / r;
    double a = (double)n / (2 * n - 1), bb = (n - 1.0) / (2 * n - 1);
    for (int k = 0; k < s; ++k) q1[k] = a * q2[k] + bb * q1[k];
    q1y = a * q2y + bb * q1y;
    for (int i = e2 + 1; i <= n * n; ++i)
    {
      STAGE(q1);
      q1[j - 1] += 1.0 / r;
    }
    memcpy(fin, q1, s * sizeof(double));
    finy = q1y;
  }
  else
  {
    for (int i = 1; i <= 5; ++i)
    {
      STAGE(q1);
      q1[j - 1] += 1.0 / 6.0;
    }
    for (int k = 0; k < s; ++k) q2[k] = (1.0 / 25.0) * q2[k] + (9.0 / 25.0) * q1[k];
    q2y = (1.0 / 25.0) * q2y + (9.0 / 25.0) * q1y;
    for (int k = 0; k < s; ++k) q1[k] = 15.0 * q2[k] + -5.0 * q1[k];
    q1y = 15.0 * q2y + -5.0 * q1y;
    for (int i = 6; i <= 9; ++i)
    {
      STAGE(q1);
      q1[j - 1] += 1.0 / 6.0;
    }
    STAGE(q1);
    for (int k = 0; k < s; ++k) fin[k] = 1.0 * q2[k] + (3.0 / 5.0) * q1[k];
    fin[j - 1] += 1.0 / 10.0;
    finy = 1.0 * q2y + (3.0 / 5.0) * q1y;
  }
#undef STAGE
  (void)finy;
  memcpy(b, fin, s * sizeof(double));
  double* bh = (double*)calloc(s, sizeof(double));
  if (type == 2)
    for (int k = 0; k < s; ++k) bh[k] = (k < s - 1) ? 1.0 / (s - 1.0) : 0.0;
  else
  {
    int m = (type == 4) ? 4 : 2;
    double* Cm = (double*)calloc((size_t)m * s, sizeof(double));
    double d[4] = {1.0, 0.5, 1.0 / 3.0, 1.0 / 6.0};
    for (int k = 0; k < s; ++k)
    {
      Cm[k]     = 1.0;
      Cm[s + k] = c[k];
      if (m == 4)
      {
        Cm[2 * s + k] = c[k] * c[k];
        double ac     = 0.0;
        for (int l = 0; l < s; ++l) ac += A[(size_t)k * s + l] * c[l];
        Cm[3 * s + k] = ac;
      }
    }
    double G[16], lam[4];
    /* reference weights: uniform; SSP(10,4) (uniform b) alternating 0.15 / 0.05 */
#define UREF(k) ((type == 4) ? (((k) & 1) ? 0.05 : 0.15) : 1.0 / s)
    for (int a = 0; a < m; ++a)
    {
      double v = 0.0;
      for (int k = 0; k < s; ++k) v += Cm[a * s + k] * UREF(k);
      lam[a] = v - d[a];
      for (int e = 0; e < m; ++e)
      {
        double g = 0.0;
        for (int k = 0; k < s; ++k) g += Cm[a * s + k] * Cm[e * s + k];
        G[a * m + e] = g;
      }
    }
    for (int col = 0; col < m; ++col)
    {
      int pr = col;
      for (int rr = col + 1; rr < m; ++rr)
        if (fabs(G[rr * m + col]) > fabs(G[pr * m + col])) pr = rr;
      if (pr != col)
      {
        for (int e = 0; e < m; ++e)
        {
          double t = G[col * m + e];
          G[col * m + e] = G[pr * m + e];
          G[pr * m + e]  = t;
        }
        double t = lam[col];
        lam[col] = lam[pr];
        lam[pr]  = t;
      }
      for (int rr = col + 1; rr < m; ++rr)
      {
        double f = G[rr * m + col] / G[col * m + col];
        for (int e = col; e < m; ++e) G[rr * m + e] -= f * G[col * m + e];
        lam[rr] -= f * lam[col];
      }
    }
    for (int col = m - 1; col >= 0; --col)
    {
      for (int e = col + 1; e < m; ++e) lam[col] -= G[col * m + e] * lam[e];
      lam[col] /= G[col * m + col];
    }
    for (int k = 0; k < s; ++k)
    {
      double v = UREF(k);
      for (int a = 0; a < m; ++a) v -= Cm[a * s + k] * lam[a];
      bh[k] = v;
    }
#undef UREF
    free(Cm);
  }
  for (int k = 0; k < s; ++k) w[k] = b[k] - bh[k];
  free(bh);
  free(q1);
  free(q2);
  free(fin);
  free(A);
  return 0;
}

/* N_Vector operation restatements (the product's arithmetic) */
/* Adaptive SSP integration (type 2 = SSP(s,2), 3 = SSP(s,3), 4 = SSP(10,4)); state in st as
 * for orc_lsrk_evolve. The controller order is the embedding order + 1. */
static int ssp_steps(const orc_prob* p, const orc_opts* o, int type, int s, orc_state* st, double tout,
                     double clip, double* y)
{
  long n    = (long)p->nx * p->ny;
  long maxs = o->maxsteps > 0 ? o->maxsteps : 500;
  double ordv = (type == 2) ? 2.0 : (type == 3 ? 3.0 : 4.0);
  double *b = (double*)malloc(s * sizeof(double)), *c = (double*)malloc(s * sizeof(double)),
         *w = (double*)malloc(s * sizeof(double));
  orc_ssp_weights(type, s, b, c, w);
  double *q1 = (double*)malloc(n * sizeof(double)), *q2 = (double*)malloc(n * sizeof(double)),
         *G = (double*)malloc(n * sizeof(double)), *E = (double*)malloc(n * sizeof(double)),
         *ynew = (double*)malloc(n * sizeof(double));
  int ret = 0;
  if (!st->initialized)
  {
    st->F = (double*)malloc(n * sizeof(double));
    st->Ff = NULL;
    orc_rhs(p, st->t, y, st->F);
    st->nfe++;
    st->hnext       = (o->hfixed > 0.0) ? o->hfixed : 0.0;
    st->initialized = 1;
  }
  long nsteps_call = 0;
  while (st->t < clip && st->t < tout)
  {
    if (nsteps_call >= maxs)
    {
      ret = -1;
      break;
    }
    if (!(st->hnext > 0.0))
    {
      st->hnext = initial_step_ord(p, o, st->t, y, st->F, (tout < clip ? tout : clip) - st->t, 0.0, &st->nfe,
                                   ordv);
      if (!(st->hnext > 0.0))
      {
        ret = -3; /* non-finite state: no usable step */
        goto done;
      }
    }
    int nef = 0;
    for (;;)
    {
      double h = st->hnext;
      int clipped = 0;
      if (st->t + h >= clip)
      {
        h       = clip - st->t;
        clipped = 1;
      }
      st->nst_attempts++;
      st->d.interp_ready = 0;
      int j = 0;
      /* stage: derivative of register q (stage 0 reuses F), E += h w_j G */
#define SSP_STAGE(q, g)                                                                                 \
  do                                                                                                    \
  {                                                                                                     \
    if (j == 0) g = st->F;                                                                              \
    else                                                                                                \
    {                                                                                                   \
      orc_rhs(p, st->t + c[j] * h, q, G);                                                               \
      g = G;                                                                                            \
    }                                                                                                   \
    if (j == 0) v_scale(n, h * w[0], g, E);                                                             \
    else v_linsum(n, h * w[j], g, 1.0, E, E);                                                           \
    ++j;                                                                                                \
  } while (0)
      const double* g;
      v_scale(n, 1.0, y, q1);
      if (type == 2)
      {
        double hr = h / (s - 1.0);
        for (int i = 0; i < s - 1; ++i)
        {
          SSP_STAGE(q1, g);
          v_linsum(n, hr, g, 1.0, q1, q1);
        }
        SSP_STAGE(q1, g);
        double cf[3] = {1.0 / s, (s - 1.0) / s, (s - 1.0) / s * hr};
        const double* X[3] = {y, q1, g};
        v_lincomb(n, 3, cf, X, ynew);
      }
      else if (type == 3)
      {
        int nn = (int)lround(sqrt((double)s));
        double hr = h / (double)(nn * nn - nn);
        int e1 = (nn - 1) * (nn - 2) / 2, e2 = nn * (nn + 1) / 2;
        for (int i = 1; i <= e1; ++i)
        {
          SSP_STAGE(q1, g);
          v_linsum(n, hr, g, 1.0, q1, q1);
        }
        v_scale(n, 1.0, q1, q2);
        for (int i = e1 + 1; i <= e2 - 1; ++i)
        {
          SSP_STAGE(q1, g);
          v_linsum(n, hr, g, 1.0, q1, q1);
        }
        SSP_STAGE(q1, g);
        {
          double cf[3] = {(double)nn / (2 * nn - 1), (nn - 1.0) / (2 * nn - 1), (nn - 1.0) / (2 * nn - 1) * hr};
          const double* X[3] = {q2, q1, g};
          v_lincomb(n, 3, cf, X, q1);
        }
        for (int i = e2 + 1; i <= nn * nn; ++i)
        {
          SSP_STAGE(q1, g);
          v_linsum(n, hr, g, 1.0, q1, q1);
        }
        v_scale(n, 1.0, q1, ynew);
      }
      else
      {
        v_scale(n, 1.0, y, q2);
        for (int i = 1; i <= 5; ++i)
        {
          SSP_STAGE(q1, g);
          v_linsum(n, h / 6.0, g, 1.0, q1, q1);
        }
        {
          double cf[2] = {1.0 / 25.0, 9.0 / 25.0};
          const double* X[2] = {q2, q1};
          v_lincomb(n, 2, cf, X, q2);
        }
        {
          double cf[2] = {15.0, -5.0};
          const double* X[2] = {q2, q1};
          v_lincomb(n, 2, cf, X, q1);
        }
        for (int i = 6; i <= 9; ++i)
        {
          SSP_STAGE(q1, g);
          v_linsum(n, h / 6.0, g, 1.0, q1, q1);
        }
        SSP_STAGE(q1, g);
        double cf[3] = {1.0, 3.0 / 5.0, h / 10.0};
        const double* X[3] = {q2, q1, g};
        v_lincomb(n, 3, cf, X, ynew);
      }
#undef SSP_STAGE
      st->nfe += s - 1;
      double dsm = wrms_ewt(o, E, y, n);
      st->stages_total += s;
      if (s > st->stage_max) st->stage_max = s;
      if (o->hfixed > 0.0 || dsm <= 1.0)
      {
        st->t = clipped ? clip : st->t + h;
        memcpy(st->d.yold, y, n * sizeof(double));
        memcpy(st->d.fold, st->F, n * sizeof(double));
        memcpy(y, ynew, n * sizeof(double));
        orc_rhs(p, st->t, y, st->F);
        st->nfe++;
        st->d.interp_ready = 1;
        const double hprev = st->hlast;
        st->hlast          = h;
        if (o->hfixed > 0.0) st->hnext = o->hfixed;
        else
        {
          double hn  = controller_ord(o->controller, h, dsm, st->ep1, st->ep2, hprev, st->nhist, ordv);
          double eta = SAFETY * hn / h;
          double emx = (st->nst == 0) ? ETAMX1 : (st->after_fail ? 1.0 : GROWTH);
          if (eta > emx) eta = emx;
          if (eta >= LBOUND && eta <= UBOUND) eta = 1.0;
          st->hnext = h * eta;
          st->ep2   = st->ep1;
          st->ep1   = dsm;
          st->nhist++;
        }
        st->after_fail = 0;
        st->nst++;
        nsteps_call++;
        break;
      }
      st->netf++;
      nef++;
      if (!(dsm == dsm) || nef > 20)
      {
        ret = -3;
        goto done;
      }
      double hn  = controller_ord(o->controller, h, dsm, st->ep1, st->ep2, st->hlast, st->nhist, ordv);
      double eta = SAFETY * hn / h;
      if (eta > 1.0) eta = 1.0;
      if (nef >= SMALL_NEF && eta > ETAMXF) eta = ETAMXF;
      if (eta < ETAMIN) eta = ETAMIN;
      st->hnext      = h * eta;
      st->after_fail = 1;
    }
  }
done:
  free(b);
  free(c);
  free(w);
  free(q1);
  free(q2);
  free(G);
  free(E);
  free(ynew);
  return ret;
}

static int ssp_fnew(void* ctx, const double** fnew)
{
  *fnew = ((orc_state*)ctx)->F; /* f(t_n, y_n), evaluated at every accepted step */
  return 0;
}

int orc_ssp_evolve(const orc_prob* p, const orc_opts* o, int type, int s, orc_state* st, double tout, double* y)
{
  if (!ssp_valid(type, s)) return -4;
  long n        = (long)p->nx * p->ny;
  const int deg = (type == 2) ? 1 : (type == 3 ? 2 : 3); /* min(q - 1, 5) */
  int ret;
  dense_alloc(&st->d, n, 1, y);
  if (dense_entry(&st->d, n, st->t, st->hlast, deg, ssp_fnew, st, 0, tout, y, &ret)) return ret;
  ret = ssp_steps(p, o, type, s, st, tout, st->d.tstopset ? st->d.tstop : INFINITY, st->d.ycur);
  return dense_finish(&st->d, n, st->t, st->hlast, deg, ssp_fnew, st, 0, tout, y, ret);
}

/* ------------------------------------------------------------------------------------
 * ARKStep restated in the product's operation sequence (csrc/arkstep.cu): implicit DIRK
 * (ARKODE_SDIRK_2_1_2, ARKODE_ARK324L2SA_DIRK_4_2_3) with Newton corrections solved by the
 * generic PCG / SPGMR above (no, Jacobi or PFMG preconditioner), or explicit ERK
 * (ARKODE_HEUN_EULER_2_1_2, ARKODE_BOGACKI_SHAMPINE_4_2_3, ARKODE_ZONNEVELD_5_3_4); ARKODE's
 * Newton convergence test, linear tolerance eplifac * 0.1 in the WRMS norm, PSetup schedule,
 * embedded error estimate and the LSRKStep controllers with order p + 1
 * (diffusion_2D/main.cpp:239-330 create and configure it).
 * ----------------------------------------------------------------------------------*/
static int ark_table(int implicit, int order, int* s, int* q, int* pe, double* A, double* b, double* d, double* c)
{
  memset(A, 0, 25 * sizeof(double));
  if (implicit && order == 2)
  {
    *s = 2; *q = 2; *pe = 1;
    A[0] = 1.0; A[2] = -1.0; A[3] = 1.0;
    b[0] = 0.5; b[1] = 0.5; d[0] = 1.0; d[1] = 0.0; c[0] = 1.0; c[1] = 0.0;
  }
  else if (implicit && order == 3)
  { /* Kennedy & Carpenter (2003), ARK3(2)4L[2]SA, implicit part */
    const double g = 1767732205903.0 / 4055673282236.0;
    *s = 4; *q = 3; *pe = 2;
    A[4] = g; A[5] = g;
    A[8] = 2746238789719.0 / 10658868560708.0; A[9] = -640167445237.0 / 6845629431997.0; A[10] = g;
    A[12] = 1471266399579.0 / 7840856788654.0; A[13] = -4482444167858.0 / 7529755066697.0;
    A[14] = 11266239266428.0 / 11593286722821.0; A[15] = g;
    for (int i = 0; i < 4; ++i) b[i] = A[12 + i];
    d[0] = 2756255671327.0 / 12835298489170.0; d[1] = -10771552573575.0 / 22201958757719.0;
    d[2] = 9247589265047.0 / 10645013368117.0; d[3] = 2193209047091.0 / 5459859503100.0;
    c[0] = 0.0; c[1] = 2.0 * g; c[2] = 3.0 / 5.0; c[3] = 1.0;
  }
  else if (!implicit && order == 2)
  { /* Heun-Euler */
    *s = 2; *q = 2; *pe = 1;
    A[2] = 1.0; b[0] = 0.5; b[1] = 0.5; d[0] = 1.0; d[1] = 0.0; c[0] = 0.0; c[1] = 1.0;
  }
  else if (!implicit && order == 3)
  { /* Bogacki-Shampine */
    *s = 4; *q = 3; *pe = 2;
    A[4] = 0.5; A[9] = 0.75; A[12] = 2.0 / 9.0; A[13] = 1.0 / 3.0; A[14] = 4.0 / 9.0;
    b[0] = 2.0 / 9.0; b[1] = 1.0 / 3.0; b[2] = 4.0 / 9.0; b[3] = 0.0;
    d[0] = 7.0 / 24.0; d[1] = 0.25; d[2] = 1.0 / 3.0; d[3] = 0.125;
    c[0] = 0.0; c[1] = 0.5; c[2] = 0.75; c[3] = 1.0;
  }
  else if (!implicit && order == 4)
  { /* Zonneveld */
    *s = 5; *q = 4; *pe = 3;
    A[5] = 0.5; A[11] = 0.5; A[17] = 1.0;
    A[20] = 5.0 / 32.0; A[21] = 7.0 / 32.0; A[22] = 13.0 / 32.0; A[23] = -1.0 / 32.0;
    b[0] = 1.0 / 6.0; b[1] = 1.0 / 3.0; b[2] = 1.0 / 3.0; b[3] = 1.0 / 6.0; b[4] = 0.0;
    d[0] = -0.5; d[1] = 7.0 / 3.0; d[2] = 7.0 / 3.0; d[3] = 13.0 / 6.0; d[4] = -16.0 / 3.0;
    c[0] = 0.0; c[1] = 0.5; c[2] = 0.5; c[3] = 1.0; c[4] = 0.75;
  }
  else return -1;
  return 0;
}

int orc_ark_table(int implicit, int order, int* s, int* q, int* pe, double* A, double* b, double* d, double* c)
{
  double A5[25], b5[5], d5[5], c5[5];
  if (ark_table(implicit, order, s, q, pe, A5, b5, d5, c5)) return -1;
  for (int i = 0; i < *s; ++i)
  {
    b[i] = b5[i];
    d[i] = d5[i];
    c[i] = c5[i];
    for (int j = 0; j < *s; ++j) A[i * *s + j] = A5[i * *s + j];
  }
  return 0;
}

typedef struct {
  const orc_prob* p;
  const orc_ark_opts* o;
  orc_ark_state* st;
  long n;
  int s, pe;
  double A[25], b[5], d[5], c[5];
  double *y, *Fn, *sdata, *z, *res, *del, *ewt, *tmp, *tmp2, *ynew, *F[5];
  orc_pfmg* mg;
  double mg_gamma;
  int fn_current;
} ark_ws;

static void ark_rhs(ark_ws* w, double t, const double* y, double* f)
{
  orc_rhs(w->p, t, y, f);
  if (w->o->implicit) w->st->nfi++;
  else w->st->nfe++;
}

static void ark_ewt(ark_ws* w)
{
  for (long k = 0; k < w->n; ++k) w->ewt[k] = 1.0 / (w->o->rtol * fabs(w->y[k]) + w->o->atol);
}

static int ark_stage(ark_ws* w, int i, double ti, double gamma)
{
  const orc_ark_opts* o = w->o;
  orc_ark_state* st     = w->st;
  long n                = w->n;
  const double epslin   = o->eplifac * 0.1;
  const int msbp        = o->msbp > 0 ? o->msbp : 20;
  memcpy(w->z, w->y, n * sizeof(double));
  double crate = 1.0, delp = 0.0;
  for (int it = 0;; ++it)
  {
    ark_rhs(w, ti, w->z, w->F[i]);
    {
      double cf[3]       = {1.0, gamma, -1.0};
      const double* X[3] = {w->sdata, w->F[i], w->z};
      v_lincomb(n, 3, cf, X, w->res);
    }
    if (it == 0 && o->prec)
    {
      int need = st->force_setup || st->nsetups == 0 || st->nst >= st->nst_setup + msbp ||
                 fabs(gamma / st->gamma_setup - 1.0) > 0.2;
      if (need)
      {
        st->npe++;
        st->nsetups++;
        st->gamma_setup = gamma;
        st->nst_setup   = st->nst;
        st->force_setup = 0;
        crate           = 1.0;
      }
    }
    double bnrm = orc_wrms(w->res, w->ewt, n);
    if (bnrm <= epslin)
      for (long k = 0; k < n; ++k) w->del[k] = 0.0;
    else
    {
      gen_op go = {w->p, gamma, 1.0 / (1.0 - gamma * w->p->cc), o->prec, w->tmp, NULL};
      if (o->prec == 2)
      { /* the product's PFMG PSolve rebuilds its hierarchy when gamma changes */
        if (!w->mg || w->mg_gamma != gamma)
        {
          if (w->mg) pfmg_destroy(w->mg);
          w->mg       = pfmg_create(w->p, gamma, o->pfmg_relax, o->pfmg_nrelax);
          w->mg_gamma = gamma;
        }
        go.mg = w->mg;
      }
      long a0 = g_gen_atimes_calls, p0 = g_gen_psolve_calls;
      int iters = 0;
      double rel;
      int lrc = (o->ls == 0) ? gen_pcg(&go, w->res, w->del, epslin / bnrm, o->maxl, &iters, &rel)
                             : spgmr_op(&go, w->res, w->del, epslin / bnrm, o->maxl, o->max_restarts, o->gstype, 0,
                                        &iters, &rel);
      st->njv += g_gen_atimes_calls - a0;
      st->nps += g_gen_psolve_calls - p0;
      st->nli += iters;
      if (lrc > 0) st->nlcf++;
    }
    st->nni++;
    v_linsum(n, 1.0, w->z, 1.0, w->del, w->z);
    double del = orc_wrms(w->del, w->ewt, n);
    if (o->linear) break;
    if (it > 0) crate = fmax(0.3 * crate, del / delp);
    double dcon = del * fmin(1.0, crate) / 0.1;
    if (dcon <= 1.0) break;
    if (it + 1 >= 3 || (it >= 1 && del > 2.3 * delp) || !(del == del)) return 1;
    delp = del;
  }
  ark_rhs(w, ti, w->z, w->F[i]);
  return 0;
}

static int ark_attempt(ark_ws* w, double h)
{
  const int s = w->s;
  long n      = w->n;
  double cf[6];
  const double* X[6];
  for (int i = 0; i < s; ++i)
  {
    double ti  = w->st->t + w->c[i] * h;
    double aii = w->A[i * s + i];
    if (i == 0 && aii == 0.0)
    {
      if (!w->fn_current)
      {
        ark_rhs(w, w->st->t, w->y, w->Fn);
        w->fn_current = 1;
      }
      memcpy(w->F[0], w->Fn, n * sizeof(double));
      continue;
    }
    cf[0] = 1.0;
    X[0]  = w->y;
    for (int j = 0; j < i; ++j)
    {
      cf[j + 1] = h * w->A[i * s + j];
      X[j + 1]  = w->F[j];
    }
    v_lincomb(n, i + 1, cf, X, w->sdata);
    if (aii == 0.0)
    {
      ark_rhs(w, ti, w->sdata, w->F[i]);
      continue;
    }
    int rc = ark_stage(w, i, ti, h * aii);
    if (rc) return rc;
  }
  return 0;
}

/* step loop: NORMAL until t >= tout, one step with o->onestep; steps clipped only at `clip` */
static int ark_steps(const orc_prob* p, const orc_ark_opts* o, orc_ark_state* st, double tout, double clip,
                     double* y)
{
  ark_ws W;
  memset(&W, 0, sizeof(W));
  W.p  = p;
  W.o  = o;
  W.st = st;
  W.n  = (long)p->nx * p->ny;
  int q;
  if (ark_table(o->implicit, o->order, &W.s, &q, &W.pe, W.A, W.b, W.d, W.c)) return -22;
  long n          = W.n;
  double** bufs[] = {&W.sdata, &W.z, &W.res, &W.del, &W.ewt, &W.tmp, &W.tmp2, &W.ynew};
  for (size_t k = 0; k < sizeof(bufs) / sizeof(bufs[0]); ++k) *bufs[k] = (double*)malloc(n * sizeof(double));
  for (int i = 0; i < W.s; ++i) W.F[i] = (double*)malloc(n * sizeof(double));
  W.y               = y;
  W.Fn              = st->Fn;
  const double ordv = (double)(W.pe + 1);
  if (!st->initialized)
  {
    st->hnext       = (o->hfixed > 0.0) ? o->hfixed : 0.0;
    st->initialized = 1;
  }
  W.fn_current     = st->fn_current;
  double target    = tout < clip ? tout : clip; /* initial-step distance */
  long nsteps_call = 0;
  int ret          = 0;
  while (st->t < clip && (o->onestep || st->t < tout))
  {
    if (nsteps_call >= (o->maxsteps > 0 ? o->maxsteps : 500))
    {
      ret = -1;
      break;
    }
    ark_ewt(&W);
    if (!(st->hnext > 0.0))
    {
      if (!W.fn_current)
      {
        ark_rhs(&W, st->t, W.y, W.Fn);
        W.fn_current = 1;
      }
      double tdist = target - st->t;
      double d0    = orc_wrms(W.y, W.ewt, n);
      double d1    = orc_wrms(W.Fn, W.ewt, n);
      double h0    = (d0 < 1.0e-5 || d1 < 1.0e-5) ? 1.0e-6 : 0.01 * (d0 / d1);
      if (h0 > tdist) h0 = tdist;
      v_linsum(n, h0, W.Fn, 1.0, W.y, W.tmp2);
      ark_rhs(&W, st->t + h0, W.tmp2, W.tmp);
      v_linsum(n, 1.0, W.tmp, -1.0, W.Fn, W.tmp);
      double d2 = orc_wrms(W.tmp, W.ewt, n) / h0;
      double dm = d1 > d2 ? d1 : d2;
      double h1 = (dm <= 1.0e-15) ? fmax(1.0e-6, h0 * 1.0e-3) : orc_pow(0.01 / dm, 1.0 / ordv);
      if (!(h1 > 0.0) || !(h1 < INFINITY)) h1 = h0;
      double hh = (100.0 * h0 < h1) ? 100.0 * h0 : h1;
      if (hh > tdist) hh = tdist;
      if (!(hh > 0.0))
      {
        ret = -3;
        goto out;
      }
      st->hnext = hh;
      st->h0    = hh;
    }
    int nef = 0, ncf = 0;
    for (;;)
    {
      double h    = st->hnext;
      int clipped = 0;
      if (st->t + h >= clip)
      {
        h       = clip - st->t;
        clipped = 1;
      }
      st->nst_att++;
      st->d.interp_ready = 0;
      int rc = ark_attempt(&W, h);
      if (rc == 1)
      {
        st->ncfn++;
        st->nnf++;
        if (o->hfixed > 0.0 || ++ncf > 10)
        {
          ret = -4;
          goto out;
        }
        st->hnext       = 0.25 * h;
        st->after_fail  = 1;
        st->force_setup = 1;
        continue;
      }
      double cf[6];
      const double* X[6];
      for (int i = 0; i < W.s; ++i)
      {
        cf[i] = h * (W.b[i] - W.d[i]);
        X[i]  = W.F[i];
      }
      v_lincomb(n, W.s, cf, X, W.tmp);
      double dsm = orc_wrms(W.tmp, W.ewt, n);
      if (o->hfixed > 0.0 || dsm <= 1.0)
      {
        cf[0] = 1.0;
        X[0]  = W.y;
        for (int i = 0; i < W.s; ++i)
        {
          cf[i + 1] = h * W.b[i];
          X[i + 1]  = W.F[i];
        }
        v_lincomb(n, W.s + 1, cf, X, W.ynew);
        memcpy(st->d.yold, W.y, n * sizeof(double));
        if (st->d.fold) memcpy(st->d.fold, W.F[0], n * sizeof(double)); /* f(t_n, y_n) of an ERK */
        memcpy(W.y, W.ynew, n * sizeof(double));
        st->d.interp_ready = 1;
        st->t        = clipped ? clip : st->t + h;
        W.fn_current = 0;
        double hprev = st->hlast;
        st->hlast    = h;
        if (o->hfixed > 0.0) st->hnext = o->hfixed;
        else
        {
          double hn  = controller_ord(o->controller, h, dsm, st->ep1, st->ep2, hprev, st->nhist, ordv);
          double eta = SAFETY * hn / h;
          double emx = (st->nst == 0) ? ETAMX1 : (st->after_fail ? 1.0 : GROWTH);
          if (eta > emx) eta = emx;
          if (eta >= LBOUND && eta <= UBOUND) eta = 1.0;
          st->hnext = h * eta;
          st->ep2   = st->ep1;
          st->ep1   = dsm;
          st->nhist++;
        }
        st->after_fail = 0;
        st->nst++;
        nsteps_call++;
        break;
      }
      st->netf++;
      nef++;
      if (!(dsm == dsm) || nef > 7)
      {
        ret = -3;
        goto out;
      }
      double hn  = controller_ord(o->controller, h, dsm, st->ep1, st->ep2, st->hlast, st->nhist, ordv);
      double eta = SAFETY * hn / h;
      if (eta > 1.0) eta = 1.0;
      if (nef >= SMALL_NEF && eta > ETAMXF) eta = ETAMXF;
      if (eta < ETAMIN) eta = ETAMIN;
      st->hnext      = h * eta;
      st->after_fail = 1;
    }
    if (o->onestep) break;
  }
out:
  st->fn_current = W.fn_current;
  if (W.mg) pfmg_destroy(W.mg);
  for (size_t k = 0; k < sizeof(bufs) / sizeof(bufs[0]); ++k) free(*bufs[k]);
  for (int i = 0; i < W.s; ++i) free(W.F[i]);
  return ret;
}

typedef struct {
  const orc_prob* p;
  const orc_ark_opts* o;
  orc_ark_state* st;
  long n;
} ark_fnew_ctx;

static int ark_fnew(void* ctx, const double** fnew)
{ /* f(t_n, y_n), evaluated (and counted) when no step start has; it then serves the next step */
  ark_fnew_ctx* c = (ark_fnew_ctx*)ctx;
  if (!c->st->fn_current)
  {
    orc_rhs(c->p, c->st->t, c->st->d.ycur, c->st->Fn);
    if (c->o->implicit) c->st->nfi++;
    else c->st->nfe++;
    c->st->fn_current = 1;
  }
  *fnew = c->st->Fn;
  return 0;
}

void orc_ark_state_free(orc_ark_state* st)
{
  free(st->Fn);
  free(st->d.ycur);
  free(st->d.yold);
  free(st->d.fold);
  st->Fn     = NULL;
  st->d.ycur = st->d.yold = st->d.fold = NULL;
}

int orc_arkstep_evolve(const orc_prob* p, const orc_ark_opts* o, orc_ark_state* st, double tout, double* y)
{
  long n = (long)p->nx * p->ny;
  int s, q, pe;
  double A[25], b[5], d[5], c[5];
  if (ark_table(o->implicit, o->order, &s, &q, &pe, A, b, d, c)) return -22;
  const int deg = q - 1 < 5 ? q - 1 : 5;
  if (!st->Fn) st->Fn = (double*)malloc(n * sizeof(double));
  dense_alloc(&st->d, n, deg == 3, y);
  ark_fnew_ctx fc = {p, o, st, n};
  int ret;
  if (dense_entry(&st->d, n, st->t, st->hlast, deg, ark_fnew, &fc, o->onestep, tout, y, &ret)) return ret;
  ret = ark_steps(p, o, st, tout, st->d.tstopset ? st->d.tstop : INFINITY, st->d.ycur);
  return dense_finish(&st->d, n, st->t, st->hlast, deg, ark_fnew, &fc, o->onestep, tout, y, ret);
}
