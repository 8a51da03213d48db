// diffusion_2D problem on the device: problem setup, RHS, Jacobian product, dominant
// eigenvalue (analytic and power iteration) and the Jacobi preconditioner.
//
// Layout: the N = nx*ny interior nodes are stored row-major, IDX(i,j,nx) = nx*j + i
// (diffusion_2D/diffusion_2D.hpp:55). Dirichlet kinds treat the (implicit) boundary ring as
// zero; the periodic kind wraps (diffusion_2D.cpp:247-249 periods={1,1}).
//
// Arithmetic contract: explicit __fma_rn where an FMA is wanted, everything else plain IEEE
// operations (the library is compiled with --fmad=false), in the order the CPU oracle uses.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdlib>
#include <vector>

#include "kernels.cuh"
#include "sts_internal.cuh"

static constexpr double PI_ = 3.14159265358979323846;

// ---------------------------------------------------------------------------------------
// host tables
// ---------------------------------------------------------------------------------------
extern "C" int STS_ManufacturedTables(sts_index n, double d, double* S, double* Sdd)
{
  for (long long i = 0; i < n; ++i)
  {
    double x = (i + 1) * d;
    double s = sin(PI_ * x);
    S[i]     = s * s;
    Sdd[i]   = 2.0 * PI_ * PI_ * cos(2.0 * PI_ * x);
  }
  return 0;
}

static double coeff_fn(double k, double x, int inhom) { return inhom ? (k * (1.0 + 0.99 * sin(x))) : k; }

extern "C" STS_Problem STS_ProblemCreate(STS_Context ctx, int kind, sts_index nx, sts_index ny,
                                         double kx, double ky, int inhomogeneous, double xl,
                                         double xu, double yl, double yu)
{
  if (!ctx || nx < 1 || ny < 1 || kind < 0 || kind > 2 || (kind == 2 && (nx < 2 || ny < 2)))
  {
    sts_set_error("STS_ProblemCreate: invalid arguments");
    return nullptr;
  }
  if ((long long)nx * ny >= (1LL << 31))
  {
    sts_set_error("STS_ProblemCreate: nx*ny must be < 2^31");
    return nullptr;
  }
  ctx_activate(ctx);
  STS_Problem p = new STS_Problem_();
  p->ctx        = ctx;
  p->kind       = kind;
  p->inhom      = (kind == STS_PROBLEM_PERIODIC) ? inhomogeneous : 0;
  p->nx         = nx;
  p->ny         = ny;
  p->kx         = kx;
  p->ky         = ky;
  if (kind == STS_PROBLEM_PERIODIC)
  { // diffusion_2D.cpp:155-160
    p->xl = xl;
    p->xu = xu;
    p->yl = yl;
    p->yu = yu;
    p->dx = (xu - xl) / (nx - 1);
    p->dy = (yu - yl) / (ny - 1);
  }
  else
  {
    p->dx = 1.0 / (nx + 1);
    p->dy = 1.0 / (ny + 1);
  }
  p->cx = kx / (p->dx * p->dx);
  p->cy = ky / (p->dy * p->dy);
  p->cc = -2.0 * (p->cx + p->cy);

  std::vector<double> tab(4 * (nx + ny));
  double* Sx  = tab.data();
  double* Sxx = Sx + nx;
  double* Sy  = Sxx + nx;
  double* Syy = Sy + ny;
  double* Dxw = Syy + ny;
  double* Dxe = Dxw + nx;
  double* Dys = Dxe + nx;
  double* Dyn = Dys + ny;
  STS_ManufacturedTables(nx, p->dx, Sx, Sxx);
  STS_ManufacturedTables(ny, p->dy, Sy, Syy);
  for (long long i = 0; i < nx; ++i)
  { // diffusion.cpp:43-46
    double xlo = p->xl + (i - 0.5) * p->dx, xhi = p->xl + (i + 0.5) * p->dx;
    Dxw[i]     = coeff_fn(kx, xlo, p->inhom) / (p->dx * p->dx);
    Dxe[i]     = coeff_fn(kx, xhi, p->inhom) / (p->dx * p->dx);
  }
  for (long long j = 0; j < ny; ++j)
  { // diffusion.cpp:36-39
    double ylo = p->yl + (j - 0.5) * p->dy, yhi = p->yl + (j + 0.5) * p->dy;
    Dys[j]     = coeff_fn(ky, ylo, p->inhom) / (p->dy * p->dy);
    Dyn[j]     = coeff_fn(ky, yhi, p->inhom) / (p->dy * p->dy);
  }
  std::vector<float> tabf(2 * (nx + ny));
  for (long long i = 0; i < 2 * (nx + ny); ++i) tabf[i] = (float)tab[i];
  if (!STS_CUDA_OK(cudaMalloc(&p->d_tab, tab.size() * sizeof(double))) ||
      !STS_CUDA_OK(cudaMalloc(&p->d_tabf, tabf.size() * sizeof(float))) ||
      !STS_CUDA_OK(cudaMemcpy(p->d_tab, tab.data(), tab.size() * sizeof(double), cudaMemcpyHostToDevice)) ||
      !STS_CUDA_OK(cudaMemcpy(p->d_tabf, tabf.data(), tabf.size() * sizeof(float), cudaMemcpyHostToDevice)))
  {
    STS_ProblemFree(&p);
    return nullptr;
  }
  ProbDev& d = p->dev;
  d.err      = ctx->d_err;
  d.nx       = nx;
  d.ny       = ny;
  d.kind     = kind;
  d.inhom    = p->inhom;
  d.kx       = kx;
  d.ky       = ky;
  d.cx       = p->cx;
  d.cy       = p->cy;
  d.cc       = p->cc;
  d.Sx       = p->d_tab;
  d.Sxx      = d.Sx + nx;
  d.Sy       = d.Sxx + nx;
  d.Syy      = d.Sy + ny;
  d.Dxw      = d.Syy + ny;
  d.Dxe      = d.Dxw + nx;
  d.Dys      = d.Dxe + nx;
  d.Dyn      = d.Dys + ny;
  d.Sxf      = p->d_tabf;
  d.Sxxf     = d.Sxf + nx;
  d.Syf      = d.Sxxf + nx;
  d.Syyf     = d.Syf + ny;
  return p;
}

extern "C" int STS_ProblemFree(STS_Problem* pp)
{
  if (!pp || !*pp) return 0;
  STS_Problem p = *pp;
  ctx_activate(p->ctx);
  cudaStreamSynchronize(p->ctx->stream);
  if (p->d_tab) cudaFree(p->d_tab);
  if (p->d_tabf) cudaFree(p->d_tabf);
  delete p;
  *pp = nullptr;
  return 0;
}

extern "C" int STS_ProblemGetInfo(STS_Problem p, double* dx, double* dy, double* cx, double* cy)
{
  if (!p) return -1;
  if (dx) *dx = p->dx;
  if (dy) *dy = p->dy;
  if (cx) *cx = p->cx;
  if (cy) *cy = p->cy;
  return 0;
}

static bool check_vec(STS_Problem p, N_Vector v, const char* who)
{
  if (!p || !v || NVL(v) != p->nx * p->ny)
  {
    sts_set_error("%s: vector length does not match the problem", who);
    return false;
  }
  return true;
}

// ---------------------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------------------
__global__ void initial_kernel(ProbDev P, double* u)
{
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long j = (long long)blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= P.nx || j >= P.ny) return;
  u[j * P.nx + i] = P.Sx[i] * P.Sy[j];
}

__global__ void exact_kernel(ProbDev P, double c, double* u)
{
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long j = (long long)blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= P.nx || j >= P.ny) return;
  u[j * P.nx + i] = (P.Sx[i] * P.Sy[j]) * c;
}

static dim3 grid2d(long long nx, long long ny, dim3 b)
{
  return dim3((unsigned)((nx + b.x - 1) / b.x), (unsigned)((ny + b.y - 1) / b.y));
}

// Initial conditions are tabulated on the host with the C math library (once per run), so
// the device state starts from the same bits as the CPU oracle.
static int upload(STS_Problem p, N_Vector u, const std::vector<double>& h)
{
  if (!STS_CUDA_OK(cudaMemcpyAsync(NVD(u), h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice,
                                   p->ctx->stream)))
    return -1;
  N_VSetShape_Sts(u, p->nx, p->ny);
  return STS_CUDA_OK(cudaStreamSynchronize(p->ctx->stream)) ? 0 : -1;
}

extern "C" int STS_Initial(double t, N_Vector u, STS_Problem p)
{
  (void)t;
  if (!check_vec(p, u, "STS_Initial")) return -1;
  ctx_activate(p->ctx);
  if (p->kind != STS_PROBLEM_PERIODIC)
  {
    dim3 b(64, 4);
    initial_kernel<<<grid2d(p->nx, p->ny, b), b, 0, p->ctx->stream>>>(p->dev, NVD(u));
    N_VSetShape_Sts(u, p->nx, p->ny);
    return STS_CUDA_OK(cudaGetLastError()) ? 0 : -1;
  }
  std::vector<double> h(p->nx * p->ny);
  for (long long j = 0; j < p->ny; ++j)
    for (long long i = 0; i < p->nx; ++i)
    { // initial.cpp:39-43
      const double x       = p->xl + i * p->dx;
      const double y       = p->yl + j * p->dy;
      h[j * p->nx + i] = (1.0 + 0.3 * sin(2.0 * x)) / sqrt(5.5 * PI_) * exp(-(y * y) / 5.5);
    }
  return upload(p, u, h);
}

extern "C" int STS_Exact(double t, N_Vector u, STS_Problem p)
{
  if (!check_vec(p, u, "STS_Exact")) return -1;
  if (p->kind != STS_PROBLEM_MANUFACTURED)
  {
    sts_set_error("STS_Exact: only the manufactured problem has an exact solution");
    return -1;
  }
  ctx_activate(p->ctx);
  dim3 b(64, 4);
  exact_kernel<<<grid2d(p->nx, p->ny, b), b, 0, p->ctx->stream>>>(p->dev, sts_c(t), NVD(u));
  return STS_CUDA_OK(cudaGetLastError()) ? 0 : -1;
}

extern "C" int STS_InitialModes(N_Vector u, STS_Problem p, int nmodes, const int* pm, const int* qm,
                                const double* amp)
{
  if (!check_vec(p, u, "STS_InitialModes") || nmodes < 0) return -1;
  ctx_activate(p->ctx);
  std::vector<double> h(p->nx * p->ny);
  for (long long j = 0; j < p->ny; ++j)
    for (long long i = 0; i < p->nx; ++i)
    {
      const double x = (i + 1) * p->dx, y = (j + 1) * p->dy;
      double v       = 0.0;
      for (int k = 0; k < nmodes; ++k) v += amp[k] * sin(pm[k] * PI_ * x) * sin(qm[k] * PI_ * y);
      h[j * p->nx + i] = v;
    }
  return upload(p, u, h);
}

// RHS, one point per thread. FORCED adds the manufactured forcing Sy_j P_i + Syy_j Q_i with
// P_i = al Sx_i + be Sxx_i, Q_i = ga Sx_i (al = c'(t), be = -c(t) kx, ga = -c(t) ky).
template <bool FORCED>
__global__ void __launch_bounds__(256) rhs_kernel(ProbDev P, double al, double be, double ga,
                                                  const double* __restrict__ u, double* __restrict__ f)
{
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long j = (long long)blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= P.nx || j >= P.ny) return;
  const long long k = j * P.nx + i;
  double acc;
  if (P.kind == STS_PROBLEM_PERIODIC)
  {
    acc = periodic_point(P, u, i, j);
  }
  else
  {
    acc = dirichlet_point(P, u, i, j);
    if (FORCED) acc = add_forcing(P, al, be, ga, i, j, acc);
  }
  f[k] = acc;
}

int sts_rhs_launch(STS_Problem p, double t, const double* u, double* f, bool forcing, cudaStream_t s)
{
  dim3 b(64, 4);
  dim3 g = grid2d(p->nx, p->ny, b);
  if (forcing && p->kind == STS_PROBLEM_MANUFACTURED)
  {
    double c = sts_c(t), cd = sts_cdot(t);
    double al = 1.0 * cd, be = -(1.0 * c) * p->kx, ga = -(1.0 * c) * p->ky;
    rhs_kernel<true><<<g, b, 0, s>>>(p->dev, al, be, ga, u, f);
  }
  else rhs_kernel<false><<<g, b, 0, s>>>(p->dev, 0.0, 0.0, 0.0, u, f);
  return STS_CUDA_OK(cudaGetLastError()) ? 0 : -1;
}

extern "C" int STS_Diffusion(double t, N_Vector u, N_Vector f, void* user_data)
{
  STS_MARK_FUNCTION;
  STS_Problem p = (STS_Problem)user_data;
  if (!check_vec(p, u, "STS_Diffusion") || !check_vec(p, f, "STS_Diffusion")) return -1;
  ctx_activate(p->ctx);
  return sts_rhs_launch(p, t, NVD(u), NVD(f), true, p->ctx->stream);
}

extern "C" int STS_JacTimes(N_Vector v, N_Vector Jv, double t, N_Vector y, N_Vector fy, void* user_data,
                            N_Vector tmp)
{
  (void)t;
  (void)y;
  (void)fy;
  (void)tmp;
  STS_Problem p = (STS_Problem)user_data;
  if (!check_vec(p, v, "STS_JacTimes") || !check_vec(p, Jv, "STS_JacTimes")) return -1;
  ctx_activate(p->ctx);
  return sts_rhs_launch(p, 0.0, NVD(v), NVD(Jv), false, p->ctx->stream);
}

// dom_eig (diffusion_2D/main.cpp:536-550)
extern "C" int STS_DomEig(double t, N_Vector y, N_Vector fn, double* lambdaR, double* lambdaI,
                          void* user_data, N_Vector temp1, N_Vector temp2, N_Vector temp3)
{
  (void)t;
  (void)y;
  (void)fn;
  (void)temp1;
  (void)temp2;
  (void)temp3;
  STS_Problem p = (STS_Problem)user_data;
  if (!p) return -1;
  double a = p->kx / p->dx / p->dx, b = p->ky / p->dy / p->dy;
  *lambdaR = -8.0 * (a > b ? a : b);
  *lambdaI = 0.0;
  return 0;
}

// SUNDomEigEstimator_Power (main.cpp:344): v <- v/||v||; repeat w = A v, lambda = v.w,
// v <- w/||w|| until |lambda - lambda_old| < reltol |lambda|. Same order as the oracle.
extern "C" int STS_PowerIteration(STS_Problem p, N_Vector v, int maxiters, double reltol, double* lambda,
                                  int* iters)
{
  if (!check_vec(p, v, "STS_PowerIteration")) return -1;
  STS_Context ctx = p->ctx;
  ctx_activate(ctx);
  long long n = NVL(v);
  double* w   = nullptr;
  if (!STS_CUDA_OK(cudaMallocAsync(&w, n * sizeof(double), ctx->stream))) return -1;
  double* vd = NVD(v);
  double nrm = sqrt(sts_dot_exact(ctx, vd, vd, n, SLOT_NRM));
  if (!(nrm > 0.0))
  {
    N_VConst_Sts(1.0, v);
    nrm = sqrt(sts_dot_exact(ctx, vd, vd, n, SLOT_NRM));
  }
  N_VScale_Sts(1.0 / nrm, v, v);
  double lam = 0.0, lam_old = 0.0;
  int k;
  for (k = 1; k <= maxiters; ++k)
  {
    sts_rhs_launch(p, 0.0, vd, w, false, ctx->stream);
    lam       = sts_dot_exact(ctx, vd, w, n, SLOT_LAM);
    double wn = sqrt(sts_dot_exact(ctx, w, w, n, SLOT_NRM));
    double wi = 1.0 / wn;
    N_Vector wv = N_VMake_Sts(n, w, ctx);
    N_VScale_Sts(wi, wv, v);
    N_VDestroy_Sts(wv);
    if (k > 1 && fabs(lam - lam_old) < reltol * fabs(lam)) break;
    lam_old = lam;
  }
  if (k > maxiters) k = maxiters;
  cudaFreeAsync(w, ctx->stream);
  if (!STS_CUDA_OK(cudaStreamSynchronize(ctx->stream))) return -1;
  *lambda = lam;
  if (iters) *iters = k;
  return 0;
}

// Jacobi preconditioner (preconditioner_jacobi.cpp:9-61): PSetup stores
// D = 1/(1 - gamma*diag) with diag = -((Dxw+Dxe)+(Dys+Dyn)); PSolve z = D r.
__global__ void jacobi_kernel(ProbDev P, double gamma, const double* __restrict__ r, double* __restrict__ z)
{
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long j = (long long)blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= P.nx || j >= P.ny) return;
  double diag;
  if (P.kind == STS_PROBLEM_PERIODIC) diag = -((P.Dxw[i] + P.Dxe[i]) + (P.Dys[j] + P.Dyn[j]));
  else diag = P.cc;
  double D              = 1.0 / (1.0 - gamma * diag);
  z[j * P.nx + i]       = D * r[j * P.nx + i];
}

extern "C" int STS_PSetup(double t, N_Vector u, N_Vector f, int jok, int* jcurPtr, double gamma,
                          void* user_data)
{
  STS_MARK_FUNCTION;
  (void)t;
  (void)u;
  (void)f;
  (void)jok;
  STS_Problem p = (STS_Problem)user_data;
  if (!p) return -1;
  p->jacobi_scale = 1.0 / (1.0 - gamma * p->cc);
  if (jcurPtr) *jcurPtr = 1;
  return 0;
}

extern "C" int STS_PSolve(double t, N_Vector u, N_Vector f, N_Vector r, N_Vector z, double gamma,
                          double delta, int lr, void* user_data)
{
  STS_MARK_FUNCTION;
  (void)t;
  (void)u;
  (void)f;
  (void)delta;
  (void)lr;
  STS_Problem p = (STS_Problem)user_data;
  if (!check_vec(p, r, "STS_PSolve") || !check_vec(p, z, "STS_PSolve")) return -1;
  ctx_activate(p->ctx);
  dim3 b(64, 4);
  jacobi_kernel<<<grid2d(p->nx, p->ny, b), b, 0, p->ctx->stream>>>(p->dev, gamma, NVD(r), NVD(z));
  return STS_CUDA_OK(cudaGetLastError()) ? 0 : -1;
}
