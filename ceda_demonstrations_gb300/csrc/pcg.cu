// Implicit comparator: preconditioned CG on (I - gamma A) x = b with the Jacobi
// preconditioner of diffusion_2D/preconditioner_jacobi.cpp (SUNLinSol_PCG + PSetup/PSolve,
// diffusion_2D/main.cpp:207-231,305-316), plus a fixed-step SDIRK2 driver (ARKStep DIRK).
//
// Fused path: the CG scalars (rz, p.q, alpha, beta, ||r||^2, convergence flag, iteration
// count) live in device memory and are produced by the last block of each reduction, so an
// iteration needs no host round trip. Iterations are issued in batches captured in a CUDA
// graph; kernels return immediately once the device-side flag says the solve has stopped,
// and the host reads the flag between batches. Per iteration:
//   KP: p = beta p + D r                                   (24 B/DOF, 2 FP64)
//   KQ: q = (I - gamma A) p, p.q -> alpha = rz / p.q        (16 B/DOF + halo, 6 FP64)
//   KX: x += alpha p, r -= alpha q, r.r -> beta             (48 B/DOF, 3 FP64)
// The Jacobi scaling D is one constant for these constant-coefficient problems, so
// r.z = r.(D r) is taken as D (r.r): one exact sum per iteration. GB300 issues FP64 at a
// small fraction of its FP32 rate (about 5e11 FP64 instructions/s measured), so these 11 FP64
// instructions per point, not the 88 bytes, bound an iteration; the elementwise kernels
// keep four independent points in flight per thread to hide the memory latency.
// All dot products use the exact accumulator, so the iterates match the CPU oracle bit
// for bit and do not depend on the launch shape.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <functional>
#include <vector>

#include "kernels.cuh"
#include "krylov.cuh"
#include "sts_internal.cuh"

struct PcgScal {
  double rz, pq, alpha, beta, rr, D, gamma, tolb;
  int iters, maxit, state; // state: 0 running, 1 converged, 2 iteration limit, 3 breakdown
  int pad_;
  unsigned long long limbs[2][xsum::NL];
  unsigned int flags[2];
  unsigned int ticket, pad2_;
};

struct PcgOut {
  int state, iters;
  double rr;
};

struct PcgWork {
  STS_Context ctx = nullptr;
  long long n     = 0;
  double *p[2]    = {nullptr, nullptr};
  double* q       = nullptr;
  double* r       = nullptr;
  PcgScal* d_s    = nullptr; // device
  PcgOut* h_out   = nullptr; // pinned, mapped: state / iteration count / ||r||^2 after each KX
  PcgOut* d_out   = nullptr;
  cudaGraphExec_t graph[2] = {nullptr, nullptr};
  long long gn = 0;
};

static constexpr int PCG_BATCH = 8; // iterations per graph launch (even: p ping-pong)

// reduction kernels: two grid-strided points per thread and trip (independent loads in
// flight) on one wave of resident blocks, so each block pays the exact-sum combine once
// (a 2048^2 sweep of unroll depth and grid on GB300: 45 us against 59 us for four points
// on eight blocks per SM)
constexpr int PCG_U = 2;

// one wave of resident blocks of a 256-thread reduction kernel, at most one trip's worth
template <typename K>
static int resident_blocks(STS_Context ctx, K kernel, long long n, int per_thread)
{
  int occ = 0;
  if (!STS_CUDA_OK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, 256, 0)) || occ < 1) occ = 1;
  long long b         = (long long)ctx->num_sms * occ;
  const long long cap = (n + 256LL * per_thread - 1) / (256LL * per_thread);
  if (b > cap) b = cap;
  return b < 1 ? 1 : (int)b;
}

// initial scalars: rr = b.b, rz = D rr (r = b)
__global__ void __launch_bounds__(256) pcg_init_kernel(long long n, const double* __restrict__ b,
                                                       PcgScal* s)
{
  xsum::Limbs a[1];
  unsigned fl[1] = {0};
  xsum::zero(a[0]);
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += stride)
  {
    const double r = b[k];
    xsum::add(a[0], r * r, fl[0]);
  }
  krylov_block_finish<256, 1>(a, fl, s, [&](const double* v) {
    s->rr   = v[0];
    s->rz   = s->D * v[0];
    s->beta = 0.0;
  });
}

__global__ void __launch_bounds__(256) pcg_p_kernel(long long n, const double* __restrict__ r,
                                                    const double* __restrict__ pold,
                                                    double* __restrict__ pnew, const PcgScal* __restrict__ s)
{
  if (s->state != 0) return;
  const double beta = s->beta, D = s->D;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += stride)
    pnew[k] = __fma_rn(beta, pold[k], D * r[k]);
}

// q = (I - gamma A) p (Dirichlet operator) with the coefficients folded,
// q = c0 p_C + c1 (p_W + p_E) + c2 (p_S + p_N); accumulate p.q; alpha = rz / p.q
__global__ void __launch_bounds__(256) pcg_q_kernel(ProbDev P, const double* __restrict__ p,
                                                    double* __restrict__ q, PcgScal* s)
{
  if (s->state != 0) return;
  const double gamma = s->gamma;
  const double c0 = 1.0 - gamma * P.cc, c1 = -gamma * P.cx, c2 = -gamma * P.cy;
  xsum::Limbs a[1];
  unsigned fl[1] = {0};
  xsum::zero(a[0]);
  const long long nx = P.nx, ny = P.ny;
  const long long i  = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nx)
    for (long long j = blockIdx.y; j < ny; j += gridDim.y)
    {
      const long long k = j * nx + i;
      const double pc   = p[k];
      const double pw   = (i > 0) ? p[k - 1] : 0.0;
      const double pe   = (i < nx - 1) ? p[k + 1] : 0.0;
      const double ps   = (j > 0) ? p[k - nx] : 0.0;
      const double pn   = (j < ny - 1) ? p[k + nx] : 0.0;
      const double sx = pw + pe, sy = ps + pn;
      const double qk = __fma_rn(c1, sx, __fma_rn(c2, sy, c0 * pc));
      q[k]            = qk;
      xsum::add(a[0], pc * qk, fl[0]);
    }
  krylov_block_finish<256, 1>(a, fl, s, [&](const double* v) {
    s->pq    = v[0];
    s->alpha = s->rz / v[0];
  });
}

__global__ void __launch_bounds__(256) pcg_x_kernel(long long n, const double* __restrict__ p,
                                                    const double* __restrict__ q, double* __restrict__ x,
                                                    double* __restrict__ r, PcgScal* s, PcgOut* out)
{
  if (s->state != 0) return;
  const double alpha = s->alpha;
  xsum::Limbs a[1];
  unsigned fl[1] = {0};
  xsum::zero(a[0]);
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long k0 = (long long)blockIdx.x * blockDim.x + threadIdx.x; k0 < n; k0 += PCG_U * stride)
  {
    double pv[PCG_U], qv[PCG_U], xv[PCG_U], rv[PCG_U];
#pragma unroll
    for (int u = 0; u < PCG_U; ++u)
    {
      const long long k = k0 + u * stride;
      const bool in     = k < n;
      pv[u]             = in ? p[k] : 0.0;
      qv[u]             = in ? q[k] : 0.0;
      xv[u]             = in ? x[k] : 0.0;
      rv[u]             = in ? r[k] : 0.0;
    }
#pragma unroll
    for (int u = 0; u < PCG_U; ++u)
    {
      const long long k = k0 + u * stride;
      if (k < n)
      {
        x[k]            = __fma_rn(alpha, pv[u], xv[u]);
        const double rk = __fma_rn(-alpha, qv[u], rv[u]);
        r[k]            = rk;
        xsum::add(a[0], rk * rk, fl[0]);
      }
    }
  }
  krylov_block_finish<256, 1>(a, fl, s, [&](const double* v) {
    s->rr = v[0];
    s->iters += 1;
    if (sqrt(v[0]) <= s->tolb) s->state = 1;
    else if (s->iters >= s->maxit) s->state = 2;
    else if (!(v[0] == v[0])) s->state = 3;
    else
    {
      const double rzn = s->D * v[0];
      s->beta          = rzn / s->rz;
      s->rz            = rzn;
    }
    out->state = s->state;
    out->iters = s->iters;
    out->rr    = v[0];
  });
}

static void pcg_free(PcgWork* w)
{
  for (int k = 0; k < 2; ++k)
  {
    if (w->graph[k]) cudaGraphExecDestroy(w->graph[k]);
    cudaFree(w->p[k]);
  }
  cudaFree(w->q);
  cudaFree(w->r);
  cudaFree(w->d_s);
  cudaFreeHost(w->h_out);
  delete w;
}

static PcgWork* pcg_alloc(STS_Context ctx, long long n)
{
  PcgWork* w = new PcgWork();
  w->ctx     = ctx;
  w->n       = n;
  bool ok    = STS_CUDA_OK(cudaMalloc(&w->p[0], n * sizeof(double))) &&
            STS_CUDA_OK(cudaMalloc(&w->p[1], n * sizeof(double))) &&
            STS_CUDA_OK(cudaMalloc(&w->q, n * sizeof(double))) && STS_CUDA_OK(cudaMalloc(&w->r, n * sizeof(double))) &&
            STS_CUDA_OK(cudaMalloc(&w->d_s, sizeof(PcgScal))) &&
            STS_CUDA_OK(cudaHostAlloc(&w->h_out, sizeof(PcgOut), cudaHostAllocMapped)) &&
            STS_CUDA_OK(cudaHostGetDevicePointer(&w->d_out, w->h_out, 0));
  if (!ok)
  {
    pcg_free(w);
    return nullptr;
  }
  return w;
}

// one PCG iteration pair (p ping-pong makes a batch of PCG_BATCH iterations self-similar)
static void pcg_record_batch(PcgWork* w, STS_Problem p, double* x)
{
  cudaStream_t st = w->ctx->stream;
  const long long n = w->n;
  const int eb      = ew_blocks(w->ctx, n, 256 * 2);
  const int ex      = resident_blocks(w->ctx, pcg_x_kernel, n, PCG_U);
  dim3 bq(256, 1);
  unsigned gx = (unsigned)((p->nx + 255) / 256);
  int occ_q   = 0;
  if (!STS_CUDA_OK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_q, pcg_q_kernel, 256, 0)) || occ_q < 1)
    occ_q = 1;
  long long gy_cap = (long long)w->ctx->num_sms * occ_q / gx; // one wave of resident blocks
  if (gy_cap < 1) gy_cap = 1;
  dim3 gq(gx, (unsigned)(p->ny < gy_cap ? p->ny : gy_cap));
  for (int it = 0; it < PCG_BATCH; ++it)
  {
    const double* pold = w->p[it & 1];
    double* pnew       = w->p[(it + 1) & 1];
    pcg_p_kernel<<<eb, 256, 0, st>>>(n, w->r, pold, pnew, w->d_s);
    pcg_q_kernel<<<gq, bq, 0, st>>>(p->dev, pnew, w->q, w->d_s);
    pcg_x_kernel<<<ex, 256, 0, st>>>(n, pnew, w->q, x, w->r, w->d_s, w->d_out);
  }
}

// Fused PCG solve; `batch_cb` (optional) is called after every graph batch of PCG_BATCH
// iterations with the device pointers of the current iterate and residual.
int sts_pcg_run(STS_Problem p, double gamma, N_Vector b, N_Vector x, double tol, int maxit, int jacobi, int* iters,
                double* relres, const std::function<void(int, const double*, const double*)>& batch_cb)
{
  if (!p || !b || !x || NVL(b) != p->nx * p->ny || NVL(x) != NVL(b) || maxit < 1)
  {
    sts_set_error("STS_ImplicitSolvePCG: invalid arguments");
    return -1;
  }
  if (p->kind == STS_PROBLEM_PERIODIC)
  {
    sts_set_error("STS_ImplicitSolvePCG: the fused solver covers the Dirichlet problems");
    return -1;
  }
  STS_Context ctx = p->ctx;
  ctx_activate(ctx);
  cudaStream_t st   = ctx->stream;
  const long long n = NVL(b);
  PcgWork* w        = pcg_alloc(ctx, n);
  if (!w) return -1;
  int ret = 0;
  // x = 0, r = b, p = 0
  cudaMemsetAsync(NVD(x), 0, n * sizeof(double), st);
  cudaMemcpyAsync(w->r, NVD(b), n * sizeof(double), cudaMemcpyDeviceToDevice, st);
  cudaMemsetAsync(w->p[0], 0, n * sizeof(double), st);
  PcgScal hs;
  memset(&hs, 0, sizeof(hs));
  hs.D     = jacobi ? 1.0 / (1.0 - gamma * p->cc) : 1.0;
  hs.gamma = gamma;
  hs.maxit = maxit;
  const double bnorm = sqrt(sts_dot_exact(ctx, NVD(b), NVD(b), n, SLOT_PCG0));
  if (!(bnorm > 0.0))
  {
    if (iters) *iters = 0;
    if (relres) *relres = 0.0;
    pcg_free(w);
    return 0;
  }
  hs.tolb = tol * bnorm;
  memset(w->h_out, 0, sizeof(PcgOut));
  cudaMemcpyAsync(w->d_s, &hs, sizeof(PcgScal), cudaMemcpyHostToDevice, st);
  pcg_init_kernel<<<ew_blocks(ctx, n, 256 * 2), 256, 0, st>>>(n, NVD(b), w->d_s);
  // the graph is recorded for this x buffer
  cudaGraph_t g;
  if (!STS_CUDA_OK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal)))
  {
    pcg_free(w);
    return -1;
  }
  pcg_record_batch(w, p, NVD(x));
  if (!STS_CUDA_OK(cudaStreamEndCapture(st, &g)) || !STS_CUDA_OK(cudaGraphInstantiate(&w->graph[0], g, 0)))
  {
    pcg_free(w);
    return -1;
  }
  cudaGraphDestroy(g);
  // the device sets state 2 at maxit; the host bound on launches is a second guard
  for (long long launches = 0;; ++launches)
  {
    if (launches > maxit / PCG_BATCH + 2)
    {
      sts_set_error("STS_ImplicitSolvePCG: the device-side stop flag was not set");
      ret = -1;
      break;
    }
    if (!STS_CUDA_OK(cudaGraphLaunch(w->graph[0], st)) || !STS_CUDA_OK(cudaStreamSynchronize(st)))
    {
      ret = -1;
      break;
    }
    if (batch_cb) batch_cb(((volatile PcgOut*)w->h_out)->iters, NVD(x), w->r);
    if (((volatile PcgOut*)w->h_out)->state != 0) break;
  }
  const int state = w->h_out->state;
  if (iters) *iters = w->h_out->iters;
  if (relres) *relres = sqrt(w->h_out->rr) / bnorm;
  if (ret == 0 && state == 3) ret = -3;
  if (ret == 0 && state == 2) ret = 1; // iteration limit: recoverable
  pcg_free(w);
  return ret;
}

extern "C" int STS_ImplicitSolvePCG(STS_Problem p, double gamma, N_Vector b, N_Vector x, double tol, int maxit,
                                    int jacobi, int* iters, double* relres)
{
  STS_MARK_FUNCTION;
  return sts_pcg_run(p, gamma, b, x, tol, maxit, jacobi, iters, relres, nullptr);
}

// ---------------------------------------------------------------------------------------
// Generic Krylov solvers through ATimes / PSolve callbacks: SUNLinSol_PCG and SUNLinSol_SPGMR
// (diffusion_2D/main.cpp:209-218), and SUNLinSol_SPFGMR, the flexible GMRES SUNDIALS offers for
// preconditioners that change from one application to the next. One object type; the solve
// dispatches on the kind.
// ---------------------------------------------------------------------------------------
enum { LS_PCG = 0, LS_SPGMR = 1, LS_SPFGMR = 2 };

struct LinSol {
  int kind          = LS_PCG;
  STS_Context ctx   = nullptr;
  int pretype       = STS_PREC_NONE;
  int maxl          = 5;
  void* A_data      = nullptr;
  STS_ATimesFn atimes = nullptr;
  void* P_data      = nullptr;
  STS_PSolveFn psolve = nullptr;
  N_Vector r = nullptr, pv = nullptr, z = nullptr, Ap = nullptr;
  // SPGMR: Krylov basis V[0..maxl], restarts, Gram-Schmidt variant, Hessenberg + Givens;
  // SPFGMR also keeps the preconditioned basis Z[0..maxl-1]
  std::vector<N_Vector> V, Z;
  int max_restarts  = 0;
  int gstype        = STS_MODIFIED_GS;
  int last_iters    = 0;
  double last_res   = 0.0;
};

static LinSol* linsol_new(int kind, N_Vector y, int pretype, int maxl, STS_Context ctx)
{
  if (!y || !ctx)
  {
    sts_set_error("SUNLinSol: NULL argument");
    return nullptr;
  }
  LinSol* L  = new LinSol();
  L->kind    = kind;
  L->ctx     = ctx;
  L->pretype = pretype;
  L->maxl    = maxl > 0 ? maxl : 5;
  L->r       = N_VClone_Sts(y);
  L->z       = N_VClone_Sts(y);
  L->Ap      = N_VClone_Sts(y);
  if (kind == LS_PCG) L->pv = N_VClone_Sts(y);
  else
    for (int k = 0; k <= L->maxl; ++k) L->V.push_back(N_VClone_Sts(y));
  if (kind == LS_SPFGMR)
    for (int k = 0; k < L->maxl; ++k) L->Z.push_back(N_VClone_Sts(y));
  return L;
}

extern "C" void* STS_SUNLinSol_PCG(N_Vector y, int pretype, int maxl, STS_Context ctx)
{
  return linsol_new(LS_PCG, y, pretype, maxl, ctx);
}

extern "C" void* STS_SUNLinSol_SPGMR(N_Vector y, int pretype, int maxl, STS_Context ctx)
{
  if (maxl > 1000)
  {
    sts_set_error("SUNLinSol_SPGMR: maxl %d > 1000", maxl);
    return nullptr;
  }
  return linsol_new(LS_SPGMR, y, pretype, maxl, ctx);
}

// SUNLinSol_SPFGMR: right preconditioning only (a left type is taken as right, as SUNDIALS does)
extern "C" void* STS_SUNLinSol_SPFGMR(N_Vector y, int pretype, int maxl, STS_Context ctx)
{
  if (maxl > 1000)
  {
    sts_set_error("SUNLinSol_SPFGMR: maxl %d > 1000", maxl);
    return nullptr;
  }
  return linsol_new(LS_SPFGMR, y, pretype == STS_PREC_NONE ? STS_PREC_NONE : STS_PREC_RIGHT, maxl, ctx);
}

extern "C" int STS_SUNLinSol_SPGMRSetMaxRestarts(void* LS, int maxrs)
{
  LinSol* L = (LinSol*)LS;
  if (!L || L->kind == LS_PCG || maxrs < 0) return -1;
  L->max_restarts = maxrs;
  return 0;
}

extern "C" int STS_SUNLinSol_SPGMRSetGSType(void* LS, int gstype)
{
  LinSol* L = (LinSol*)LS;
  if (!L || L->kind == LS_PCG || (gstype != STS_MODIFIED_GS && gstype != STS_CLASSICAL_GS)) return -1;
  L->gstype = gstype;
  return 0;
}

extern "C" int STS_SUNLinSol_SPFGMRSetMaxRestarts(void* LS, int maxrs)
{
  LinSol* L = (LinSol*)LS;
  return (L && L->kind == LS_SPFGMR) ? STS_SUNLinSol_SPGMRSetMaxRestarts(LS, maxrs) : -1;
}

extern "C" int STS_SUNLinSol_SPFGMRSetGSType(void* LS, int gstype)
{
  LinSol* L = (LinSol*)LS;
  return (L && L->kind == LS_SPFGMR) ? STS_SUNLinSol_SPGMRSetGSType(LS, gstype) : -1;
}

extern "C" int STS_SUNLinSolSetATimes(void* LS, void* A_data, STS_ATimesFn atimes)
{
  if (!LS) return -1;
  ((LinSol*)LS)->A_data = A_data;
  ((LinSol*)LS)->atimes = atimes;
  return 0;
}

extern "C" int STS_SUNLinSolSetPreconditioner(void* LS, void* P_data, STS_PSolveFn psolve)
{
  if (!LS) return -1;
  ((LinSol*)LS)->P_data = P_data;
  ((LinSol*)LS)->psolve = psolve;
  return 0;
}

// standard PCG, x0 = 0, stop when ||r||_2 <= delta ||b||_2
static int pcg_solve(LinSol* L, N_Vector x, N_Vector b, double delta)
{
  const bool prec = L->pretype != STS_PREC_NONE && L->psolve;
  N_VConst_Sts(0.0, x);
  N_VLinearSum_Sts(1.0, b, 0.0, b, L->r);
  const double bnorm = sqrt(N_VDotProd_Sts(b, b));
  if (!(bnorm > 0.0)) return 0;
  if (prec)
  {
    if (L->psolve(L->P_data, L->r, L->z, delta, L->pretype)) return 1;
  }
  else N_VLinearSum_Sts(1.0, L->r, 0.0, L->r, L->z);
  double rz = N_VDotProd_Sts(L->r, L->z);
  N_VLinearSum_Sts(1.0, L->z, 0.0, L->z, L->pv);
  for (int it = 1; it <= L->maxl; ++it)
  {
    if (L->atimes(L->A_data, L->pv, L->Ap)) return 1;
    const double pq    = N_VDotProd_Sts(L->pv, L->Ap);
    const double alpha = rz / pq;
    N_VLinearSum_Sts(alpha, L->pv, 1.0, x, x);
    N_VLinearSum_Sts(-alpha, L->Ap, 1.0, L->r, L->r);
    const double rr = N_VDotProd_Sts(L->r, L->r);
    L->last_iters   = it;
    L->last_res     = sqrt(rr) / bnorm;
    if (sqrt(rr) <= delta * bnorm) return 0;
    if (prec)
    {
      if (L->psolve(L->P_data, L->r, L->z, delta, L->pretype)) return 1;
    }
    else N_VLinearSum_Sts(1.0, L->r, 0.0, L->r, L->z);
    const double rzn = N_VDotProd_Sts(L->r, L->z);
    const double beta = rzn / rz;
    rz                = rzn;
    N_VLinearSum_Sts(1.0, L->z, beta, L->pv, L->pv);
  }
  return 1; // SUNLS_CONV_FAIL (recoverable)
}

// Givens rotation (c, s) with [c s; -s c] [a; b] = [r; 0], scaled to avoid overflow
static void givens(double a, double b, double* c, double* s)
{
  if (b == 0.0)
  {
    *c = 1.0;
    *s = 0.0;
  }
  else if (fabs(b) > fabs(a))
  {
    const double t = a / b;
    *s             = 1.0 / sqrt(1.0 + t * t);
    *c             = *s * t;
  }
  else
  {
    const double t = b / a;
    *c             = 1.0 / sqrt(1.0 + t * t);
    *s             = *c * t;
  }
}

// Restarted GMRES(maxl) with right preconditioning (Saad & Schultz 1986), x0 = 0: minimise
// ||b - A P^-1 u|| over the Krylov space of the current residual, x += P^-1 u at the end of
// each cycle; Arnoldi by modified Gram-Schmidt (one exact dot and one LinearSum per basis
// vector) or classical Gram-Schmidt with one re-orthogonalisation pass (two N_VDotProdMulti +
// N_VLinearCombination); the Hessenberg matrix is reduced by Givens rotations on the host, so
// the residual estimate |g_{j+1}| is known after every iteration. Stop when it is at most
// delta ||b||_2; after max_restarts restarts without convergence return 1 (recoverable).
// Flexible variant (SPFGMR, Saad 1993): the preconditioned vectors z_j = P_j^-1 v_j are kept,
// w = A z_j, and the cycle ends with x += Z y, so P may differ between applications.
static int spgmr_solve(LinSol* L, N_Vector x, N_Vector b, double delta)
{
  const bool prec = L->pretype != STS_PREC_NONE && L->psolve;
  const bool flex = L->kind == LS_SPFGMR && prec;
  const int m     = L->maxl;
  std::vector<double> H((size_t)(m + 1) * m, 0.0), cs(m), sn(m), g(m + 1), y(m), h(m + 1), h2(m + 1);
  std::vector<double> cf(m + 2);
  std::vector<N_Vector> X(m + 2);
  auto Hij = [&](int i, int j) -> double& { return H[(size_t)i * m + j]; };
  N_VConst_Sts(0.0, x);
  N_VLinearSum_Sts(1.0, b, 0.0, b, L->r);
  const double bnorm = sqrt(N_VDotProd_Sts(b, b));
  if (!(bnorm > 0.0)) return 0;
  double beta = bnorm;
  for (int cycle = 0; cycle <= L->max_restarts; ++cycle)
  {
    N_VScale_Sts(1.0 / beta, L->r, L->V[0]);
    for (int k = 0; k <= m; ++k) g[k] = 0.0;
    g[0]          = beta;
    int k         = 0; // columns built in this cycle
    bool converged = false;
    for (int j = 0; j < m; ++j)
    {
      N_Vector w = L->V[j + 1];
      if (prec)
      {
        N_Vector zj = flex ? L->Z[j] : L->z;
        if (L->psolve(L->P_data, L->V[j], zj, delta, L->pretype)) return 1;
        if (L->atimes(L->A_data, zj, w)) return 1;
      }
      else if (L->atimes(L->A_data, L->V[j], w)) return 1;
      if (L->gstype == STS_MODIFIED_GS)
      {
        for (int i = 0; i <= j; ++i)
        {
          Hij(i, j) = N_VDotProd_Sts(w, L->V[i]);
          N_VLinearSum_Sts(-Hij(i, j), L->V[i], 1.0, w, w);
        }
      }
      else
      {
        for (int pass = 0; pass < 2; ++pass)
        {
          double* hp = pass ? h2.data() : h.data();
          if (N_VDotProdMulti_Sts(j + 1, w, L->V.data(), hp)) return -1;
          cf[0] = 1.0;
          X[0]  = w;
          for (int i = 0; i <= j; ++i)
          {
            cf[i + 1] = -hp[i];
            X[i + 1]  = L->V[i];
          }
          N_VLinearCombination_Sts(j + 2, cf.data(), X.data(), w);
        }
        for (int i = 0; i <= j; ++i) Hij(i, j) = h[i] + h2[i];
      }
      const double hn = sqrt(N_VDotProd_Sts(w, w));
      Hij(j + 1, j)   = hn;
      // apply the previous rotations to column j, then the new one
      for (int i = 0; i < j; ++i)
      {
        const double a = Hij(i, j), bb = Hij(i + 1, j);
        Hij(i, j)     = cs[i] * a + sn[i] * bb;
        Hij(i + 1, j) = cs[i] * bb - sn[i] * a;
      }
      givens(Hij(j, j), Hij(j + 1, j), &cs[j], &sn[j]);
      Hij(j, j)     = cs[j] * Hij(j, j) + sn[j] * Hij(j + 1, j);
      Hij(j + 1, j) = 0.0;
      g[j + 1]      = -sn[j] * g[j];
      g[j]          = cs[j] * g[j];
      k             = j + 1;
      L->last_iters++;
      L->last_res = fabs(g[j + 1]) / bnorm;
      if (hn > 0.0) N_VScale_Sts(1.0 / hn, w, w);
      if (fabs(g[j + 1]) <= delta * bnorm || !(hn > 0.0))
      {
        converged = fabs(g[j + 1]) <= delta * bnorm;
        break;
      }
    }
    // y = H^-1 g (upper triangular, k columns); u = V y; x += P^-1 u (flexible: x += Z y)
    for (int i = k - 1; i >= 0; --i)
    {
      double sacc = g[i];
      for (int q = i + 1; q < k; ++q) sacc = sacc - Hij(i, q) * y[q];
      y[i] = sacc / Hij(i, i);
    }
    if (flex)
    {
      N_VLinearCombination_Sts(k, y.data(), L->Z.data(), L->Ap);
      N_VLinearSum_Sts(1.0, x, 1.0, L->Ap, x);
    }
    else
    {
      N_VLinearCombination_Sts(k, y.data(), L->V.data(), L->Ap);
      if (prec)
      {
        if (L->psolve(L->P_data, L->Ap, L->z, delta, L->pretype)) return 1;
        N_VLinearSum_Sts(1.0, x, 1.0, L->z, x);
      }
      else N_VLinearSum_Sts(1.0, x, 1.0, L->Ap, x);
    }
    if (converged) return 0;
    if (cycle == L->max_restarts) break;
    // restart from the true residual r = b - A x
    if (L->atimes(L->A_data, x, L->Ap)) return 1;
    N_VLinearSum_Sts(1.0, b, -1.0, L->Ap, L->r);
    beta = sqrt(N_VDotProd_Sts(L->r, L->r));
    L->last_res = beta / bnorm;
    if (beta <= delta * bnorm) return 0;
  }
  return 1; // SUNLS_CONV_FAIL / SUNLS_RES_REDUCED (recoverable)
}

extern "C" int STS_SUNLinSolSolve(void* LS, N_Vector x, N_Vector b, double delta)
{
  STS_MARK_FUNCTION;
  LinSol* L = (LinSol*)LS;
  if (!L || !L->atimes || !x || !b) return -1;
  L->last_iters = 0;
  L->last_res   = 0.0;
  return L->kind == LS_PCG ? pcg_solve(L, x, b, delta) : spgmr_solve(L, x, b, delta);
}

extern "C" int STS_SUNLinSolNumIters(void* LS) { return LS ? ((LinSol*)LS)->last_iters : 0; }
extern "C" double STS_SUNLinSolResNorm(void* LS) { return LS ? ((LinSol*)LS)->last_res : 0.0; }

extern "C" int STS_SUNLinSolFree(void* LS)
{
  LinSol* L = (LinSol*)LS;
  if (!L) return 0;
  N_VDestroy_Sts(L->r);
  N_VDestroy_Sts(L->z);
  N_VDestroy_Sts(L->Ap);
  if (L->pv) N_VDestroy_Sts(L->pv);
  for (N_Vector v : L->V) N_VDestroy_Sts(v);
  for (N_Vector v : L->Z) N_VDestroy_Sts(v);
  delete L;
  return 0;
}

// ---------------------------------------------------------------------------------------
// SDIRK2 (Alexander, gamma = 1 - 1/sqrt(2)), each stage's linear Newton correction solved
// by the fused Jacobi-PCG; same arithmetic order as the oracle's orc_sdirk2.
// ---------------------------------------------------------------------------------------
// stage solves through `solve(gamma, rhs, d, &iters)`; returns < 0 on failure
template <typename Solve>
static int sdirk2_run(STS_Problem p, N_Vector y, double t0, double h, int nsteps, long long* total_iters, Solve solve)
{
  if (!p || !y || NVL(y) != p->nx * p->ny) return -1;
  const double g = 1.0 - sqrt(0.5);
  N_Vector f = N_VClone_Sts(y), f1 = N_VClone_Sts(y), rhs = N_VClone_Sts(y), d = N_VClone_Sts(y),
           Y1 = N_VClone_Sts(y);
  long long iters = 0;
  double t        = t0;
  int ret         = 0;
  for (int s = 0; s < nsteps && ret == 0; ++s)
  {
    const double hg = h * g;
    int it          = 0;
    STS_Diffusion(t + g * h, y, f, p);
    N_VScale_Sts(hg, f, rhs);
    if (solve(hg, rhs, d, &it) < 0) ret = -1;
    iters += it;
    N_VLinearSum_Sts(1.0, y, 1.0, d, Y1);
    STS_Diffusion(t + g * h, Y1, f1, p);
    STS_Diffusion(t + h, y, f, p);
    const double h1g = h * (1.0 - g);
    N_VLinearSum_Sts(h1g, f1, hg, f, rhs);
    if (solve(hg, rhs, d, &it) < 0) ret = -1;
    iters += it;
    N_VLinearSum_Sts(1.0, y, 1.0, d, y);
    t = t0 + (s + 1) * h;
  }
  STS_ContextSynchronize(p->ctx);
  N_VDestroy_Sts(f);
  N_VDestroy_Sts(f1);
  N_VDestroy_Sts(rhs);
  N_VDestroy_Sts(d);
  N_VDestroy_Sts(Y1);
  if (total_iters) *total_iters = iters;
  return ret;
}

extern "C" int STS_SDIRK2Evolve(STS_Problem p, N_Vector y, double t0, double h, int nsteps, double tol, int maxit,
                                long long* total_iters)
{
  STS_MARK_FUNCTION;
  return sdirk2_run(p, y, t0, h, nsteps, total_iters, [&](double hg, N_Vector rhs, N_Vector d, int* it) {
    double rel;
    return STS_ImplicitSolvePCG(p, hg, rhs, d, tol, maxit, 1, it, &rel);
  });
}

// The SDIRK2 driver with a generic SUNLinearSolver: ATimes v -> v - gamma A v through the
// problem's J*v, PSolve the Jacobi STS_PSolve (ARKODE's linear-solver interface attaches its
// own ATimes and the user's preconditioner in the same way, main.cpp:302-316).
namespace {
struct ShiftedOp {
  STS_Problem p;
  double gamma;
  N_Vector tmp;
};
int shifted_atimes(void* d, N_Vector v, N_Vector z)
{
  ShiftedOp* a = (ShiftedOp*)d;
  if (STS_JacTimes(v, a->tmp, 0.0, nullptr, nullptr, a->p, nullptr)) return -1;
  N_VLinearSum_Sts(1.0, v, -a->gamma, a->tmp, z);
  return 0;
}
int jacobi_psolve(void* d, N_Vector r, N_Vector z, double tol, int lr)
{
  ShiftedOp* a = (ShiftedOp*)d;
  return STS_PSolve(0.0, nullptr, nullptr, r, z, a->gamma, tol, lr, a->p);
}
} // namespace

extern "C" int STS_SDIRK2EvolveLS(STS_Problem p, void* LS, int precond, N_Vector y, double t0, double h,
                                  int nsteps, double tol, long long* total_iters)
{
  STS_MARK_FUNCTION;
  LinSol* L = (LinSol*)LS;
  if (!p || !L || !y) return -1;
  ShiftedOp op{p, 0.0, N_VClone_Sts(y)};
  STS_SUNLinSolSetATimes(L, &op, shifted_atimes);
  STS_SUNLinSolSetPreconditioner(L, precond ? &op : nullptr, precond ? jacobi_psolve : nullptr);
  const int rc = sdirk2_run(p, y, t0, h, nsteps, total_iters, [&](double hg, N_Vector rhs, N_Vector d, int* it) {
    op.gamma     = hg;
    const int sr = STS_SUNLinSolSolve(L, d, rhs, tol);
    *it          = STS_SUNLinSolNumIters(L);
    return sr < 0 ? -1 : 0;
  });
  STS_SUNLinSolSetATimes(L, nullptr, nullptr);
  STS_SUNLinSolSetPreconditioner(L, nullptr, nullptr);
  N_VDestroy_Sts(op.tmp);
  return rc;
}

// One shifted system (I - gamma A) x = b through a generic solver object (PCG, SPGMR or
// SPFGMR): ATimes is the shifted operator, the preconditioner none (prec 0), the Jacobi PSolve
// (1) or the caller's (2: P_data and psolve, e.g. STS_PFMGPrecSolve or STS_NetPrecSolve after
// their PSetup). The solver keeps no reference to the callbacks after the call.
extern "C" int STS_ImplicitSolveLS(STS_Problem p, double gamma, void* LS, int prec, void* P_data,
                                   STS_PSolveFn psolve, N_Vector b, N_Vector x, double tol, int* iters,
                                   double* relres)
{
  STS_MARK_FUNCTION;
  LinSol* L = (LinSol*)LS;
  if (!p || !L || !b || !x || prec < 0 || prec > 2 || (prec == 2 && !psolve) ||
      (prec != 0 && L->pretype == STS_PREC_NONE))
  {
    sts_set_error("ImplicitSolveLS: invalid arguments (a preconditioner needs a solver made with a "
                  "preconditioning type)");
    return -1;
  }
  ShiftedOp op{p, gamma, N_VClone_Sts(b)};
  STS_SUNLinSolSetATimes(L, &op, shifted_atimes);
  if (prec == 1) STS_SUNLinSolSetPreconditioner(L, &op, jacobi_psolve);
  else if (prec == 2) STS_SUNLinSolSetPreconditioner(L, P_data, psolve);
  else STS_SUNLinSolSetPreconditioner(L, nullptr, nullptr);
  const int rc = STS_SUNLinSolSolve(L, x, b, tol);
  if (iters) *iters = STS_SUNLinSolNumIters(L);
  if (relres) *relres = STS_SUNLinSolResNorm(L);
  STS_SUNLinSolSetATimes(L, nullptr, nullptr);
  STS_SUNLinSolSetPreconditioner(L, nullptr, nullptr);
  N_VDestroy_Sts(op.tmp);
  return rc;
}

// The SDIRK2 driver with each stage solved by CG with the PFMG-role multigrid preconditioner
// (the reference built with hypre: preconditioner_hypre.cpp attached by main.cpp:311)
extern "C" int STS_SDIRK2EvolvePFMG(STS_Problem p, STS_PFMG mg, N_Vector y, double t0, double h, int nsteps,
                                    double tol, int maxit, long long* total_iters)
{
  STS_MARK_FUNCTION;
  if (!mg) return -1;
  return sdirk2_run(p, y, t0, h, nsteps, total_iters, [&](double hg, N_Vector rhs, N_Vector d, int* it) {
    double rel;
    return STS_ImplicitSolvePFMG(p, hg, mg, rhs, d, tol, maxit, it, &rel) < 0 ? -1 : 0;
  });
}

// The same SDIRK2 driver with each stage solved by STS_ImplicitSolveLearned (FCG with the
// learned preconditioner where the condition estimate favours it, Jacobi-PCG elsewhere).
extern "C" int STS_SDIRK2EvolveLearned(STS_Problem p, STS_Net net, N_Vector y, double t0, double h, int nsteps,
                                       double tol, int maxit, long long* total_iters)
{
  STS_MARK_FUNCTION;
  return sdirk2_run(p, y, t0, h, nsteps, total_iters, [&](double hg, N_Vector rhs, N_Vector d, int* it) {
    double rel;
    int used;
    return STS_ImplicitSolveLearned(p, hg, net, rhs, d, tol, maxit, 0.0, it, &rel, &used);
  });
}
