// Structured multigrid preconditioner for the implicit comparator, in the role hypre's PFMG
// plays in diffusion_2D/preconditioner_hypre.cpp (PSetup :13-108, PSolve :111-180): one
// V-cycle per PSolve (PFMG MaxIter 1, zero initial guess), semicoarsening one direction at a
// time, non-Galerkin coarse operators (RAPType 1), weighted Jacobi, symmetric or nonsymmetric
// red/black Gauss-Seidel relaxation (--pfmg_relax 1 / 2 / 3; the reference's default 2, its
// experiment harness passes 3) with --pfmg_nrelax
// pre and post sweeps (default 2).
//
// The restatement (hypre is not in the reference tree):
//   Level 0 is M = I - gamma A on the nx x ny interior grid: diagonal d = 1 - gamma cc,
//   couplings a_x = gamma cx, a_y = gamma cy. A level is coarsened in the direction with the
//   larger coupling (among the directions with more than two points): coarse point I is fine
//   point 2I + 1 in that direction (floor(n/2) coarse points), the coupling there becomes
//   a/4 (twice the spacing), the other direction's is kept, d = 1 + 2 (a_x + a_y).
//   Prolongation P: linear interpolation in the coarsened direction (fine 2I+1 takes coarse I,
//   fine 2I the mean of coarse I-1 and I, zero beyond the boundary); restriction R = P^T / 2
//   (full weighting 1/4, 1/2, 1/4). Relaxation with symmetric schedules (Jacobi with the same
//   weight before and after; red then black before, black then red after), the coarsest
//   level (at most 2 x 2 points) relaxed 8 times: the V-cycle is a symmetric positive
//   definite operator, so it preconditions CG.
// Every kernel is elementwise with an explicit operation order (fused multiply-adds written
// out), so the CPU oracle reproduces the V-cycle bit for bit. The cycle for a given gamma is
// captured once in a CUDA graph (about 7 kernels per level, ~22 levels at 2048^2).
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "sts_internal.cuh"

namespace {

constexpr double PFMG_OMEGA = 0.8; // weighted-Jacobi factor (2-D five-point stencil)
constexpr int PFMG_COARSE_SWEEPS = 8;
constexpr int PFMG_MAX_LEVELS    = 64;

struct PfmgLevel {
  long long nx = 0, ny = 0;
  double ax = 0, ay = 0, d = 1, dinv = 1, wd = 1;
  int dir = -1;                 // direction coarsened towards the next level (0 x, 1 y), -1 coarsest
  double *f = nullptr, *u = nullptr, *t = nullptr; // right side, iterate, scratch (residual / Jacobi)
  // periodic problems: coupling of each x face (i + 1/2, i = 0..nx-1, the last one wrapping to
  // column 0) and y face, on the device and the host
  double *axf = nullptr, *ayf = nullptr;
  std::vector<double> hax, hay;
};

__device__ __forceinline__ double at(const double* u, long long nx, long long ny, long long i, long long j)
{
  return (i >= 0 && i < nx && j >= 0 && j < ny) ? u[j * nx + i] : 0.0;
}

// M u at (i, j): d u - a_x (u_w + u_e) - a_y (u_s + u_n)
__device__ __forceinline__ double apply_m(const double* u, long long nx, long long ny, long long i, long long j,
                                          double ax, double ay, double d)
{
  const double sx = at(u, nx, ny, i - 1, j) + at(u, nx, ny, i + 1, j);
  const double sy = at(u, nx, ny, i, j - 1) + at(u, nx, ny, i, j + 1);
  double m        = d * u[j * nx + i];
  m               = __fma_rn(-ax, sx, m);
  m               = __fma_rn(-ay, sy, m);
  return m;
}

// weighted Jacobi: out = in + wd (f - M in)
__global__ void jacobi_kernel(long long nx, long long ny, double ax, double ay, double d, double wd,
                              const double* __restrict__ f, const double* __restrict__ in, double* __restrict__ out)
{
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long j = (long long)blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= nx || j >= ny) return;
  const long long k = j * nx + i;
  out[k]            = __fma_rn(wd, f[k] - apply_m(in, nx, ny, i, j, ax, ay, d), in[k]);
}

// Gauss-Seidel on the points with (i + j) % 2 == color: u = dinv (f + a_x (u_w + u_e) + a_y (u_s + u_n))
__global__ void rbgs_kernel(long long nx, long long ny, double ax, double ay, double dinv, const double* __restrict__ f,
                            double* u, int color)
{
  const long long i = 2 * ((long long)blockIdx.x * blockDim.x + threadIdx.x);
  const long long j = (long long)blockIdx.y * blockDim.y + threadIdx.y;
  const long long ii = i + ((j + color) & 1); // the point of this color in the pair (i, i+1)
  if (ii >= nx || j >= ny) return;
  const double sx = at(u, nx, ny, ii - 1, j) + at(u, nx, ny, ii + 1, j);
  const double sy = at(u, nx, ny, ii, j - 1) + at(u, nx, ny, ii, j + 1);
  double v        = __fma_rn(ax, sx, f[j * nx + ii]);
  v               = __fma_rn(ay, sy, v);
  u[j * nx + ii]  = dinv * v;
}

__global__ void residual_kernel(long long nx, long long ny, double ax, double ay, double d, const double* __restrict__ f,
                                const double* __restrict__ u, double* __restrict__ r)
{
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long j = (long long)blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= nx || j >= ny) return;
  r[j * nx + i] = f[j * nx + i] - apply_m(u, nx, ny, i, j, ax, ay, d);
}

// full weighting in direction dir onto the coarse grid (cnx x cny): fc = 0.5 b + 0.25 (a + c)
__global__ void restrict_kernel(long long nx, long long ny, int dir, long long cnx, long long cny,
                                const double* __restrict__ r, double* __restrict__ fc)
{
  const long long I = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long J = (long long)blockIdx.y * blockDim.y + threadIdx.y;
  if (I >= cnx || J >= cny) return;
  double a, b, c;
  if (dir == 0)
  {
    a = at(r, nx, ny, 2 * I, J);
    b = at(r, nx, ny, 2 * I + 1, J);
    c = at(r, nx, ny, 2 * I + 2, J);
  }
  else
  {
    a = at(r, nx, ny, I, 2 * J);
    b = at(r, nx, ny, I, 2 * J + 1);
    c = at(r, nx, ny, I, 2 * J + 2);
  }
  fc[J * cnx + I] = __fma_rn(0.5, b, 0.25 * (a + c));
}

// u += P uc (linear interpolation in direction dir)
__global__ void prolong_kernel(long long nx, long long ny, int dir, long long cnx, long long cny,
                               const double* __restrict__ uc, double* __restrict__ u)
{
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long j = (long long)blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= nx || j >= ny) return;
  const long long q = dir == 0 ? i : j;
  double e;
  if (q & 1)
  {
    const long long Q = q >> 1;
    e = dir == 0 ? at(uc, cnx, cny, Q, j) : at(uc, cnx, cny, i, Q);
  }
  else
  {
    const long long Q = q >> 1; // between coarse Q - 1 and Q
    const double lo = dir == 0 ? at(uc, cnx, cny, Q - 1, j) : at(uc, cnx, cny, i, Q - 1);
    const double hi = dir == 0 ? at(uc, cnx, cny, Q, j) : at(uc, cnx, cny, i, Q);
    e = 0.5 * (lo + hi);
  }
  u[j * nx + i] += e;
}

// ---- periodic levels (the reference's problem): variable face couplings, wrapped neighbours.
// M u = d u - (w u_W + e u_E + s u_S + n u_N), w = axf[i-1], e = axf[i], s = ayf[j-1], n = ayf[j],
// d = 1 + ((w + e) + (s + n)).
__device__ __forceinline__ long long wrap(long long i, long long n) { return i < 0 ? i + n : (i >= n ? i - n : i); }

struct PerPoint {
  double w, e, s, n, d, uW, uE, uS, uN;
};

__device__ __forceinline__ PerPoint per_point(const double* u, long long nx, long long ny, long long i, long long j,
                                              const double* axf, const double* ayf)
{
  PerPoint q;
  const long long iw = wrap(i - 1, nx), ie = wrap(i + 1, nx), js = wrap(j - 1, ny), jn = wrap(j + 1, ny);
  q.w  = axf[iw];
  q.e  = axf[i];
  q.s  = ayf[js];
  q.n  = ayf[j];
  q.d  = 1.0 + ((q.w + q.e) + (q.s + q.n));
  q.uW = u[j * nx + iw];
  q.uE = u[j * nx + ie];
  q.uS = u[js * nx + i];
  q.uN = u[jn * nx + i];
  return q;
}

__device__ __forceinline__ double per_m(const PerPoint& q, double uc)
{
  double m = q.d * uc;
  m        = __fma_rn(-q.w, q.uW, m);
  m        = __fma_rn(-q.e, q.uE, m);
  m        = __fma_rn(-q.s, q.uS, m);
  m        = __fma_rn(-q.n, q.uN, m);
  return m;
}

__global__ void per_jacobi_kernel(long long nx, long long ny, const double* __restrict__ axf,
                                  const double* __restrict__ ayf, const double* __restrict__ f,
                                  const double* __restrict__ in, double* __restrict__ out)
{
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long j = (long long)blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= nx || j >= ny) return;
  const long long k = j * nx + i;
  const PerPoint q  = per_point(in, nx, ny, i, j, axf, ayf);
  const double wd   = PFMG_OMEGA * (1.0 / q.d);
  out[k]            = __fma_rn(wd, f[k] - per_m(q, in[k]), in[k]);
}

// one colour of red/black Gauss-Seidel from `in` into `out` (the other colour copied): on odd
// periodic sizes, where two points of one colour meet across the wrap, the sweep stays
// deterministic
__global__ void per_rbgs_kernel(long long nx, long long ny, const double* __restrict__ axf,
                                const double* __restrict__ ayf, const double* __restrict__ f,
                                const double* __restrict__ in, double* __restrict__ out, int color)
{
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long j = (long long)blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= nx || j >= ny) return;
  const long long k = j * nx + i;
  if (((i + j) & 1) != color)
  {
    out[k] = in[k];
    return;
  }
  const PerPoint q = per_point(in, nx, ny, i, j, axf, ayf);
  double v         = __fma_rn(q.w, q.uW, f[k]);
  v                = __fma_rn(q.e, q.uE, v);
  v                = __fma_rn(q.s, q.uS, v);
  v                = __fma_rn(q.n, q.uN, v);
  out[k]           = v / q.d;
}

__global__ void per_residual_kernel(long long nx, long long ny, const double* __restrict__ axf,
                                    const double* __restrict__ ayf, const double* __restrict__ f,
                                    const double* __restrict__ u, double* __restrict__ r)
{
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long j = (long long)blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= nx || j >= ny) return;
  const PerPoint q = per_point(u, nx, ny, i, j, axf, ayf);
  r[j * nx + i]    = f[j * nx + i] - per_m(q, u[j * nx + i]);
}

// full weighting with wrap: coarse I <- fine 2I, 2I+1, 2I+2 (mod n)
__global__ void per_restrict_kernel(long long nx, long long ny, int dir, long long cnx, long long cny,
                                    const double* __restrict__ r, double* __restrict__ fc)
{
  const long long I = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long J = (long long)blockIdx.y * blockDim.y + threadIdx.y;
  if (I >= cnx || J >= cny) return;
  double a, b, c;
  if (dir == 0)
  {
    a = r[J * nx + 2 * I];
    b = r[J * nx + 2 * I + 1];
    c = r[J * nx + wrap(2 * I + 2, nx)];
  }
  else
  {
    a = r[(2 * J) * nx + I];
    b = r[(2 * J + 1) * nx + I];
    c = r[wrap(2 * J + 2, ny) * nx + I];
  }
  fc[J * cnx + I] = __fma_rn(0.5, b, 0.25 * (a + c));
}

// u += P uc with wrap: fine 2Q+1 <- coarse Q, fine 2Q <- mean of coarse Q-1 (mod) and Q
__global__ void per_prolong_kernel(long long nx, long long ny, int dir, long long cnx, long long cny,
                                   const double* __restrict__ uc, double* __restrict__ u)
{
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long j = (long long)blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= nx || j >= ny) return;
  const long long q = dir == 0 ? i : j;
  const long long Q = q >> 1;
  double e;
  if (q & 1) e = dir == 0 ? uc[j * cnx + Q] : uc[Q * cnx + i];
  else
  {
    const long long Qm = wrap(Q - 1, dir == 0 ? cnx : cny);
    const double lo    = dir == 0 ? uc[j * cnx + Qm] : uc[Qm * cnx + i];
    const double hi    = dir == 0 ? uc[j * cnx + Q] : uc[Q * cnx + i];
    e                  = 0.5 * (lo + hi);
  }
  u[j * nx + i] += e;
}

dim3 blocks2d(long long nx, long long ny, dim3 b) { return dim3((unsigned)((nx + b.x - 1) / b.x), (unsigned)((ny + b.y - 1) / b.y)); }

// coarse coupling of two fine faces in series (twice the spacing): 0.5 a1 a2 / (a1 + a2)
double series_coupling(double a1, double a2)
{
  const double s = a1 + a2;
  if (!(s > 0.0)) return 0.0;
  const double t = a1 * a2;
  return 0.5 * (t / s);
}

} // namespace

struct STS_PFMG_ {
  STS_Problem p   = nullptr;
  STS_Context ctx = nullptr; // kept separately: freeing the PFMG must not need the problem
  int relax       = 2;
  int nrelax      = 2;
  bool periodic   = false;
  std::vector<double> dxe, dyn; // periodic problems: the problem's face coefficients (host copy)
  double gamma    = NAN; // the gamma the hierarchy and graph were built for
  std::vector<PfmgLevel> L;
  cudaGraphExec_t graph = nullptr;
  long long vcycles = 0;
};

static void pfmg_free_levels(STS_PFMG mg)
{
  for (auto& l : mg->L)
  {
    cudaFree(l.f);
    cudaFree(l.u);
    cudaFree(l.t);
    if (l.axf) cudaFree(l.axf);
    if (l.ayf) cudaFree(l.ayf);
  }
  mg->L.clear();
  if (mg->graph) cudaGraphExecDestroy(mg->graph);
  mg->graph = nullptr;
}

// the level hierarchy of M = I - gamma A (host rules, restated in the oracle)
// periodic problems: per-face couplings; coarsening of an even direction with a coupling at
// least the other's (largest face), the coarse faces two fine faces in series
static bool pfmg_build_periodic(STS_PFMG mg, double gamma)
{
  STS_Problem p = mg->p;
  PfmgLevel l;
  l.nx = p->nx;
  l.ny = p->ny;
  l.hax.resize(l.nx);
  l.hay.resize(l.ny);
  for (long long i = 0; i < l.nx; ++i) l.hax[i] = gamma * mg->dxe[i];
  for (long long j = 0; j < l.ny; ++j) l.hay[j] = gamma * mg->dyn[j];
  for (int lev = 0; lev < PFMG_MAX_LEVELS; ++lev)
  {
    if (lev > 0)
    {
      const PfmgLevel& f = mg->L.back();
      PfmgLevel c;
      c.nx  = f.dir == 0 ? f.nx / 2 : f.nx;
      c.ny  = f.dir == 1 ? f.ny / 2 : f.ny;
      c.hax = f.hax;
      c.hay = f.hay;
      if (f.dir == 0)
      {
        c.hax.resize(c.nx);
        for (long long I = 0; I < c.nx; ++I) c.hax[I] = series_coupling(f.hax[2 * I + 1], f.hax[(2 * I + 2) % f.nx]);
      }
      else
      {
        c.hay.resize(c.ny);
        for (long long J = 0; J < c.ny; ++J) c.hay[J] = series_coupling(f.hay[2 * J + 1], f.hay[(2 * J + 2) % f.ny]);
      }
      l = c;
    }
    double axm = 0.0, aym = 0.0;
    for (double a : l.hax) axm = a > axm ? a : axm;
    for (double a : l.hay) aym = a > aym ? a : aym;
    const bool cx = l.nx > 2 && l.nx % 2 == 0, cy = l.ny > 2 && l.ny % 2 == 0;
    if (cx && (axm >= aym || !cy)) l.dir = 0;
    else if (cy) l.dir = 1;
    else l.dir = -1;
    const size_t bytes = (size_t)(l.nx * l.ny) * sizeof(double);
    if (!STS_CUDA_OK(cudaMalloc(&l.f, bytes)) || !STS_CUDA_OK(cudaMalloc(&l.u, bytes)) ||
        !STS_CUDA_OK(cudaMalloc(&l.t, bytes)) || !STS_CUDA_OK(cudaMalloc(&l.axf, l.nx * sizeof(double))) ||
        !STS_CUDA_OK(cudaMalloc(&l.ayf, l.ny * sizeof(double))) ||
        !STS_CUDA_OK(cudaMemcpy(l.axf, l.hax.data(), l.nx * sizeof(double), cudaMemcpyHostToDevice)) ||
        !STS_CUDA_OK(cudaMemcpy(l.ayf, l.hay.data(), l.ny * sizeof(double), cudaMemcpyHostToDevice)))
    {
      mg->L.push_back(l);
      return false;
    }
    mg->L.push_back(l);
    if (l.dir < 0) break;
  }
  return mg->L.back().dir < 0;
}

static bool pfmg_build(STS_PFMG mg, double gamma)
{
  pfmg_free_levels(mg);
  if (mg->periodic) return pfmg_build_periodic(mg, gamma);
  STS_Problem p = mg->p;
  PfmgLevel l0;
  l0.nx = p->nx;
  l0.ny = p->ny;
  l0.ax = gamma * p->cx;
  l0.ay = gamma * p->cy;
  l0.d  = 1.0 - gamma * p->cc;
  for (int lev = 0; lev < PFMG_MAX_LEVELS; ++lev)
  {
    PfmgLevel l = lev == 0 ? l0 : mg->L.back();
    if (lev > 0)
    {
      const PfmgLevel& f = mg->L.back();
      l.f = l.u = l.t = nullptr;
      if (f.dir == 0)
      {
        l.nx = f.nx / 2;
        l.ax = f.ax * 0.25;
      }
      else
      {
        l.ny = f.ny / 2;
        l.ay = f.ay * 0.25;
      }
      l.d = 1.0 + 2.0 * (l.ax + l.ay);
    }
    l.dinv = 1.0 / l.d;
    l.wd   = PFMG_OMEGA * l.dinv;
    if (l.nx > 2 && (l.ax >= l.ay || l.ny <= 2)) l.dir = 0;
    else if (l.ny > 2) l.dir = 1;
    else l.dir = -1;
    const size_t bytes = (size_t)(l.nx * l.ny) * sizeof(double);
    if (!STS_CUDA_OK(cudaMalloc(&l.f, bytes)) || !STS_CUDA_OK(cudaMalloc(&l.u, bytes)) ||
        !STS_CUDA_OK(cudaMalloc(&l.t, bytes)))
      return false;
    mg->L.push_back(l);
    if (l.dir < 0) break;
  }
  return mg->L.back().dir < 0;
}

// smoothing sweeps on level l (u holds the iterate; Jacobi ping-pongs through t and copies back)
static void pfmg_smooth(STS_PFMG mg, PfmgLevel& l, int sweeps, bool post, cudaStream_t st)
{
  const dim3 b(32, 8);
  if (mg->periodic)
  { // every half sweep reads one buffer and writes the other; the result ends in u
    const size_t bytes = (size_t)(l.nx * l.ny) * sizeof(double);
    int nw             = 0;
    for (int s = 0; s < sweeps; ++s)
    {
      if (mg->relax == 1)
      {
        const double* in = (nw & 1) ? l.t : l.u;
        double* out      = (nw & 1) ? l.u : l.t;
        per_jacobi_kernel<<<blocks2d(l.nx, l.ny, b), b, 0, st>>>(l.nx, l.ny, l.axf, l.ayf, l.f, in, out);
        ++nw;
      }
      else
        for (int h = 0; h < 2; ++h)
        {
          const int color  = (post && mg->relax == 2) ? 1 - h : h;
          const double* in = (nw & 1) ? l.t : l.u;
          double* out      = (nw & 1) ? l.u : l.t;
          per_rbgs_kernel<<<blocks2d(l.nx, l.ny, b), b, 0, st>>>(l.nx, l.ny, l.axf, l.ayf, l.f, in, out, color);
          ++nw;
        }
    }
    if (nw & 1) cudaMemcpyAsync(l.u, l.t, bytes, cudaMemcpyDeviceToDevice, st);
    return;
  }
  if (mg->relax == 1)
  {
    for (int s = 0; s < sweeps; ++s)
    {
      const double* in = (s & 1) ? l.t : l.u;
      double* out      = (s & 1) ? l.u : l.t;
      jacobi_kernel<<<blocks2d(l.nx, l.ny, b), b, 0, st>>>(l.nx, l.ny, l.ax, l.ay, l.d, l.wd, l.f, in, out);
    }
    if (sweeps & 1) cudaMemcpyAsync(l.u, l.t, (size_t)(l.nx * l.ny) * sizeof(double), cudaMemcpyDeviceToDevice, st);
  }
  else
  {
    const dim3 g = blocks2d((l.nx + 1) / 2, l.ny, b);
    for (int s = 0; s < sweeps; ++s)
      for (int h = 0; h < 2; ++h)
      {
        // red then black before; after: black then red (relax 2, symmetric) or red then black
        // again (relax 3, nonsymmetric)
        const int color = (post && mg->relax == 2) ? 1 - h : h;
        rbgs_kernel<<<g, b, 0, st>>>(l.nx, l.ny, l.ax, l.ay, l.dinv, l.f, l.u, color);
      }
  }
}

// one V-cycle with a zero initial guess: L[0].u = B L[0].f
static void pfmg_vcycle(STS_PFMG mg, cudaStream_t st)
{
  const dim3 b(32, 8);
  const int nl = (int)mg->L.size();
  for (int lev = 0; lev < nl; ++lev)
  {
    PfmgLevel& l = mg->L[lev];
    cudaMemsetAsync(l.u, 0, (size_t)(l.nx * l.ny) * sizeof(double), st);
    if (l.dir < 0)
    {
      pfmg_smooth(mg, l, PFMG_COARSE_SWEEPS, false, st);
      break;
    }
    pfmg_smooth(mg, l, mg->nrelax, false, st);
    PfmgLevel& c = mg->L[lev + 1];
    if (mg->periodic)
    {
      per_residual_kernel<<<blocks2d(l.nx, l.ny, b), b, 0, st>>>(l.nx, l.ny, l.axf, l.ayf, l.f, l.u, l.t);
      per_restrict_kernel<<<blocks2d(c.nx, c.ny, b), b, 0, st>>>(l.nx, l.ny, l.dir, c.nx, c.ny, l.t, c.f);
      continue;
    }
    residual_kernel<<<blocks2d(l.nx, l.ny, b), b, 0, st>>>(l.nx, l.ny, l.ax, l.ay, l.d, l.f, l.u, l.t);
    restrict_kernel<<<blocks2d(c.nx, c.ny, b), b, 0, st>>>(l.nx, l.ny, l.dir, c.nx, c.ny, l.t, c.f);
  }
  for (int lev = nl - 2; lev >= 0; --lev)
  {
    PfmgLevel& l = mg->L[lev];
    const PfmgLevel& c = mg->L[lev + 1];
    if (mg->periodic)
      per_prolong_kernel<<<blocks2d(l.nx, l.ny, b), b, 0, st>>>(l.nx, l.ny, l.dir, c.nx, c.ny, c.u, l.u);
    else prolong_kernel<<<blocks2d(l.nx, l.ny, b), b, 0, st>>>(l.nx, l.ny, l.dir, c.nx, c.ny, c.u, l.u);
    pfmg_smooth(mg, l, mg->nrelax, true, st);
  }
}

extern "C" STS_PFMG STS_PFMGCreate(STS_Problem p, int relax_type, int nrelax)
{
  if (!p || relax_type < 1 || relax_type > 3 || nrelax < 1 || nrelax > 16)
  {
    sts_set_error("STS_PFMGCreate: relax 1 (weighted Jacobi), 2 (symmetric red/black Gauss-Seidel) or 3 "
                  "(nonsymmetric red/black Gauss-Seidel), 1 <= nrelax <= 16");
    return nullptr;
  }
  STS_PFMG mg   = new STS_PFMG_();
  mg->p         = p;
  mg->ctx       = p->ctx;
  mg->relax     = relax_type;
  mg->nrelax    = nrelax;
  mg->periodic  = p->kind == STS_PROBLEM_PERIODIC;
  if (mg->periodic)
  { // the face coefficients / d^2 of the problem's operator (diffusion.cpp:36-46)
    mg->dxe.resize(p->nx);
    mg->dyn.resize(p->ny);
    ctx_activate(p->ctx);
    if (!STS_CUDA_OK(cudaMemcpy(mg->dxe.data(), p->dev.Dxe, p->nx * sizeof(double), cudaMemcpyDeviceToHost)) ||
        !STS_CUDA_OK(cudaMemcpy(mg->dyn.data(), p->dev.Dyn, p->ny * sizeof(double), cudaMemcpyDeviceToHost)))
    {
      delete mg;
      return nullptr;
    }
  }
  return mg;
}

extern "C" void STS_PFMGFree(STS_PFMG* mg)
{
  if (!mg || !*mg) return;
  ctx_activate((*mg)->ctx);
  cudaStreamSynchronize((*mg)->ctx->stream);
  pfmg_free_levels(*mg);
  delete *mg;
  *mg = nullptr;
}

extern "C" int STS_PFMGNumLevels(STS_PFMG mg) { return mg ? (int)mg->L.size() : 0; }
extern "C" long long STS_PFMGNumVCycles(STS_PFMG mg) { return mg ? mg->vcycles : 0; }

// PSetup (preconditioner_hypre.cpp:13-108): the hierarchy and the captured V-cycle for gamma
extern "C" int STS_PFMGPSetup(double t, N_Vector u, N_Vector f, int jok, int* jcurPtr, double gamma, void* user_data)
{
  STS_MARK_FUNCTION;
  (void)t;
  (void)u;
  (void)f;
  (void)jok;
  STS_PFMG mg = (STS_PFMG)user_data;
  if (!mg || !(gamma >= 0.0)) return -1;
  if (jcurPtr) *jcurPtr = 1;
  if (gamma == mg->gamma && mg->graph) return 0;
  ctx_activate(mg->p->ctx);
  cudaStream_t st = mg->p->ctx->stream;
  if (!STS_CUDA_OK(cudaStreamSynchronize(st)) || !pfmg_build(mg, gamma))
  {
    sts_set_error("STS_PFMGPSetup: out of device memory");
    return -1;
  }
  cudaGraph_t g;
  if (!STS_CUDA_OK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal))) return -1;
  pfmg_vcycle(mg, st);
  if (!STS_CUDA_OK(cudaStreamEndCapture(st, &g))) return -1;
  const bool ok = STS_CUDA_OK(cudaGraphInstantiate(&mg->graph, g, 0));
  cudaGraphDestroy(g);
  if (!ok) return -1;
  mg->gamma = gamma;
  return 0;
}

// PSolve (preconditioner_hypre.cpp:111-180): z = one V-cycle applied to r
extern "C" int STS_PFMGPSolve(double t, N_Vector u, N_Vector f, N_Vector r, N_Vector z, double gamma, double delta,
                              int lr, void* user_data)
{
  STS_MARK_FUNCTION;
  (void)t;
  (void)u;
  (void)f;
  (void)delta;
  (void)lr;
  STS_PFMG mg = (STS_PFMG)user_data;
  if (!mg || !r || !z) return -1;
  const long long n = mg->p->nx * mg->p->ny;
  if (NVL(r) != n || NVL(z) != n) return -1;
  if (!(gamma == mg->gamma && mg->graph) && STS_PFMGPSetup(0.0, nullptr, nullptr, 0, nullptr, gamma, mg) != 0)
    return -1;
  ctx_activate(mg->p->ctx);
  cudaStream_t st = mg->p->ctx->stream;
  PfmgLevel& l0   = mg->L[0];
  if (!STS_CUDA_OK(cudaMemcpyAsync(l0.f, NVD(r), n * sizeof(double), cudaMemcpyDeviceToDevice, st)) ||
      !STS_CUDA_OK(cudaGraphLaunch(mg->graph, st)) ||
      !STS_CUDA_OK(cudaMemcpyAsync(NVD(z), l0.u, n * sizeof(double), cudaMemcpyDeviceToDevice, st)))
    return -1;
  mg->vcycles++;
  return 0;
}

// the SUNLinSol PSolve callback form (P_data = the STS_PFMG, set up for the system's gamma)
extern "C" int STS_PFMGPrecSolve(void* P_data, N_Vector r, N_Vector z, double tol, int lr)
{
  STS_MARK_FUNCTION;
  STS_PFMG mg = (STS_PFMG)P_data;
  return mg ? STS_PFMGPSolve(0.0, nullptr, nullptr, r, z, mg->gamma, tol, lr, mg) : -1;
}

// (I - gamma A) x = b by CG with the PFMG preconditioner (SUNLinSol_PCG through the callbacks,
// x0 = 0, stop at ||r||_2 <= tol ||b||_2)
namespace {
struct ShiftOp {
  STS_Problem p;
  double gamma;
  N_Vector tmp;
};
int shift_atimes(void* d, N_Vector v, N_Vector z)
{
  ShiftOp* a = (ShiftOp*)d;
  if (STS_JacTimes(v, a->tmp, 0.0, nullptr, nullptr, a->p, nullptr)) return -1;
  N_VLinearSum_Sts(1.0, v, -a->gamma, a->tmp, z);
  return 0;
}
} // namespace

extern "C" int STS_ImplicitSolvePFMG(STS_Problem p, double gamma, STS_PFMG mg, N_Vector b, N_Vector x, double tol,
                                     int maxit, int* iters, double* relres)
{
  STS_MARK_FUNCTION;
  if (!p || !mg || mg->p != p || !b || !x || maxit < 1) return -1;
  if (STS_PFMGPSetup(0.0, nullptr, nullptr, 0, nullptr, gamma, mg) != 0) return -1;
  void* LS = STS_SUNLinSol_PCG(b, STS_PREC_RIGHT, maxit, p->ctx);
  if (!LS) return -1;
  ShiftOp op{p, gamma, N_VClone_Sts(b)};
  STS_SUNLinSolSetATimes(LS, &op, shift_atimes);
  STS_SUNLinSolSetPreconditioner(LS, mg, STS_PFMGPrecSolve);
  const int rc = STS_SUNLinSolSolve(LS, x, b, tol);
  if (iters) *iters = STS_SUNLinSolNumIters(LS);
  if (relres) *relres = STS_SUNLinSolResNorm(LS);
  STS_SUNLinSolFree(LS);
  N_VDestroy_Sts(op.tmp);
  return rc;
}
