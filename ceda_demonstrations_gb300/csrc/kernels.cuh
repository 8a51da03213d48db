// Device kernels of the fused STS path: point stencils, the FP64 stage kernel (Y form), the
// mixed FP32-increment stage kernel, the stage-1 kernels and the step-end kernels that fuse
// F(y_{n+1}), the embedded error estimate and its exact WRMS norm.
//
// Stage recurrence (LSRKStep RKC2/RKL2, restated from rkc.f / Meyer-Balsara-Aslam 2014):
//   Y_j = mu_j Y_{j-1} + nu_j Y_{j-2} + (1-mu_j-nu_j) Y_0 + h mus_j F(Y_{j-1}) - h mus_j a_{j-1} F_0
// With F(Y) = cc Y_C + cx (Y_W+Y_E) + cy (Y_S+Y_N) + b(t) the per-stage scalars fold into
//   Y_j = gc Y_C + gx (Y_W+Y_E) + gy (Y_S+Y_N) + gn Y_{j-2} + g0 Y_0 + gf F_0 + hm b(t_j)
// (gc = mu + hm cc, gx = hm cx, gy = hm cy, gn = nu, g0 = 1-mu-nu, gf = -hm a_{j-1}, hm = h mus).
// The mixed form streams d_j = Y_j - Y_0 in FP32 and uses F(Y_{j-1}) = F_0 + A d_{j-1} + (b_j - b_0):
//   d_j = mu d_{j-1} + nu d_{j-2} + hm A d_{j-1} + hm (1-a_{j-1}) F_0 + hm (b_j - b_0),
// evaluated in difference form (mixed_point below): d_j = d_C + inc with
//   inc = gs d_C + gx ((d_W-d_C) + (d_E-d_C)) + gy ((d_S-d_C) + (d_N-d_C)) + gm (d_C - d_{j-2})
//       + gF F_0 + hm (b_j - b_0),
//   gs = mu + nu - 1 + hm (cc + 2 cx + 2 cy), gm = -nu, gF = hm (1 - a_{j-1}).
// Every FP32 operation then rounds a quantity of the size of the stage-to-stage increment,
// not of d itself: the neighbour differences of a smooth field and d_C - d_{j-2} are exact
// (Sterbenz) or small, and d_C + inc is the only rounding at the scale of d. Summing the
// large terms gc d_C + gx (d_W+d_E) + ... directly lets the FP32 roundings of O(|d|) sums
// feed a coherent error through the (s - j)-fold growth of the Chebyshev recurrence for
// smooth modes; on the 8192^2 anisotropic RKC2 workload it reached 1.6e-6 relative L2 against
// FP64 at t = 0.05, against about 1e-8 in the difference form.
#pragma once
#include <cuda_runtime.h>

#include "sts_internal.cuh"

struct StageArgs {
  double gc, gx, gy, gn, g0, gf, al, be, ga;
  // mixed (difference) form: gsf = mu + nu - 1 + hm (cc + 2 cx + 2 cy), gmf = -nu
  float gsf, gxf, gyf, gmf, gFf, alf, bef, gaf;
};

struct StepArgs {
  double hm1;            // h mus_1 (stage 1)
  double p4h;            // 0.4 h
  double rtol, atol;
  double al, be, ga;     // forcing scalars at t + h (unscaled)
  float hm1f;
  float pad_;
};

// ---------------------------------------------------------------------------------------
// point operators
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ double dirichlet_point(const ProbDev& P, const double* __restrict__ u,
                                                  long long i, long long j)
{
  const long long k = j * P.nx + i;
  const double uc   = u[k];
  const double uw   = (i > 0) ? u[k - 1] : 0.0;
  const double ue   = (i < P.nx - 1) ? u[k + 1] : 0.0;
  const double us   = (j > 0) ? u[k - P.nx] : 0.0;
  const double un   = (j < P.ny - 1) ? u[k + P.nx] : 0.0;
  const double sx = uw + ue, sy = us + un;
  double acc = P.cc * uc;
  acc        = __fma_rn(P.cx, sx, acc);
  acc        = __fma_rn(P.cy, sy, acc);
  return acc;
}

// laplacian() of diffusion.cpp:34-55 with periodic neighbours (reference mode)
__device__ __forceinline__ double periodic_point(const ProbDev& P, const double* __restrict__ u,
                                                 long long i, long long j)
{
  const long long nx = P.nx, ny = P.ny;
  const long long iw = (i == 0) ? nx - 1 : i - 1, ie = (i == nx - 1) ? 0 : i + 1;
  const long long js = (j == 0) ? ny - 1 : j - 1, jn = (j == ny - 1) ? 0 : j + 1;
  const double Dxw = P.Dxw[i], Dxe = P.Dxe[i], Dys = P.Dys[j], Dyn = P.Dyn[j];
  double v = -((Dxw + Dxe) + (Dys + Dyn)) * u[j * nx + i];
  v        = v + Dxw * u[j * nx + iw];
  v        = v + Dxe * u[j * nx + ie];
  v        = v + Dys * u[js * nx + i];
  v        = v + Dyn * u[jn * nx + i];
  return v;
}

__device__ __forceinline__ double add_forcing(const ProbDev& P, double al, double be, double ga,
                                              long long i, long long j, double acc)
{
  const double Pi = __fma_rn(al, P.Sx[i], be * P.Sxx[i]);
  const double Qi = ga * P.Sx[i];
  acc             = __fma_rn(P.Sy[j], Pi, acc);
  acc             = __fma_rn(P.Syy[j], Qi, acc);
  return acc;
}

// Mixed stage at one point, difference form (header comment): d_C and its four neighbours
// of d_{j-1}, m2 = d_{j-2} (0 at stage 2), q0 = FP32 F_0, and the forcing products
// syj * pi + syyj * qi of hm (b_j - b_0) (FORCED only). The same operations in the same order
// as the oracle's stage32.
template <bool FORCED>
__device__ __forceinline__ float mixed_point(float gs, float gx, float gy, float gm, float gF, float dc, float dw,
                                             float de, float ds, float dn, float m2, float q0, float syj,
                                             float pi, float syyj, float qi)
{
  const float lx = __fadd_rn(__fsub_rn(dw, dc), __fsub_rn(de, dc));
  const float ly = __fadd_rn(__fsub_rn(ds, dc), __fsub_rn(dn, dc));
  float inc      = __fmul_rn(gs, dc);
  inc            = __fmaf_rn(gx, lx, inc);
  inc            = __fmaf_rn(gy, ly, inc);
  inc            = __fmaf_rn(gm, __fsub_rn(dc, m2), inc);
  inc            = __fmaf_rn(gF, q0, inc);
  if (FORCED)
  {
    inc = __fmaf_rn(syj, pi, inc);
    inc = __fmaf_rn(syyj, qi, inc);
  }
  return __fadd_rn(dc, inc);
}

// mixed_point on two points at once with the paired FP32 instructions of sm_100 and later
// (__fadd2_rn, __fmul2_rn, __ffma2_rn: per component the same rounding as __fadd_rn,
// __fmul_rn, __fmaf_rn). A difference a - b is taken as a + (-b), which IEEE arithmetic gives
// exactly, signed zeros included; the negations are multiplications by -1 (exact). The two
// components are bit-identical to two mixed_point calls. Operands are (point 0, point 1)
// pairs; the scalars arrive duplicated.
template <bool FORCED>
__device__ __forceinline__ float2 mixed_pair(float2 gs, float2 gx, float2 gy, float2 gm, float2 gF, float2 dc,
                                             float2 dw, float2 de, float2 ds, float2 dn, float2 m2, float2 q0,
                                             float2 syj, float2 pi, float2 syyj, float2 qi)
{
  const float2 neg1 = make_float2(-1.0f, -1.0f);
  const float2 ndc  = __fmul2_rn(dc, neg1);
  const float2 lx   = __fadd2_rn(__fadd2_rn(dw, ndc), __fadd2_rn(de, ndc));
  const float2 ly   = __fadd2_rn(__fadd2_rn(ds, ndc), __fadd2_rn(dn, ndc));
  float2 inc        = __fmul2_rn(gs, dc);
  inc               = __ffma2_rn(gx, lx, inc);
  inc               = __ffma2_rn(gy, ly, inc);
  inc               = __ffma2_rn(gm, __fadd2_rn(dc, __fmul2_rn(m2, neg1)), inc);
  inc               = __ffma2_rn(gF, q0, inc);
  if (FORCED)
  {
    inc = __ffma2_rn(syj, pi, inc);
    inc = __ffma2_rn(syyj, qi, inc);
  }
  return __fadd2_rn(dc, inc);
}

// Error weight of the mixed form's step end, 1 / (rtol |y| + atol) to within a few ulp with five
// FP64-pipe operations instead of a correctly rounded division (about ten on GB300, whose FP64
// pipe bounds this kernel): den = fma(rtol, |y|, atol), the correctly rounded FP32 reciprocal of
// the FP32-rounded den as the seed, one Newton step in FP64 (relative error below 1e-14). A den
// outside [2^-120, 2^120] takes the division. The oracle's step end restates it.
__device__ __forceinline__ double mixed_weight(double rtol, double atol, double y)
{
  const double den = __fma_rn(rtol, fabs(y), atol);
  // den in [2^-120, 2^120], decided on the bit pattern: for doubles with the sign bit clear the
  // order of the bit patterns as signed integers is the order of the values, and every
  // negative value, zero, infinity and NaN falls outside the range exactly as with the two
  // floating-point comparisons (which would take the FP64 pipe)
  const long long u = __double_as_longlong(den);
  if (u >= 0x3870000000000000LL && u <= 0x4770000000000000LL)
  {
    const double r0 = (double)__frcp_rn(__double2float_rn(den));
    const double e1 = __fma_rn(-den, r0, 1.0);
    return __fma_rn(r0, e1, r0);
  }
  return 1.0 / den;
}

// ---------------------------------------------------------------------------------------
// vector load/store helpers
// ---------------------------------------------------------------------------------------
template <typename T, int V>
struct VecIO;
template <>
struct VecIO<double, 1> {
  static __device__ __forceinline__ void ld(const double* p, double (&v)[1]) { v[0] = __ldg(p); }
  static __device__ __forceinline__ void st(double* p, const double (&v)[1]) { p[0] = v[0]; }
};
template <>
struct VecIO<double, 2> {
  static __device__ __forceinline__ void ld(const double* p, double (&v)[2])
  {
    double2 t = __ldg(reinterpret_cast<const double2*>(p));
    v[0]      = t.x;
    v[1]      = t.y;
  }
  static __device__ __forceinline__ void st(double* p, const double (&v)[2])
  {
    *reinterpret_cast<double2*>(p) = make_double2(v[0], v[1]);
  }
};
template <>
struct VecIO<float, 1> {
  static __device__ __forceinline__ void ld(const float* p, float (&v)[1]) { v[0] = __ldg(p); }
  static __device__ __forceinline__ void st(float* p, const float (&v)[1]) { p[0] = v[0]; }
};
template <>
struct VecIO<float, 4> {
  static __device__ __forceinline__ void ld(const float* p, float (&v)[4])
  {
    float4 t = __ldg(reinterpret_cast<const float4*>(p));
    v[0]     = t.x;
    v[1]     = t.y;
    v[2]     = t.z;
    v[3]     = t.w;
  }
  static __device__ __forceinline__ void st(float* p, const float (&v)[4])
  {
    *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
  }
};

// ---------------------------------------------------------------------------------------
// FP64 stage kernel, Y form. Each thread owns VEC consecutive columns and marches down RY
// rows keeping rows j-1, j, j+1 of Y_{j-1} in registers; W/E neighbours at the thread's
// edge come through L1. One read of each input stream, one write of Y_j.
// ---------------------------------------------------------------------------------------
template <int VEC, int RY, bool FORCED>
__global__ void __launch_bounds__(256) stage64_kernel(ProbDev P, const StageArgs* __restrict__ A,
                                                      const double* __restrict__ ym1,
                                                      const double* __restrict__ ym2,
                                                      const double* __restrict__ y0,
                                                      const double* __restrict__ f0,
                                                      double* __restrict__ yj)
{
  using IO           = VecIO<double, VEC>;
  const long long nx = P.nx, ny = P.ny;
  const long long i0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) * VEC;
  const long long jb = ((long long)blockIdx.y * blockDim.y + threadIdx.y) * RY;
  if (i0 >= nx || jb >= ny) return;
  const long long je = (jb + RY < ny) ? jb + RY : ny;
  // the thread's VEC-wide loads and stores stay inside the row
  if (!STS_IN_BOUNDS(i0 + VEC <= nx && i0 % VEC == 0, P.err)) return;
  const double gc = A->gc, gx = A->gx, gy = A->gy, gn = A->gn, g0 = A->g0, gf = A->gf;
  double Pi[VEC], Qi[VEC];
  if (FORCED)
  {
    const double al = A->al, be = A->be, ga = A->ga;
#pragma unroll
    for (int v = 0; v < VEC; ++v)
    {
      Pi[v] = __fma_rn(al, P.Sx[i0 + v], be * P.Sxx[i0 + v]);
      Qi[v] = ga * P.Sx[i0 + v];
    }
  }
  double up[VEC], cur[VEC], dn[VEC];
  if (jb > 0) IO::ld(ym1 + (jb - 1) * nx + i0, up);
  else
#pragma unroll
    for (int v = 0; v < VEC; ++v) up[v] = 0.0;
  IO::ld(ym1 + jb * nx + i0, cur);
  for (long long j = jb; j < je; ++j)
  {
    const long long row = j * nx + i0;
    if (j + 1 < ny) IO::ld(ym1 + row + nx, dn);
    else
#pragma unroll
      for (int v = 0; v < VEC; ++v) dn[v] = 0.0;
    const double w = (i0 > 0) ? __ldg(ym1 + row - 1) : 0.0;
    const double e = (i0 + VEC < nx) ? __ldg(ym1 + row + VEC) : 0.0;
    double m2[VEC], z0[VEC], q0[VEC], out[VEC];
    IO::ld(ym2 + row, m2);
    IO::ld(y0 + row, z0);
    IO::ld(f0 + row, q0);
    double syj = 0.0, syyj = 0.0;
    if (FORCED)
    {
      syj  = __ldg(P.Sy + j);
      syyj = __ldg(P.Syy + j);
    }
#pragma unroll
    for (int v = 0; v < VEC; ++v)
    {
      const double uw = (v == 0) ? w : cur[v - 1];
      const double ue = (v == VEC - 1) ? e : cur[v + 1];
      const double sx = uw + ue, sy = up[v] + dn[v];
      double acc      = gc * cur[v];
      acc             = __fma_rn(gx, sx, acc);
      acc             = __fma_rn(gy, sy, acc);
      acc             = __fma_rn(gn, m2[v], acc);
      acc             = __fma_rn(g0, z0[v], acc);
      acc             = __fma_rn(gf, q0[v], acc);
      if (FORCED)
      {
        acc = __fma_rn(syj, Pi[v], acc);
        acc = __fma_rn(syyj, Qi[v], acc);
      }
      out[v] = acc;
    }
    IO::st(yj + row, out);
#pragma unroll
    for (int v = 0; v < VEC; ++v)
    {
      up[v]  = cur[v];
      cur[v] = dn[v];
    }
  }
}

// Mixed stage kernel: FP32 increments d_j = Y_j - Y_0.
template <int VEC, int RY, bool FORCED, bool HAS_M2>
__global__ void __launch_bounds__(256) stage32_kernel(ProbDev P, const StageArgs* __restrict__ A,
                                                      const float* __restrict__ dm1,
                                                      const float* __restrict__ dm2,
                                                      const float* __restrict__ f0f,
                                                      float* __restrict__ dj)
{
  using IO           = VecIO<float, VEC>;
  const long long nx = P.nx, ny = P.ny;
  const long long i0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) * VEC;
  const long long jb = ((long long)blockIdx.y * blockDim.y + threadIdx.y) * RY;
  if (i0 >= nx || jb >= ny) return;
  const long long je = (jb + RY < ny) ? jb + RY : ny;
  if (!STS_IN_BOUNDS(i0 + VEC <= nx && i0 % VEC == 0, P.err)) return;
  const float gs = A->gsf, gx = A->gxf, gy = A->gyf, gm = A->gmf, gF = A->gFf;
  float Pi[VEC], Qi[VEC];
#pragma unroll
  for (int v = 0; v < VEC; ++v) Pi[v] = Qi[v] = 0.0f;
  if (FORCED)
  {
    const float al = A->alf, be = A->bef, ga = A->gaf;
#pragma unroll
    for (int v = 0; v < VEC; ++v)
    {
      Pi[v] = __fmaf_rn(al, P.Sxf[i0 + v], be * P.Sxxf[i0 + v]);
      Qi[v] = ga * P.Sxf[i0 + v];
    }
  }
  float up[VEC], cur[VEC], dn[VEC];
  if (jb > 0) IO::ld(dm1 + (jb - 1) * nx + i0, up);
  else
#pragma unroll
    for (int v = 0; v < VEC; ++v) up[v] = 0.0f;
  IO::ld(dm1 + jb * nx + i0, cur);
  for (long long j = jb; j < je; ++j)
  {
    const long long row = j * nx + i0;
    if (j + 1 < ny) IO::ld(dm1 + row + nx, dn);
    else
#pragma unroll
      for (int v = 0; v < VEC; ++v) dn[v] = 0.0f;
    const float w = (i0 > 0) ? __ldg(dm1 + row - 1) : 0.0f;
    const float e = (i0 + VEC < nx) ? __ldg(dm1 + row + VEC) : 0.0f;
    float m2[VEC], q0[VEC], out[VEC];
    if (HAS_M2) IO::ld(dm2 + row, m2);
    else
#pragma unroll
      for (int v = 0; v < VEC; ++v) m2[v] = 0.0f;
    IO::ld(f0f + row, q0);
    float syj = 0.0f, syyj = 0.0f;
    if (FORCED)
    {
      syj  = __ldg(P.Syf + j);
      syyj = __ldg(P.Syyf + j);
    }
#pragma unroll
    for (int v = 0; v < VEC; ++v)
    {
      const float uw = (v == 0) ? w : cur[v - 1];
      const float ue = (v == VEC - 1) ? e : cur[v + 1];
      out[v] = mixed_point<FORCED>(gs, gx, gy, gm, gF, cur[v], uw, ue, up[v], dn[v], m2[v], q0[v], syj, Pi[v],
                                   syyj, Qi[v]);
    }
    IO::st(dj + row, out);
#pragma unroll
    for (int v = 0; v < VEC; ++v)
    {
      up[v]  = cur[v];
      cur[v] = dn[v];
    }
  }
}

// stage 1: Y_1 = Y_0 + hm1 F_0 (FP64) / d_1 = hm1 F_0 (FP32)
static __global__ void __launch_bounds__(256) stage1_64_kernel(long long n, const StepArgs* __restrict__ S,
                                                        const double* __restrict__ y0,
                                                        const double* __restrict__ f0,
                                                        double* __restrict__ y1)
{
  const double hm1       = S->hm1;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += stride)
    y1[k] = __fma_rn(hm1, f0[k], y0[k]);
}

static __global__ void __launch_bounds__(256) stage1_32_kernel(long long n, const StepArgs* __restrict__ S,
                                                        const float* __restrict__ f0f,
                                                        float* __restrict__ d1)
{
  const float hm1        = S->hm1f;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += stride)
    d1[k] = hm1 * f0f[k];
}

// ---------------------------------------------------------------------------------------
// Step end. Fnew = F(t+h, ynew); err = 0.8 (yn - ynew) + 0.4 h (Fn + Fnew);
// dsm = sqrt(sum (err/(rtol |yn| + atol))^2 / N) with the exact accumulator.
// MIXED: ynew = yn + (double) ds is formed on the fly (also at the stencil neighbours) and
// written out together with Fnew and its FP32 copy; yn - ynew is taken as -ds and the weight
// comes from mixed_weight.
// Grid: blockDim.x columns per block, blocks stride over rows.
// ---------------------------------------------------------------------------------------
template <bool MIXED, bool FORCED>
__global__ void __launch_bounds__(256) stepend_kernel(ProbDev P, const StepArgs* __restrict__ S,
                                                      const double* __restrict__ yn,
                                                      const double* __restrict__ Ys,
                                                      const float* __restrict__ ds,
                                                      const double* __restrict__ Fn,
                                                      double* __restrict__ ynew,
                                                      double* __restrict__ Fnew,
                                                      float* __restrict__ Fnewf, RedWork* w,
                                                      double* slot)
{
  const long long nx = P.nx, ny = P.ny;
  const long long i  = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const double p4h = S->p4h, rtol = S->rtol, atol = S->atol;
  const double al = S->al, be = S->be, ga = S->ga;
  xsum::Limbs acc;
  xsum::zero(acc);
  unsigned flags = 0;
  if (i < nx)
  {
    double Pi = 0.0, Qi = 0.0;
    if (FORCED)
    {
      Pi = __fma_rn(al, P.Sx[i], be * P.Sxx[i]);
      Qi = ga * P.Sx[i];
    }
    for (long long j = blockIdx.y; j < ny; j += gridDim.y)
    {
      const long long k = j * nx + i;
      double uc, uw, ue, us, un;
      if (MIXED)
      {
        uc = yn[k] + (double)ds[k];
        uw = (i > 0) ? yn[k - 1] + (double)ds[k - 1] : 0.0;
        ue = (i < nx - 1) ? yn[k + 1] + (double)ds[k + 1] : 0.0;
        us = (j > 0) ? yn[k - nx] + (double)ds[k - nx] : 0.0;
        un = (j < ny - 1) ? yn[k + nx] + (double)ds[k + nx] : 0.0;
      }
      else
      {
        uc = Ys[k];
        uw = (i > 0) ? Ys[k - 1] : 0.0;
        ue = (i < nx - 1) ? Ys[k + 1] : 0.0;
        us = (j > 0) ? Ys[k - nx] : 0.0;
        un = (j < ny - 1) ? Ys[k + nx] : 0.0;
      }
      const double sx = uw + ue, sy = us + un;
      double f        = P.cc * uc;
      f               = __fma_rn(P.cx, sx, f);
      f               = __fma_rn(P.cy, sy, f);
      if (FORCED)
      {
        f = __fma_rn(P.Sy[j], Pi, f);
        f = __fma_rn(P.Syy[j], Qi, f);
      }
      Fnew[k] = f;
      if (MIXED)
      {
        ynew[k]  = uc;
        Fnewf[k] = (float)f;
      }
      const double y = yn[k];
      // the mixed form takes y_n - y_{n+1} as -d_s itself (exact) and the fast weight
      const double d = MIXED ? -(double)ds[k] : y - uc;
      double e       = 0.8 * d;
      e              = __fma_rn(p4h, Fn[k], e);
      e              = __fma_rn(p4h, f, e);
      const double wt = MIXED ? mixed_weight(rtol, atol, y) : 1.0 / (rtol * fabs(y) + atol);
      const double x  = e * wt;
      xsum::add(acc, x * x, flags);
    }
  }
  xsum_block_finish<256>(acc, flags, w, slot, 1, (double)(nx * ny));
}

// Step end, row-marching form (nx even): a thread owns 2 consecutive columns and 16 rows,
// keeps rows j-1, j, j+1 of y_{n+1} in registers (formed once per point, yn + ds in the
// mixed form), and gets the west/east neighbours from the neighbouring lanes; per point the
// arithmetic is identical to stepend_kernel.
template <bool MIXED, bool FORCED>
__global__ void __launch_bounds__(256) stepend_march_kernel(ProbDev P, const StepArgs* __restrict__ S,
                                                            const double* __restrict__ yn,
                                                            const double* __restrict__ Ys,
                                                            const float* __restrict__ ds,
                                                            const double* __restrict__ Fn,
                                                            double* __restrict__ ynew,
                                                            double* __restrict__ Fnew,
                                                            float* __restrict__ Fnewf, RedWork* w,
                                                            double* slot)
{
  constexpr int RYS = 16;
  const long long nx = P.nx, ny = P.ny;
  const long long i0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) * 2;
  const long long jb = ((long long)blockIdx.y * blockDim.y + threadIdx.y) * RYS;
  const int lane     = threadIdx.x & 31;
  const double p4h = S->p4h, rtol = S->rtol, atol = S->atol;
  xsum::Limbs acc;
  xsum::zero(acc);
  unsigned flags   = 0;
  const bool colok = i0 < nx; // nx even: both columns valid
  // no early return here: the block reduction below has barriers
  const bool active = colok && jb < ny && STS_IN_BOUNDS(i0 + 2 <= nx, P.err);
  // y_{n+1} at (row, i0..i0+1); zero outside the domain
  auto row2 = [&](long long j, double (&v)[2]) {
    if (!active || j < 0 || j >= ny)
    {
      v[0] = v[1] = 0.0;
      return;
    }
    const long long k = j * nx + i0;
    if (MIXED)
    {
      const double2 a = __ldg(reinterpret_cast<const double2*>(yn + k));
      const float2 b  = __ldg(reinterpret_cast<const float2*>(ds + k));
      v[0]            = a.x + (double)b.x;
      v[1]            = a.y + (double)b.y;
    }
    else
    {
      const double2 a = __ldg(reinterpret_cast<const double2*>(Ys + k));
      v[0]            = a.x;
      v[1]            = a.y;
    }
  };
  auto point = [&](long long j, long long i) -> double { // single y_{n+1} value (edges)
    if (i < 0 || i >= nx || j < 0 || j >= ny) return 0.0;
    const long long k = j * nx + i;
    return MIXED ? yn[k] + (double)ds[k] : Ys[k];
  };
  double Pi[2] = {0.0, 0.0}, Qi[2] = {0.0, 0.0};
  if (FORCED && colok)
  {
    const double al = S->al, be = S->be, ga = S->ga;
#pragma unroll
    for (int v = 0; v < 2; ++v)
    {
      Pi[v] = __fma_rn(al, P.Sx[i0 + v], be * P.Sxx[i0 + v]);
      Qi[v] = ga * P.Sx[i0 + v];
    }
  }
  double up[2], cur[2], dn[2];
  row2(jb - 1, up);
  row2(jb, cur);
  for (int r = 0; r < RYS; ++r)
  {
    const long long j = jb + r;
    row2(j + 1, dn);
    // west/east neighbours from the neighbouring lanes (the warp spans 64 consecutive columns)
    double wv = __shfl_up_sync(0xffffffffu, cur[1], 1);
    double ev = __shfl_down_sync(0xffffffffu, cur[0], 1);
    if (lane == 0) wv = active && j < ny ? point(j, i0 - 1) : 0.0;
    if (lane == 31) ev = active && j < ny ? point(j, i0 + 2) : 0.0;
    if (active && j < ny)
    {
      if (i0 + 2 >= nx) ev = 0.0;
      if (i0 == 0) wv = 0.0;
      const long long k = j * nx + i0;
      const double2 ynv = __ldg(reinterpret_cast<const double2*>(yn + k));
      const double2 fnv = __ldg(reinterpret_cast<const double2*>(Fn + k));
      const double yv[2] = {ynv.x, ynv.y}, fv[2] = {fnv.x, fnv.y};
      float dsv[2] = {0.f, 0.f};
      if (MIXED)
      {
        const float2 t = __ldg(reinterpret_cast<const float2*>(ds + k));
        dsv[0]         = t.x;
        dsv[1]         = t.y;
      }
      double syj = 0.0, syyj = 0.0;
      if (FORCED)
      {
        syj  = P.Sy[j];
        syyj = P.Syy[j];
      }
      double fo[2];
#pragma unroll
      for (int v = 0; v < 2; ++v)
      {
        const double uc = cur[v];
        const double uw = (v == 0) ? wv : cur[0];
        const double ue = (v == 1) ? ev : cur[1];
        const double sx = uw + ue, sy = up[v] + dn[v];
        double f        = P.cc * uc;
        f               = __fma_rn(P.cx, sx, f);
        f               = __fma_rn(P.cy, sy, f);
        if (FORCED)
        {
          f = __fma_rn(syj, Pi[v], f);
          f = __fma_rn(syyj, Qi[v], f);
        }
        fo[v]           = f;
        const double d  = MIXED ? -(double)dsv[v] : yv[v] - uc;
        double e        = 0.8 * d;
        e               = __fma_rn(p4h, fv[v], e);
        e               = __fma_rn(p4h, f, e);
        const double wt = MIXED ? mixed_weight(rtol, atol, yv[v]) : 1.0 / (rtol * fabs(yv[v]) + atol);
        const double x  = e * wt;
        xsum::add(acc, x * x, flags);
      }
      *reinterpret_cast<double2*>(Fnew + k) = make_double2(fo[0], fo[1]);
      if (MIXED)
      {
        *reinterpret_cast<double2*>(ynew + k) = make_double2(cur[0], cur[1]);
        *reinterpret_cast<float2*>(Fnewf + k) = make_float2((float)fo[0], (float)fo[1]);
      }
    }
#pragma unroll
    for (int v = 0; v < 2; ++v)
    {
      up[v]  = cur[v];
      cur[v] = dn[v];
    }
  }
  xsum_block_finish<256>(acc, flags, w, slot, 1, (double)(nx * ny));
}

// WRMS with ewt(y): mode 0 -> x = a w(y), mode 1 -> x = (a - b) w(y)
template <int MODE>
__global__ void __launch_bounds__(256) wrms_ewt_kernel(long long n, const double* __restrict__ a,
                                                       const double* __restrict__ b,
                                                       const double* __restrict__ y, double rtol,
                                                       double atol, RedWork* w, double* slot)
{
  xsum::Limbs acc;
  xsum::zero(acc);
  unsigned flags         = 0;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += stride)
  {
    const double wt = 1.0 / (rtol * fabs(y[k]) + atol);
    const double v  = (MODE == 0) ? a[k] : (a[k] - b[k]);
    const double x  = v * wt;
    xsum::add(acc, x * x, flags);
  }
  xsum_block_finish<256>(acc, flags, w, slot, 1, (double)n);
}

// exact reductions: mode 0 = sum x*y, 1 = sum (x*w)^2 -> sqrt(./n)
template <int MODE>
__global__ void __launch_bounds__(256) xred_kernel(long long n, const double* __restrict__ x,
                                                   const double* __restrict__ y, RedWork* w,
                                                   double* slot)
{
  xsum::Limbs acc;
  xsum::zero(acc);
  unsigned flags         = 0;
  const long long stride = (long long)gridDim.x * blockDim.x;
  auto term = [&](long long k) -> double {
    if constexpr (MODE == 0) return __dmul_rn(x[k], y[k]);
    const double q = __dmul_rn(x[k], y[k]);
    return __dmul_rn(q, q);
  };
  // two terms per trip with both loads issued before the integer accumulation (1.3x on
  // fields larger than L2); the exact sum does not depend on the order
  long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  for (; k + stride < n; k += 2 * stride)
  {
    const double v0 = term(k), v1 = term(k + stride);
    xsum::add(acc, v0, flags);
    xsum::add(acc, v1, flags);
  }
  if (k < n) xsum::add(acc, term(k), flags);
  xsum_block_finish<256>(acc, flags, w, slot, MODE, (double)n);
}
