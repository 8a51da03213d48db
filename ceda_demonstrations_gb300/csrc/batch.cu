// Batched STS: many independent 2-D heat problems (homogeneous Dirichlet, no forcing, their
// own grid size and diffusivities) advanced to a common final time in ONE persistent launch.
//
// Work distribution: instances are ordered by an estimate of their cost (largest first) and
// CTAs take the next instance from a device-side counter. A CTA integrates its instance
// completely: RKL2/RKC2 stages as grid sweeps separated by __syncthreads, the step end
// (F(y_{n+1}), embedded error, exact WRMS reduced inside the CTA) and the step control
// (controller, stage cap, stop time, rejections) run on the device with the rules of the
// single-problem integrator (lsrk.cu). No host round trip happens per step; the host only
// launches the batch and reads the per-instance statistics afterwards.
//
// Precision: FP64 throughout (the path is FP64-ALU-bound on GB300). Every step decision uses
// the arithmetic of the single-problem integrator and the CPU oracle: stage coefficients from
// the host's table, IEEE sqrt/divide, and the deterministic pow of portable_math.cuh in the
// controller, so each instance follows the oracle's step sequence and matches it bit for bit.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#include "kernels.cuh"
#include "portable_math.cuh"
#include "sts_internal.cuh"

struct BatchInst {
  int n;           // interior nodes per direction
  int status;      // 0 running/finished ok, < 0 failure
  long long off;   // offset of the instance in each state array
  double kx, ky, cx, cy, cc, rho;
  // statistics
  long long nst, nst_att, netf, nfe, nst_exp, stage_max, stages_total;
  double t, hlast, hnext;
};

struct BatchArrays {
  double* y;    // state y_n (input and output)
  double* buf[5]; // F_n, F_{n+1} / Y work buffers (instance-local regions)
};

// Stage coefficients come from a table the host fills with STS_LSRKStageCoeffs for every
// stage count 2..smax (the single-problem integrator's and the oracle's values, bit for bit):
// entry (s, j) = {mu_j, nu_j, mus_j, a_{j-1}}.
struct CoefT {
  double mu, nu, mus, ajm1;
};

struct BatchParams {
  double tf, rtol, atol, eig_safety;
  int method, smax, controller, maxsteps;
  const void* coef; // CoefT table [(smax + 1) x (smax + 1)]
  int mixed;        // 1: FP32 stage increments relative to the FP64 step start
  int pad_;
};

struct STS_Batch_ {
  STS_Context ctx = nullptr;
  int ninst       = 0;
  long long total = 0;
  std::vector<BatchInst> hinst;
  BatchInst* dinst = nullptr;
  int* dorder      = nullptr;
  int* dqueue      = nullptr;
  double* y        = nullptr;
  double* work     = nullptr; // 6 x total
  int block        = 512;
  int ctas_per_sm  = 2;
  double last_ms   = 0.0;
  CoefT* dcoef     = nullptr; // stage-coefficient table of (coef_method, coef_smax)
  int coef_method = -1, coef_smax = -1;
  int mixed        = 0; // FP32 stage increments (STS_BatchSetMixed)
  // instances with n >= big_n run on clusters of `cluster` CTAs (1: all on single CTAs)
  int cluster      = 1;
  int big_n        = 256;
  int nbig         = 0;
  double big_share = 0.0;      // estimated cost share of the clustered group
  int* dorder_big   = nullptr; // cost-ordered indices of each group
  int* dorder_small = nullptr;
  cudaStream_t side = nullptr; // second stream for the single-CTA group
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  std::vector<double> cost;
};

// ---------------------------------------------------------------------------------------
// device helpers
// ---------------------------------------------------------------------------------------
namespace {

constexpr double B_ORD = 3.0, B_BIAS = 1.5, B_TINY = 1.0e-10;
constexpr double B_SAFETY = 0.96, B_GROWTH = 20.0, B_ETAMX1 = 10000.0, B_ETAMXF = 0.3, B_ETAMIN = 0.1;

// hp: previous accepted step size (implicit Gustafsson controller); the host integrator's rules
__device__ double d_controller(int controller, double h, double dsm, double ep1, double ep2, double hp,
                               long long nhist)
{
  double e1 = fmax(B_BIAS * dsm, B_TINY), e2 = fmax(B_BIAS * ep1, B_TINY), e3 = fmax(B_BIAS * ep2, B_TINY);
  if (controller == 0)
  {
    if (nhist < 1) return h * stsm::pow(e1, -0.58 / B_ORD);
    if (nhist < 2) return h * stsm::pow(e1, -0.58 / B_ORD) * stsm::pow(e2, 0.21 / B_ORD);
    return h * stsm::pow(e1, -0.58 / B_ORD) * stsm::pow(e2, 0.21 / B_ORD) * stsm::pow(e3, -0.1 / B_ORD);
  }
  if (controller == 1)
  {
    if (nhist < 1) return h * stsm::pow(e1, -0.8 / B_ORD);
    return h * stsm::pow(e1, -0.8 / B_ORD) * stsm::pow(e2, 0.31 / B_ORD);
  }
  if (controller >= 3 && controller <= 5 && nhist >= 1 && hp > 0.0)
  { // Gustafsson: explicit (3), implicit (4), the smaller of the two (5)
    const double r    = e1 / e2;
    const double hexp = h * stsm::pow(e1, -0.367 / B_ORD) * stsm::pow(r, -0.268 / B_ORD);
    if (controller == 3) return hexp;
    const double himp = h * (h / hp) * stsm::pow(e1, -0.98 / B_ORD) * stsm::pow(r, -0.95 / B_ORD);
    if (controller == 4) return himp;
    return hexp < himp ? hexp : himp;
  }
  return h * stsm::pow(e1, -1.0 / B_ORD);
}

// The controller evaluated by one thread of the CTA and broadcast through shared memory: every
// thread holds the same inputs, so the value is the one each thread would compute (and every
// CTA of a cluster computes it from the same reduced values), without 256-512 redundant
// evaluations of the FP64 pow series per step. Called by all threads of the CTA.
__device__ __forceinline__ double block_control(int controller, double h, double dsm, double ep1, double ep2,
                                                double hp, long long nhist, double* shn)
{
  if (threadIdx.x == 0) *shn = d_controller(controller, h, dsm, ep1, ep2, hp, nhist);
  __syncthreads();
  const double v = *shn;
  __syncthreads(); // read by every thread before the next proposal overwrites it
  return v;
}

__device__ int d_stages(int method, double h, double rho, int smax, double* hmax)
{
  double ss;
  const double sm = (double)smax;
  if (method == 0)
  {
    ss    = 1.0 + floor(sqrt(1.0 + 1.54 * h * rho));
    *hmax = (rho > 0.0) ? 0.96 * (sm * sm - 1.0) / (1.54 * rho) : 1e300;
  }
  else
  {
    ss    = ceil((sqrt(9.0 + 8.0 * h * rho) - 1.0) / 2.0);
    *hmax = (rho > 0.0) ? 0.96 * (sm * sm + sm - 2.0) / (2.0 * rho) : 1e300;
  }
  // a non-finite step (NaN state) gives the 2-stage minimum, as max(ss, 2) does
  if (!(ss >= 2.0)) ss = 2.0;
  if (ss > 1e9) ss = 1e9;
  return (int)ss;
}

// Barrier over the CTAs that share an instance: the whole thread-block cluster (barrier.cluster
// with release/acquire semantics, so the other CTAs' global stores of the previous sweep are
// visible), or the CTA when an instance has one CTA.
template <int CL>
__device__ __forceinline__ void inst_sync()
{
  if constexpr (CL > 1) cooperative_groups::this_cluster().sync();
  else __syncthreads();
}

// Exact sum over all threads of the instance's CTAs, returned to every thread. Each CTA
// combines its threads' limbs (warp shuffles + shared memory) into climb[]; with a cluster,
// every CTA then reads all CTAs' climb[] through distributed shared memory and adds them in
// rank order, so all CTAs obtain the same integer and the same rounded value.
template <int NT, int CL>
__device__ double inst_exact_sum(xsum::Limbs& a, unsigned flags, long long (*sm)[xsum::NL], long long* climb,
                                 unsigned* cflags, double* sres)
{
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) *cflags = 0;
#pragma unroll
  for (int k = 0; k < xsum::NL; ++k)
  {
    long long v = a.l[k];
#pragma unroll
    for (int m = 16; m >= 1; m >>= 1) v += shfl_xor_ll(v, m);
    if (lane == 0) sm[warp][k] = v;
  }
  __syncthreads();
  if (flags) atomicOr(cflags, flags);
  if (tid < xsum::NL)
  {
    long long v = 0;
    for (int w = 0; w < NT / 32; ++w) v += sm[w][tid];
    climb[tid] = v;
  }
  inst_sync<CL>(); // climb[] and cflags of every CTA complete
  if (tid == 0)
  {
    long long tot[xsum::NL];
    unsigned fl = 0;
    if constexpr (CL > 1)
    {
      cooperative_groups::cluster_group cl = cooperative_groups::this_cluster();
      for (int k = 0; k < xsum::NL; ++k) tot[k] = 0;
      for (int r = 0; r < CL; ++r)
      {
        const long long* rl = cl.map_shared_rank(climb, r);
        for (int k = 0; k < xsum::NL; ++k) tot[k] += rl[k];
        fl |= *cl.map_shared_rank(cflags, r);
      }
    }
    else
    {
      for (int k = 0; k < xsum::NL; ++k) tot[k] = climb[k];
      fl = *cflags;
    }
    *sres = xsum::finalize(tot, fl);
  }
  inst_sync<CL>(); // every CTA has read the others' climb[] before they are reused
  return *sres;
}

// Stencil-row load: rows owned by another CTA of the cluster are read through L2 (ld.cg),
// so no stale L1 line of an earlier sweep is used.
__device__ __forceinline__ double ldrow(const double* p, bool foreign) { return foreign ? __ldcg(p) : *p; }
__device__ __forceinline__ float ldrowf(const float* p, bool foreign) { return foreign ? __ldcg(p) : *p; }

__device__ __forceinline__ double lap(const double* __restrict__ u, int n, int i, int j, int j0, int j1, double cx,
                                      double cy, double cc)
{
  const long long k = (long long)j * n + i;
  const double uc = u[k];
  const double uw = (i > 0) ? u[k - 1] : 0.0;
  const double ue = (i < n - 1) ? u[k + 1] : 0.0;
  const double us = (j > 0) ? ldrow(&u[k - n], j - 1 < j0) : 0.0;
  const double un = (j < n - 1) ? ldrow(&u[k + n], j + 1 >= j1) : 0.0;
  const double sx = uw + ue, sy = us + un;
  double acc      = cc * uc;
  acc             = __fma_rn(cx, sx, acc);
  acc             = __fma_rn(cy, sy, acc);
  return acc;
}

// CL CTAs (a thread-block cluster when CL > 1) integrate one instance together: CTA `rank`
// owns rows [j0, j1) of every sweep; sweeps are separated by cluster barriers and the exact
// reductions are combined through distributed shared memory. Every CTA of the cluster
// evaluates the step control from the same reduced values, so all take the same decisions.
template <int NT, int CL, bool MIXED>
__global__ void __launch_bounds__(NT, 1024 / NT) batch_kernel(BatchInst* __restrict__ insts, const int* __restrict__ order,
                                                   int ninst, int* queue, double* __restrict__ yall,
                                                   double* __restrict__ work, long long total, BatchParams prm)
{
  __shared__ long long sm[NT / 32][xsum::NL];
  __shared__ long long climb[xsum::NL];
  __shared__ unsigned sflags;
  __shared__ double sres;
  __shared__ double shn; // step-size proposal of the controller, computed by one thread
  __shared__ int sidx;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  constexpr int NW = NT / 32;
  int rank = 0;
  if constexpr (CL > 1) rank = (int)cooperative_groups::this_cluster().block_rank();

  for (;;)
  {
    if (rank == 0 && tid == 0) sidx = atomicAdd(queue, 1);
    inst_sync<CL>();
    int idx = sidx;
    if constexpr (CL > 1) idx = *cooperative_groups::this_cluster().map_shared_rank(&sidx, 0);
    inst_sync<CL>(); // every CTA has read the index before rank 0 fetches the next one
    if (idx >= ninst) break;
    BatchInst& I = insts[order[idx]];
    const int n = I.n;
    const int j0 = (int)((long long)n * rank / CL), j1 = (int)((long long)n * (rank + 1) / CL);
    const long long N = (long long)n * n;
#ifdef STS_DEBUG_BOUNDS
    // the instance's region lies inside the state arrays and every CTA of the cluster owns rows
    if (I.off < 0 || I.off + N > total || n < CL)
    {
      if (rank == 0 && tid == 0) I.status = -5;
      continue;
    }
#endif
    const double cx = I.cx, cy = I.cy, cc = I.cc, rho = I.rho;
    // seven instance-local regions: the y array and six work regions; roles are indices.
    // FP64 stages: y, F, F_new and three Y stage buffers (regions 3-5). Mixed stages: y, F,
    // F_new, y_new (region 3) and, as FP32 arrays of N values, three increments d (regions 4
    // and 5) and the FP32 copies of F and F_new (region 5, second half, and region 6).
    double* P[7];
    P[0] = yall + I.off;
    for (int q = 0; q < 6; ++q) P[q + 1] = work + (long long)q * total + I.off;
    int iy = 0, iF = 1, iFn = 2;
    int bufs[3] = {3, 4, 5}; // stage buffers (rotated like the single-problem integrator)
    int iyn = 3, iff = 0;    // mixed: y_new region, which FP32 F copy is current
    float* D[3]  = {reinterpret_cast<float*>(P[4]), reinterpret_cast<float*>(P[4]) + N,
                    reinterpret_cast<float*>(P[5])};
    float* Ff[2] = {reinterpret_cast<float*>(P[5]) + N, reinterpret_cast<float*>(P[6])};

    // F_0 = A y_0 (and its FP32 copy for the mixed stages)
    for (int j = j0 + warp; j < j1; j += NW)
      for (int i = lane; i < n; i += 32)
      {
        const long long k = (long long)j * n + i;
        const double f    = lap(P[iy], n, i, j, j0, j1, cx, cy, cc);
        P[iF][k]          = f;
        if (MIXED) Ff[0][k] = (float)f;
      }
    inst_sync<CL>();
    long long nfe = 1, nst = 0, natt = 0, netf = 0, nexp = 0, stmax = 0, sttot = 0, nhist = 0;
    double t = 0.0, hnext = 0.0, hlast = 0.0, ep1 = 0.0, ep2 = 0.0;
    bool after_fail = false;
    int status      = 0;

    // initial step (Hairer-Norsett-Wanner II.4, probe capped at 1/rho)
    {
      const double* yc = P[iy];
      const double* F0 = P[iF];
      xsum::Limbs a0, a1;
      xsum::zero(a0);
      xsum::zero(a1);
      unsigned f0 = 0, f1 = 0;
      for (int j = j0 + warp; j < j1; j += NW)
        for (int i = lane; i < n; i += 32)
        {
          const long long k = (long long)j * n + i;
          const double wt   = 1.0 / (prm.rtol * fabs(yc[k]) + prm.atol);
          const double x0 = yc[k] * wt, x1 = F0[k] * wt;
          xsum::add(a0, x0 * x0, f0);
          xsum::add(a1, x1 * x1, f1);
        }
      const double d0 = sqrt(inst_exact_sum<NT, CL>(a0, f0, sm, climb, &sflags, &sres) / (double)N);
      const double d1 = sqrt(inst_exact_sum<NT, CL>(a1, f1, sm, climb, &sflags, &sres) / (double)N);
      double h0       = (d0 < 1.0e-5 || d1 < 1.0e-5) ? 1.0e-6 : 0.01 * (d0 / d1);
      if (rho > 0.0 && h0 * rho > 1.0) h0 = 1.0 / rho;
      if (h0 > prm.tf) h0 = prm.tf;
      double* y1 = P[bufs[0]];
      for (int j = j0 + warp; j < j1; j += NW)
        for (int i = lane; i < n; i += 32)
        {
          const long long k = (long long)j * n + i;
          y1[k]             = __fma_rn(h0, F0[k], yc[k]);
        }
      inst_sync<CL>();
      xsum::Limbs a2;
      xsum::zero(a2);
      unsigned f2 = 0;
      for (int j = j0 + warp; j < j1; j += NW)
        for (int i = lane; i < n; i += 32)
        {
          const long long k = (long long)j * n + i;
          const double f1v  = lap(y1, n, i, j, j0, j1, cx, cy, cc);
          const double wt   = 1.0 / (prm.rtol * fabs(yc[k]) + prm.atol);
          const double x    = (f1v - F0[k]) * wt;
          xsum::add(a2, x * x, f2);
        }
      nfe++;
      const double d2 = sqrt(inst_exact_sum<NT, CL>(a2, f2, sm, climb, &sflags, &sres) / (double)N) / h0;
      const double dm = d1 > d2 ? d1 : d2;
      double h1       = (dm <= 1.0e-15) ? fmax(1.0e-6, h0 * 1.0e-3) : stsm::pow(0.01 / dm, 1.0 / B_ORD);
      if (!(h1 > 0.0) || !(h1 < 1e300)) h1 = h0;
      double h = (100.0 * h0 < h1) ? 100.0 * h0 : h1;
      if (h > prm.tf) h = prm.tf;
      hnext = h;
      if (!(h > 0.0)) status = -3; // a non-finite state gives no usable step
    }

    while (t < prm.tf && status == 0)
    {
      if (nst >= prm.maxsteps)
      {
        status = -1;
        break;
      }
      int nef = 0;
      for (;;)
      {
        double h = hnext, hmax;
        bool clipped = false;
        int s        = d_stages(prm.method, h, rho, prm.smax, &hmax);
        if (s > prm.smax)
        {
          h = hmax;
          nexp++;
        }
        if (t + h >= prm.tf)
        {
          h       = prm.tf - t;
          clipped = true;
        }
        s = d_stages(prm.method, h, rho, prm.smax, &hmax);
        natt++;
        const CoefT* ct = reinterpret_cast<const CoefT*>(prm.coef) + (long long)s * (prm.smax + 1);
        const double* yc = P[iy];
        const double* F0 = P[iF];
        xsum::Limbs ae;
        xsum::zero(ae);
        unsigned fe      = 0;
        const double p4h = 0.4 * h;
        int last         = 0; // FP64 stages: index into bufs of Y_{j-1}
        if constexpr (MIXED)
        {
          // stage 1: d_1 = (h mus_1) F_0 in FP32
          {
            const float hm1  = (float)(h * ct[1].mus);
            const float* ff  = Ff[iff];
            float* d1        = D[0];
            for (int j = j0 + warp; j < j1; j += NW)
              for (int i = lane; i < n; i += 32)
              {
                const long long k = (long long)j * n + i;
                d1[k]             = hm1 * ff[k];
              }
            inst_sync<CL>();
          }
          const float* dm2 = nullptr; // d_{j-2}; none at stage 2
          int lastd        = 0;
          double* yn       = P[iyn];
          for (int jst = 2; jst <= s; ++jst)
          {
            const double mu = ct[jst].mu, nu = ct[jst].nu, mus = ct[jst].mus, ajm1 = ct[jst].ajm1;
            const double hm = h * mus;
            const float gs = (float)(((mu + nu) - 1.0) + hm * ((cc + 2.0 * cx) + 2.0 * cy));
            const float gx = (float)(hm * cx), gy = (float)(hm * cy), gm = (float)(-nu);
            const float gF   = (float)(hm * (1.0 - ajm1));
            const float* dm1 = D[lastd];
            const float* ff  = Ff[iff];
            const int nxt    = (lastd + 1) % 3;
            float* dj        = D[nxt];
            for (int j = j0 + warp; j < j1; j += NW)
              for (int i = lane; i < n; i += 32)
              {
                const long long k = (long long)j * n + i;
                const float dw = (i > 0) ? dm1[k - 1] : 0.0f;
                const float de = (i < n - 1) ? dm1[k + 1] : 0.0f;
                const float ds = (j > 0) ? ldrowf(&dm1[k - n], j - 1 < j0) : 0.0f;
                const float dn = (j < n - 1) ? ldrowf(&dm1[k + n], j + 1 >= j1) : 0.0f;
                const float m2 = dm2 ? dm2[k] : 0.0f;
                const float dv = mixed_point<false>(gs, gx, gy, gm, gF, dm1[k], dw, de, ds, dn, m2, ff[k], 0.f, 0.f,
                                                    0.f, 0.f);
                dj[k] = dv;
                if (jst == s) yn[k] = yc[k] + (double)dv; // the last stage also forms y_new = y + d_s
              }
            inst_sync<CL>();
            dm2   = dm1;
            lastd = nxt;
          }
          // step end: F_new = A y_new, its FP32 copy and the error
          const float* dsv = D[lastd];
          double* Fnew = P[iFn];
          float* Ffn   = Ff[1 - iff];
          for (int j = j0 + warp; j < j1; j += NW)
            for (int i = lane; i < n; i += 32)
            {
              const long long k = (long long)j * n + i;
              const double f    = lap(yn, n, i, j, j0, j1, cx, cy, cc);
              Fnew[k]           = f;
              Ffn[k]            = (float)f;
              const double yv   = yc[k];
              const double d    = -(double)dsv[k]; // y_n - y_{n+1} as -d_s (the single-problem form)
              double e          = 0.8 * d;
              e                 = __fma_rn(p4h, F0[k], e);
              e                 = __fma_rn(p4h, f, e);
              const double wt   = mixed_weight(prm.rtol, prm.atol, yv);
              const double x    = e * wt;
              xsum::add(ae, x * x, fe);
            }
        }
        else
        {
          // stage 1 -> bufs[0]
          {
            const double hm1 = h * ct[1].mus;
            double* y1       = P[bufs[0]];
            for (int j = j0 + warp; j < j1; j += NW)
              for (int i = lane; i < n; i += 32)
              {
                const long long k = (long long)j * n + i;
                y1[k]             = __fma_rn(hm1, F0[k], yc[k]);
              }
            inst_sync<CL>();
          }
          const double* ym2 = yc;
          for (int jst = 2; jst <= s; ++jst)
          {
            const double mu = ct[jst].mu, nu = ct[jst].nu, mus = ct[jst].mus, ajm1 = ct[jst].ajm1;
            const double hm = h * mus;
            const double tm = hm * cc;
            const double gc = mu + tm, gx = hm * cx, gy = hm * cy, gn = nu, g0 = (1.0 - mu) - nu;
            const double gf = -(hm * ajm1);
            const double* ym1 = P[bufs[last]];
            const int nxt     = (last + 1) % 3;
            double* yj        = P[bufs[nxt]];
            for (int j = j0 + warp; j < j1; j += NW)
              for (int i = lane; i < n; i += 32)
              {
                const long long k = (long long)j * n + i;
                const double uw = (i > 0) ? ym1[k - 1] : 0.0;
                const double ue = (i < n - 1) ? ym1[k + 1] : 0.0;
                const double us = (j > 0) ? ldrow(&ym1[k - n], j - 1 < j0) : 0.0;
                const double un = (j < n - 1) ? ldrow(&ym1[k + n], j + 1 >= j1) : 0.0;
                const double sx = uw + ue, sy = us + un;
                double acc      = gc * ym1[k];
                acc             = __fma_rn(gx, sx, acc);
                acc             = __fma_rn(gy, sy, acc);
                acc             = __fma_rn(gn, ym2[k], acc);
                acc             = __fma_rn(g0, yc[k], acc);
                acc             = __fma_rn(gf, F0[k], acc);
                yj[k]           = acc;
              }
            inst_sync<CL>();
            ym2  = ym1;
            last = nxt;
          }
          const double* Ys = P[bufs[last]];
          double* Fnew     = P[iFn];
          // step end: Fnew = A Ys, err = 0.8 (y - Ys) + 0.4 h (F + Fnew), exact WRMS
          for (int j = j0 + warp; j < j1; j += NW)
            for (int i = lane; i < n; i += 32)
            {
              const long long k = (long long)j * n + i;
              const double f    = lap(Ys, n, i, j, j0, j1, cx, cy, cc);
              Fnew[k]           = f;
              const double yv   = yc[k];
              const double d    = yv - Ys[k];
              double e          = 0.8 * d;
              e                 = __fma_rn(p4h, F0[k], e);
              e                 = __fma_rn(p4h, f, e);
              const double wt   = 1.0 / (prm.rtol * fabs(yv) + prm.atol);
              const double x    = e * wt;
              xsum::add(ae, x * x, fe);
            }
        }
        const double dsm = sqrt(inst_exact_sum<NT, CL>(ae, fe, sm, climb, &sflags, &sres) / (double)N);
        nfe += s;
        sttot += s;
        if (s > stmax) stmax = s;
        if (dsm <= 1.0)
        { // accept: y <- Ys (role swap with its stage buffer or with y_new), F <- Fnew
          t = clipped ? prm.tf : t + h;
          if constexpr (MIXED)
          {
            const int yv_ = iyn;
            iyn           = iy;
            iy            = yv_;
            iff           = 1 - iff;
          }
          else
          {
            const int ys = bufs[last];
            bufs[last]   = iy;
            iy           = ys;
          }
          const int tf_ = iF;
          iF           = iFn;
          iFn          = tf_;
          const double hprev = hlast;
          hlast        = h;
          double hn    = block_control(prm.controller, h, dsm, ep1, ep2, hprev, nhist, &shn);
          double eta   = B_SAFETY * hn / h;
          const double emx = (nst == 0) ? B_ETAMX1 : (after_fail ? 1.0 : B_GROWTH);
          if (eta > emx) eta = emx;
          if (eta >= 1.0 && eta <= 1.5) eta = 1.0;
          hnext      = h * eta;
          ep2        = ep1;
          ep1        = dsm;
          nhist++;
          after_fail = false;
          nst++;
          break;
        }
        netf++;
        nef++;
        if (!(dsm == dsm) || nef > 20)
        {
          status = -3;
          break;
        }
        double hn  = block_control(prm.controller, h, dsm, ep1, ep2, hlast, nhist, &shn);
        double eta = B_SAFETY * hn / h;
        if (eta > 1.0) eta = 1.0;
        if (nef >= 2 && eta > B_ETAMXF) eta = B_ETAMXF;
        if (eta < B_ETAMIN) eta = B_ETAMIN;
        hnext      = h * eta;
        after_fail = true;
      }
    }
    // final state into the y array
    if (iy != 0)
    {
      const double* yc = P[iy];
      for (int j = j0 + warp; j < j1; j += NW)
        for (int i = lane; i < n; i += 32)
        {
          const long long k = (long long)j * n + i;
          P[0][k]           = yc[k];
        }
    }
    __syncthreads();
    if (tid == 0 && rank == 0)
    {
      I.status       = status;
      I.nst          = nst;
      I.nst_att      = natt;
      I.netf         = netf;
      I.nfe          = nfe;
      I.nst_exp      = nexp;
      I.stage_max    = stmax;
      I.stages_total = sttot;
      I.t            = t;
      I.hlast        = hlast;
      I.hnext        = hnext;
    }
    __syncthreads();
  }
}

} // namespace
// ---------------------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------------------
template <int NT, int CL, bool MIXED>
static bool launch_group(const STS_Batch b, const BatchParams& prm, const int* order, int count, int* queue, int grid,
                         cudaStream_t st)
{
  if constexpr (CL > 8)
  { // 16-CTA clusters are a non-portable size: opt in, and launch only if one fits
    static int fits = -1;
    if (fits < 0)
    {
      fits = 0;
      if (cudaFuncSetAttribute(batch_kernel<NT, CL, MIXED>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess)
      {
        cudaLaunchConfig_t q = {};
        q.gridDim            = dim3(CL, 1, 1);
        q.blockDim           = dim3(NT, 1, 1);
        cudaLaunchAttribute qa[1];
        qa[0].id               = cudaLaunchAttributeClusterDimension;
        qa[0].val.clusterDim.x = CL;
        qa[0].val.clusterDim.y = 1;
        qa[0].val.clusterDim.z = 1;
        q.attrs                = qa;
        q.numAttrs             = 1;
        int nc                 = 0;
        if (cudaOccupancyMaxActiveClusters(&nc, batch_kernel<NT, CL, MIXED>, &q) == cudaSuccess && nc > 0) fits = 1;
      }
      cudaGetLastError();
    }
    if (!fits)
    {
      sts_set_error("STS_Batch: %d-CTA clusters of %d threads cannot be scheduled", CL, NT);
      return false;
    }
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim            = dim3((unsigned)grid, 1, 1);
  cfg.blockDim           = dim3(NT, 1, 1);
  cfg.dynamicSmemBytes   = 0;
  cfg.stream             = st;
  cudaLaunchAttribute attr[1];
  attr[0].id               = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = CL;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs                = attr;
  cfg.numAttrs             = CL > 1 ? 1 : 0;
  return STS_CUDA_OK(cudaLaunchKernelEx(&cfg, batch_kernel<NT, CL, MIXED>, b->dinst, order, count, queue, b->y, b->work,
                                        b->total, prm));
}

// the FP64 and the mixed forms are separate instantiations: each gets its own register
// allocation (the kernel runs at the 64-register cap of four 256-thread CTAs per SM)
template <int NT, bool MIXED>
static bool launch_cl_m(const STS_Batch b, const BatchParams& prm, int cl, const int* order, int count, int* queue,
                        int grid, cudaStream_t st)
{
  switch (cl)
  {
  case 2: return launch_group<NT, 2, MIXED>(b, prm, order, count, queue, grid, st);
  case 4: return launch_group<NT, 4, MIXED>(b, prm, order, count, queue, grid, st);
  case 8: return launch_group<NT, 8, MIXED>(b, prm, order, count, queue, grid, st);
  case 16: return launch_group<NT, 16, MIXED>(b, prm, order, count, queue, grid, st);
  default: return launch_group<NT, 1, MIXED>(b, prm, order, count, queue, grid, st);
  }
}

template <int NT>
static bool launch_cl(const STS_Batch b, const BatchParams& prm, int cl, const int* order, int count, int* queue,
                      int grid, cudaStream_t st)
{
  return prm.mixed ? launch_cl_m<NT, true>(b, prm, cl, order, count, queue, grid, st)
                   : launch_cl_m<NT, false>(b, prm, cl, order, count, queue, grid, st);
}

// One launch (cluster size 1), or two concurrent launches: instances with n >= big_n on
// clusters of `cluster` CTAs (launched first), the rest on single CTAs on a second stream.
// The CTA slots (SMs x CTAs per SM) are split between the two in proportion to their
// estimated cost.
static bool batch_launch(STS_Batch b, const BatchParams& prm, int threads, int ctas_per_sm)
{
  STS_Context ctx = b->ctx;
  cudaStream_t st = ctx->stream;
  if (!STS_CUDA_OK(cudaMemsetAsync(b->dqueue, 0, 2 * sizeof(int), st))) return false;
  const int slots = ctx->num_sms * ctas_per_sm;
  auto go = [&](int cl, const int* order, int count, int* queue, int grid, cudaStream_t s) {
    return threads == 256 ? launch_cl<256>(b, prm, cl, order, count, queue, grid, s)
                          : launch_cl<512>(b, prm, cl, order, count, queue, grid, s);
  };
  const int CL = b->cluster;
  if (CL <= 1 || b->nbig == 0)
    return go(1, b->dorder, b->ninst, b->dqueue, std::max(1, std::min(b->ninst, slots)), st);
  const int nsmall = b->ninst - b->nbig;
  int gbig = (int)std::lround(b->big_share * slots / CL) * CL;
  gbig     = std::max(CL, std::min(gbig, b->nbig * CL));
  gbig     = std::min(gbig, (slots / CL) * CL);
  int gsm  = std::max(1, std::min(nsmall, slots - gbig));
  bool ok  = go(CL, b->dorder_big, b->nbig, b->dqueue, gbig, st);
  if (ok && nsmall > 0)
  {
    ok = STS_CUDA_OK(cudaEventRecord(b->ev_fork, st)) && STS_CUDA_OK(cudaStreamWaitEvent(b->side, b->ev_fork, 0)) &&
         go(1, b->dorder_small, nsmall, b->dqueue + 1, gsm, b->side) &&
         STS_CUDA_OK(cudaEventRecord(b->ev_join, b->side)) && STS_CUDA_OK(cudaStreamWaitEvent(st, b->ev_join, 0));
  }
  return ok;
}

// split the cost-ordered instances into the clustered group (n >= big_n) and the rest
static bool batch_regroup(STS_Batch b)
{
  std::vector<int> order(b->ninst), big, small;
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return b->cost[x] > b->cost[y]; });
  double cb = 0.0, ct = 0.0;
  for (int i : order)
  {
    ct += b->cost[i];
    if (b->cluster > 1 && b->hinst[i].n >= b->big_n)
    {
      big.push_back(i);
      cb += b->cost[i];
    }
    else small.push_back(i);
  }
  b->nbig      = (int)big.size();
  b->big_share = ct > 0.0 ? cb / ct : 0.0;
  return (big.empty() || STS_CUDA_OK(cudaMemcpy(b->dorder_big, big.data(), big.size() * sizeof(int),
                                                 cudaMemcpyHostToDevice))) &&
         (small.empty() || STS_CUDA_OK(cudaMemcpy(b->dorder_small, small.data(), small.size() * sizeof(int),
                                                   cudaMemcpyHostToDevice)));
}

extern "C" STS_Batch STS_BatchCreate(STS_Context ctx, int ninst, const int* n, const double* kx, const double* ky)
{
  if (!ctx || ninst < 1 || !n || !kx || !ky)
  {
    sts_set_error("STS_BatchCreate: invalid arguments");
    return nullptr;
  }
  ctx_activate(ctx);
  STS_Batch b = new STS_Batch_();
  b->ctx      = ctx;
  b->ninst    = ninst;
  b->hinst.resize(ninst);
  long long off = 0;
  std::vector<double> cost(ninst);
  for (int i = 0; i < ninst; ++i)
  {
    if (n[i] < 2 || n[i] > 46340)
    {
      sts_set_error("STS_BatchCreate: instance %d: grid size %d out of range", i, n[i]);
      delete b;
      return nullptr;
    }
    BatchInst& I = b->hinst[i];
    memset(&I, 0, sizeof(I));
    I.n          = n[i];
    I.off        = off;
    const double d = 1.0 / (n[i] + 1);
    I.kx         = kx[i];
    I.ky         = ky[i];
    I.cx         = kx[i] / (d * d);
    I.cy         = ky[i] / (d * d);
    I.cc         = -2.0 * (I.cx + I.cy);
    // analytic dominant eigenvalue (diffusion_2D/main.cpp:544) with the 1.01 safety factor
    const double a = kx[i] / d / d, c = ky[i] / d / d;
    I.rho        = 1.01 * fabs(-8.0 * (a > c ? a : c));
    off += (long long)n[i] * n[i];
    cost[i] = (double)n[i] * n[i] * sqrt(I.rho);
  }
  b->total = off;
  b->cost  = cost;
  std::vector<int> order(ninst);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return cost[x] > cost[y]; });
  bool ok = STS_CUDA_OK(cudaMalloc(&b->dinst, ninst * sizeof(BatchInst))) &&
            STS_CUDA_OK(cudaMalloc(&b->dorder, ninst * sizeof(int))) &&
            STS_CUDA_OK(cudaMalloc(&b->dorder_big, ninst * sizeof(int))) &&
            STS_CUDA_OK(cudaMalloc(&b->dorder_small, ninst * sizeof(int))) &&
            STS_CUDA_OK(cudaMalloc(&b->dqueue, 2 * sizeof(int))) &&
            STS_CUDA_OK(cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking)) &&
            STS_CUDA_OK(cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming)) &&
            STS_CUDA_OK(cudaEventCreateWithFlags(&b->ev_join, cudaEventDisableTiming)) &&
            STS_CUDA_OK(cudaMalloc(&b->y, b->total * sizeof(double))) &&
            STS_CUDA_OK(cudaMalloc(&b->work, 6 * b->total * sizeof(double))) &&
            STS_CUDA_OK(cudaMemcpy(b->dinst, b->hinst.data(), ninst * sizeof(BatchInst), cudaMemcpyHostToDevice)) &&
            STS_CUDA_OK(cudaMemcpy(b->dorder, order.data(), ninst * sizeof(int), cudaMemcpyHostToDevice)) &&
            STS_CUDA_OK(cudaMemset(b->y, 0, b->total * sizeof(double))) && batch_regroup(b);
  if (!ok)
  {
    STS_BatchFree(&b);
    return nullptr;
  }
  return b;
}

extern "C" int STS_BatchFree(STS_Batch* pb)
{
  if (!pb || !*pb) return 0;
  STS_Batch b = *pb;
  cudaSetDevice(b->ctx->device);
  cudaFree(b->dinst);
  cudaFree(b->dorder);
  cudaFree(b->dqueue);
  cudaFree(b->y);
  cudaFree(b->work);
  cudaFree(b->dcoef);
  cudaFree(b->dorder_big);
  cudaFree(b->dorder_small);
  if (b->side) cudaStreamDestroy(b->side);
  if (b->ev_fork) cudaEventDestroy(b->ev_fork);
  if (b->ev_join) cudaEventDestroy(b->ev_join);
  delete b;
  *pb = nullptr;
  return 0;
}

extern "C" long long STS_BatchTotalDOF(STS_Batch b) { return b ? b->total : 0; }

extern "C" int STS_BatchSetState(STS_Batch b, const double* host_y)
{
  if (!b || !host_y) return -1;
  ctx_activate(b->ctx);
  return STS_CUDA_OK(cudaMemcpy(b->y, host_y, b->total * sizeof(double), cudaMemcpyHostToDevice)) ? 0 : -1;
}

extern "C" int STS_BatchGetState(STS_Batch b, double* host_y)
{
  if (!b || !host_y) return -1;
  ctx_activate(b->ctx);
  if (!STS_CUDA_OK(cudaStreamSynchronize(b->ctx->stream))) return -1;
  return STS_CUDA_OK(cudaMemcpy(host_y, b->y, b->total * sizeof(double), cudaMemcpyDeviceToHost)) ? 0 : -1;
}

// initial states sum_k a_k sin(p_k pi x) sin(q_k pi y), nmodes per instance (host tabulated)
extern "C" int STS_BatchSetInitialModes(STS_Batch b, int nmodes, const int* p, const int* q, const double* a)
{
  if (!b || nmodes < 0) return -1;
  std::vector<double> h(b->total);
  const double PI = 3.14159265358979323846;
  for (int i = 0; i < b->ninst; ++i)
  {
    const BatchInst& I = b->hinst[i];
    const int n        = I.n;
    const double d     = 1.0 / (n + 1);
    for (int jj = 0; jj < n; ++jj)
      for (int ii = 0; ii < n; ++ii)
      {
        const double x = (ii + 1) * d, y = (jj + 1) * d;
        double v       = 0.0;
        for (int k = 0; k < nmodes; ++k)
        {
          const int m = i * nmodes + k;
          v += a[m] * sin(p[m] * PI * x) * sin(q[m] * PI * y);
        }
        h[I.off + (long long)jj * n + ii] = v;
      }
  }
  return STS_BatchSetState(b, h.data());
}

extern "C" int STS_BatchEvolve(STS_Batch b, double tf, int method, double rtol, double atol, int smax, int controller,
                               long long maxsteps)
{
  STS_MARK_FUNCTION;
  if (!b || !(tf > 0.0) || smax < 2 || smax > 10000) return STS_ILL_INPUT;
  if (controller < STS_ADAPT_PID || controller > STS_ADAPT_IMEX_GUS) return STS_ILL_INPUT;
  if (method != STS_LSRK_RKC_2 && method != STS_LSRK_RKL_2) return STS_ILL_INPUT;
  ctx_activate(b->ctx);
  BatchParams prm;
  prm.tf         = tf;
  prm.rtol       = rtol;
  prm.atol       = atol;
  prm.eig_safety = 1.01;
  prm.method     = method;
  prm.smax       = smax;
  prm.controller = controller;
  prm.maxsteps   = (int)(maxsteps > 0 ? std::min<long long>(maxsteps, 1LL << 30) : 1000000);
  prm.mixed      = b->mixed;
  prm.pad_       = 0;
  if (b->coef_method != method || b->coef_smax != smax)
  {
    const int S = smax + 1;
    std::vector<CoefT> tab((size_t)S * S);
    std::vector<double> mu(S), nu(S), mus(S), ajm1(S), cjm1(S);
    for (int sc = 2; sc <= smax; ++sc)
    {
      STS_LSRKStageCoeffs(method, sc, mu.data(), nu.data(), mus.data(), ajm1.data(), cjm1.data());
      for (int j = 1; j <= sc; ++j) tab[(size_t)sc * S + j] = CoefT{mu[j], nu[j], mus[j], ajm1[j]};
    }
    cudaFree(b->dcoef);
    b->dcoef = nullptr;
    if (!STS_CUDA_OK(cudaMalloc(&b->dcoef, tab.size() * sizeof(CoefT))) ||
        !STS_CUDA_OK(cudaMemcpy(b->dcoef, tab.data(), tab.size() * sizeof(CoefT), cudaMemcpyHostToDevice)))
      return -1;
    b->coef_method = method;
    b->coef_smax   = smax;
  }
  prm.coef = b->dcoef;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, b->ctx->stream);
  const bool ok = batch_launch(b, prm, b->block, b->ctas_per_sm);
  cudaEventRecord(e1, b->ctx->stream);
  if (!ok || !STS_CUDA_OK(cudaEventSynchronize(e1)))
  {
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return STS_ERR_FAILURE;
  }
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  b->last_ms = ms;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (!STS_CUDA_OK(cudaMemcpy(b->hinst.data(), b->dinst, b->ninst * sizeof(BatchInst), cudaMemcpyDeviceToHost)))
    return STS_ERR_FAILURE;
  for (const BatchInst& I : b->hinst)
    if (I.status < 0) return I.status;
  return STS_SUCCESS;
}

extern "C" double STS_BatchLastMilliseconds(STS_Batch b) { return b ? b->last_ms : 0.0; }

extern "C" int STS_BatchGetInstanceStats(STS_Batch b, int inst, STS_Stats* s)
{
  if (!b || inst < 0 || inst >= b->ninst || !s) return -1;
  const BatchInst& I = b->hinst[inst];
  memset(s, 0, sizeof(*s));
  s->nst             = I.nst;
  s->nst_attempts    = I.nst_att;
  s->netf            = I.netf;
  s->nfe             = I.nfe;
  s->nst_exp         = I.nst_exp;
  s->stage_max       = I.stage_max;
  s->stages_total    = I.stages_total;
  s->t               = I.t;
  s->hlast           = I.hlast;
  s->hnext           = I.hnext;
  s->spectral_radius = I.rho;
  return 0;
}

extern "C" int STS_BatchSetMixed(STS_Batch b, int mixed)
{
  if (!b || (mixed != 0 && mixed != 1)) return STS_ILL_INPUT;
  b->mixed = mixed;
  return 0;
}

extern "C" int STS_BatchSetLaunch(STS_Batch b, int threads, int ctas_per_sm)
{
  if (!b || (threads != 256 && threads != 512) || ctas_per_sm < 1 || ctas_per_sm > 8)
    return STS_ILL_INPUT;
  b->block       = threads;
  b->ctas_per_sm = ctas_per_sm;
  return 0;
}

extern "C" int STS_BatchSetCluster(STS_Batch b, int cluster, int big_n)
{
  if (!b || (cluster != 1 && cluster != 2 && cluster != 4 && cluster != 8 && cluster != 16) || big_n < 2)
    return STS_ILL_INPUT;
  ctx_activate(b->ctx);
  b->cluster = cluster;
  b->big_n   = big_n;
  return batch_regroup(b) ? 0 : STS_ERR_FAILURE;
}

extern "C" int STS_BatchGetLaunch(STS_Batch b, int* threads, int* ctas_per_sm, int* cluster, int* big_n)
{
  if (!b) return STS_ILL_INPUT;
  if (threads) *threads = b->block;
  if (ctas_per_sm) *ctas_per_sm = b->ctas_per_sm;
  if (cluster) *cluster = b->cluster;
  if (big_n) *big_n = b->big_n;
  return 0;
}

// Autotuner: runs the batch from its current state to tf_probe with every launch shape
// (threads per CTA, CTAs per SM, cluster size for the large instances), restores the state
// after each probe, and keeps the fastest shape.
extern "C" int STS_BatchAutotune(STS_Batch b, double tf_probe, int method, double rtol, double atol, int smax,
                                 int* threads, int* ctas_per_sm, double* ms_best)
{
  if (!b) return -1;
  ctx_activate(b->ctx);
  double* save = nullptr;
  if (!STS_CUDA_OK(cudaMalloc(&save, b->total * sizeof(double)))) return -1;
  cudaMemcpyAsync(save, b->y, b->total * sizeof(double), cudaMemcpyDeviceToDevice, b->ctx->stream);
  // {threads per CTA, CTAs per SM, cluster size of the large-instance group}
  // (the kernel is compiled for 1024 resident threads per SM: 64 registers per thread).
  // 16-CTA clusters stay available through STS_BatchSetCluster but are not candidates: the
  // short probe favours them while whole runs measured them slower than 8-CTA clusters
  // (5.85 s against 5.46 s on the 512-instance workload).
  const int shapes[][3] = {{256, 4, 1}, {512, 2, 1}, {256, 4, 4}, {512, 2, 4}, {256, 4, 8},
                           {512, 2, 8}, {512, 1, 8}};
  double best           = 1e30;
  int bt = b->block, bc = b->ctas_per_sm, bcl = b->cluster;
  for (auto& sh : shapes)
  {
    b->block       = sh[0];
    b->ctas_per_sm = sh[1];
    b->cluster     = sh[2];
    if (!batch_regroup(b)) break;
    const int rc = STS_BatchEvolve(b, tf_probe, method, rtol, atol, smax, 0, 0); // PID, as evolve
    cudaMemcpyAsync(b->y, save, b->total * sizeof(double), cudaMemcpyDeviceToDevice, b->ctx->stream);
    if (rc == 0 && b->last_ms < best)
    {
      best = b->last_ms;
      bt   = sh[0];
      bc   = sh[1];
      bcl  = sh[2];
    }
  }
  cudaStreamSynchronize(b->ctx->stream);
  cudaFree(save);
  b->block       = bt;
  b->ctas_per_sm = bc;
  b->cluster     = bcl;
  batch_regroup(b);
  if (threads) *threads = bt;
  if (ctas_per_sm) *ctas_per_sm = bc;
  if (ms_best) *ms_best = best;
  return 0;
}
