// Fused mixed stages (temporal blocking): several consecutive FP32-increment stages per
// launch on shared-memory tiles, the same bits as one launch per stage (stage_tma.cu).
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <type_traits>

#include "kernels.cuh"
#include "stage_tma.cuh"
#include "sts_internal.cuh"
#include "tma_util.cuh"

namespace {

// ---------------------------------------------------------------------------------------
// Fused stages (temporal blocking): KS consecutive mixed stages j .. j+KS-1 in one pass.
//
// A CTA loads one 128 x (TH+8) tile of d_{j-1}, d_{j-2} and F_0 (4-cell halo on every side:
// x from x0-4 keeps the 16-byte alignment, out-of-range parts arrive zero-filled) and runs
// the stages in shared memory. Stage l of the group (l = 0 .. KS-1) is evaluated on the tile
// rows [-(KS-1-l), TH+KS-1-l) and on all 128 columns; the cone of valid values shrinks by one
// cell per stage and per side, so after KS <= 4 stages the 120 x TH output block is exact.
// (Column 0 and 127 of the shared tile see a stand-in for their missing outer neighbour:
// the error they carry moves inward by one column per stage and never reaches the output
// columns 4 .. 123.) Each stage reads d_{j+l-2} only at the point itself, so its result is
// written over that array in place: two stage arrays and F_0, 3 x 128 x (TH+8) floats.
// Points outside the domain are set to zero after every stage (homogeneous Dirichlet ghost
// values), exactly what the single-stage kernels read there; tiles whose loaded region lies
// inside the domain skip that mask. The forcing rows of the tile and the group's stage
// scalars are staged in shared memory once. Only the group's last two
// stages are stored to global memory (o2 = d_{j+KS-2}, o1 = d_{j+KS-1}): the next group, or
// the step end, needs nothing else. Per point the arithmetic is mixed_point's with the
// operands of the single-stage kernels, evaluated two columns at a time by mixed_pair (the
// paired FP32 instructions, the same rounding per component), so a group gives the bits of
// KS single launches. Rows march three per trip, so the row window rotates through registers
// without copies.
//
// HBM traffic per point and group: 12 B read (d_{j-1}, d_{j-2}, F_0; the halo overlap of
// neighbouring tiles is mostly served by L2) + 8 B written, 20 / KS B per DOF-stage against
// 16 B for a single-stage launch.
// ---------------------------------------------------------------------------------------
constexpr int FW  = 128;    // loaded tile width (floats): 32 lanes x 4 columns
constexpr int FH  = 4;      // halo rows / columns of the loaded tiles (KS <= FH)
constexpr int FOW = FW - 2 * FH; // output columns per tile

// TH output rows per tile, NT threads per CTA, MINB CTAs per SM, NSET tile buffers per CTA
// (2: the next tile's copies run while the CTA computes this one)
template <int TH_, int NT_, int MINB_, int NSET_>
struct FCfg {
  static constexpr int TH = TH_, NT = NT_, MINB = MINB_, NSET = NSET_;
  static constexpr int NW         = NT / 32;
  static constexpr int AH         = TH + 2 * FH;
  static constexpr int ARR_BYTES  = FW * AH * 4;
  static constexpr int SY_BYTES   = (2 * AH * 8 + 127) / 128 * 128; // Sy | Syy rows, as (v, v) pairs
  static constexpr int SET_BYTES  = 3 * ARR_BYTES + SY_BYTES;
  static constexpr int COEF_OFF   = NSET * SET_BYTES;               // 4 stages x 8 FP32 scalars
  static constexpr int BAR_OFF    = COEF_OFF + 128;
  static constexpr int SMEM_BYTES = BAR_OFF + 16;
  static_assert(NT % 32 == 0 && NSET >= 1 && NSET <= 2, "whole warps, one or two tile buffers");
};

template <class K, int KS, bool FORCED, bool HAS_M2>
__global__ void __launch_bounds__(K::NT, K::MINB)
  stage32_fused_kernel(const __grid_constant__ CUtensorMap mm1, const __grid_constant__ CUtensorMap mm2,
                       const __grid_constant__ CUtensorMap mf0, ProbDev P, const StageArgs* __restrict__ A,
                       float* __restrict__ o2, float* __restrict__ o1, int* err)
{
  static_assert(KS >= 2 && KS <= FH, "group of 2 .. 4 stages");
  extern __shared__ __align__(128) unsigned char smem[];
  float* coef   = reinterpret_cast<float*>(smem + K::COEF_OFF);
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + K::BAR_OFF);
  const int nx = (int)P.nx, ny = (int)P.ny;
  const int tiles_x = (nx + FOW - 1) / FOW;
  const int ntiles  = tiles_x * ((ny + K::TH - 1) / K::TH);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int c = lane * 4; // this lane's first column in the shared tile

  // set b: d_{j-1} | d_{j-2} | F_0 | Sy, Syy of the tile rows
  auto arr = [&](int b, int a) { return reinterpret_cast<float*>(smem + b * K::SET_BYTES + a * K::ARR_BYTES); };
  auto issue = [&](int b, int t) {
    const int x0 = (t % tiles_x) * FOW, y0 = (t / tiles_x) * K::TH;
    // earlier generic-proxy reads and writes of this set are ordered before the copies by
    // the barrier that ended its last use
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    mbar_expect_tx(&bar[b], (HAS_M2 ? 3 : 2) * K::ARR_BYTES);
    tma_load_2d(arr(b, 0), &mm1, &bar[b], x0 - FH, y0 - FH);
    if (HAS_M2) tma_load_2d(arr(b, 1), &mm2, &bar[b], x0 - FH, y0 - FH);
    tma_load_2d(arr(b, 2), &mf0, &bar[b], x0 - FH, y0 - FH);
  };
  if (tid == 0)
  {
    for (int b = 0; b < K::NSET; ++b) mbar_init(&bar[b], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  static_assert(offsetof(StageArgs, gaf) - offsetof(StageArgs, gsf) == 7 * sizeof(float),
                "the eight FP32 stage scalars are consecutive");
  if (tid < KS * 8) // gs, gx, gy, gm, gF, al, be, ga of the group's stages
    coef[tid] = reinterpret_cast<const float*>(reinterpret_cast<const char*>(A + tid / 8) +
                                               offsetof(StageArgs, gsf))[tid % 8];
  __syncthreads();
  if (tid == 0)
    for (int b = 0; b < K::NSET; ++b)
      if ((int)blockIdx.x + b * (int)gridDim.x < ntiles) issue(b, blockIdx.x + b * gridDim.x);

  bool failed = false;
  int k       = 0;
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x, ++k)
  {
    const int b  = k % K::NSET;
    const int x0 = (t % tiles_x) * FOW, y0 = (t / tiles_x) * K::TH;
    float* arr0  = arr(b, 0); // d_{j-1}, then stages j+1, j+3
    float* arr1  = arr(b, 1); // d_{j-2}, then stages j, j+2
    const float* f0s = arr(b, 2);
    float2* sys  = reinterpret_cast<float2*>(arr(b, 3)); // Sy rows, then Syy rows, duplicated
    // the forcing columns of this lane and the forcing rows of the tile load while the tile's
    // copies are in flight (all loads issued before the first shared-memory store)
    const int x        = x0 - FH + c; // global column of this lane's first point
    const bool quad_in = x >= 0 && x < nx; // nx % 4 == 0: a quad is wholly inside or outside
    const bool store_q = lane >= 1 && lane <= 30 && quad_in && STS_IN_BOUNDS(x + 4 <= nx, err);
    float sx[4] = {0.f, 0.f, 0.f, 0.f}, sxx[4] = {0.f, 0.f, 0.f, 0.f};
    if (FORCED && quad_in)
    {
#pragma unroll
      for (int v = 0; v < 4; ++v)
      {
        sx[v]  = __ldg(P.Sxf + x + v);
        sxx[v] = __ldg(P.Sxxf + x + v);
      }
    }
    if (FORCED)
    {
      static_assert(2 * K::AH <= K::NT, "one forcing row per thread");
      const int r = tid % K::AH, y = y0 - FH + r;
      float v = 0.0f;
      if (tid < 2 * K::AH && y >= 0 && y < ny) v = __ldg((tid < K::AH ? P.Syf : P.Syyf) + y);
      if (tid < 2 * K::AH) sys[tid] = make_float2(v, v);
    }
    const bool ok = mbar_wait_bounded(&bar[b], (uint32_t)((k / K::NSET) & 1));
    if (__syncthreads_or(!ok))
    {
      failed = true;
      break;
    }
    // tiles whose loaded region lies inside the domain need no masking of outside points
    const bool interior = x0 - FH >= 0 && x0 + FOW + FH <= nx && y0 - FH >= 0 && y0 + K::TH + FH <= ny;
    auto stages = [&](auto maskc) {
      constexpr bool MASK = decltype(maskc)::value;
#pragma unroll
      for (int l = 0; l < KS; ++l)
      {
        const float* X = (l & 1) ? arr1 : arr0; // d_{j+l-1}: centre and neighbours
        float* Y       = (l & 1) ? arr0 : arr1; // d_{j+l-2} at the point, overwritten by d_{j+l}
        const float* cf = coef + 8 * l;
        const float2 gs = make_float2(cf[0], cf[0]), gx = make_float2(cf[1], cf[1]);
        const float2 gy = make_float2(cf[2], cf[2]), gm = make_float2(cf[3], cf[3]);
        const float2 gF = make_float2(cf[4], cf[4]);
        float Pi[4] = {0.f, 0.f, 0.f, 0.f}, Qi[4] = {0.f, 0.f, 0.f, 0.f};
        if (FORCED)
        {
          const float al = cf[5], be = cf[6], ga = cf[7];
#pragma unroll
          for (int v = 0; v < 4; ++v)
          {
            Pi[v] = __fmaf_rn(al, sx[v], be * sxx[v]);
            Qi[v] = ga * sx[v];
          }
        }
        const float2 pi01 = make_float2(Pi[0], Pi[1]), pi23 = make_float2(Pi[2], Pi[3]);
        const float2 qi01 = make_float2(Qi[0], Qi[1]), qi23 = make_float2(Qi[2], Qi[3]);
        const int h     = KS - 1 - l; // rows of this stage: [-h, TH + h)
        const int rows  = K::TH + 2 * h;
        const int chunk = (rows + K::NW - 1) / K::NW;
        const int ra    = -h + warp * chunk;
        const int rb    = min(ra + chunk, K::TH + h);
        if (ra < rb) // warp-uniform
        {
          // row r from rows r-1, r, r+1 of d_{j+l-1}
          auto row = [&](int r, const float4& up, const float4& cur, const float4& dn) {
            // lanes 0 and 31 get their own value in place of the columns -1 and 128 of the
            // tile, which are not loaded: what they compute lies outside the valid cone
            const float w = __shfl_up_sync(0xffffffffu, cur.w, 1);
            const float e = __shfl_down_sync(0xffffffffu, cur.x, 1);
            float4 m2 = make_float4(0.f, 0.f, 0.f, 0.f);
            if (HAS_M2 || l > 0) m2 = *reinterpret_cast<const float4*>(Y + (r + FH) * FW + c);
            const float4 q0 = *reinterpret_cast<const float4*>(f0s + (r + FH) * FW + c);
            const int y     = y0 + r;
            float2 syj = make_float2(0.f, 0.f), syyj = make_float2(0.f, 0.f);
            if (FORCED)
            {
              syj  = sys[r + FH];
              syyj = sys[K::AH + r + FH];
            }
            // columns (0, 1) and (2, 3) of this lane as pairs (mixed_point per component)
            const float2 o01 = mixed_pair<FORCED>(
              gs, gx, gy, gm, gF, make_float2(cur.x, cur.y), make_float2(w, cur.x), make_float2(cur.y, cur.z),
              make_float2(up.x, up.y), make_float2(dn.x, dn.y), make_float2(m2.x, m2.y), make_float2(q0.x, q0.y), syj,
              pi01, syyj, qi01);
            const float2 o23 = mixed_pair<FORCED>(
              gs, gx, gy, gm, gF, make_float2(cur.z, cur.w), make_float2(cur.y, cur.z), make_float2(cur.w, e),
              make_float2(up.z, up.w), make_float2(dn.z, dn.w), make_float2(m2.z, m2.w), make_float2(q0.z, q0.w), syj,
              pi23, syyj, qi23);
            float4 ov = make_float4(o01.x, o01.y, o23.x, o23.y);
            if (MASK && !(quad_in && y >= 0 && y < ny)) ov = make_float4(0.f, 0.f, 0.f, 0.f);
            if (l < KS - 1) // the last stage is read by no later stage of this group
              *reinterpret_cast<float4*>(Y + (r + FH) * FW + c) = ov;
            if (l >= KS - 2 && r >= 0 && r < K::TH && (!MASK || y < ny) && store_q)
              *reinterpret_cast<float4*>((l == KS - 1 ? o1 : o2) + (long long)y * nx + x) = ov;
          };
          auto ld = [&](int r) { return *reinterpret_cast<const float4*>(X + (r + FH) * FW + c); };
          // three rows per trip: the rows rotate through registers without copies
          float4 a = ld(ra - 1), bq = ld(ra);
          int r = ra;
          for (; r + 2 < rb; r += 3)
          {
            const float4 c1 = ld(r + 1);
            row(r, a, bq, c1);
            const float4 c2 = ld(r + 2);
            row(r + 1, bq, c1, c2);
            const float4 c3 = ld(r + 3);
            row(r + 2, c1, c2, c3);
            a  = c2;
            bq = c3;
          }
          for (; r < rb; ++r)
          {
            const float4 c1 = ld(r + 1);
            row(r, a, bq, c1);
            a  = bq;
            bq = c1;
          }
        }
        __syncthreads(); // stage l complete before stage l+1 reads its neighbours (and, after
                         // the last stage, before this set is loaded again)
      }
    };
    if (interior) stages(std::false_type{});
    else stages(std::true_type{});
    if (tid == 0)
    {
      const int tn = t + K::NSET * gridDim.x;
      if (tn < ntiles) issue(b, tn);
    }
  }
  if (failed && tid == 0)
  {
    *(volatile int*)err = 1;
    // drain the copies this CTA still has in flight (bounded)
    for (int kk = k; kk < k + K::NSET; ++kk)
    {
      const int tt = blockIdx.x + kk * gridDim.x;
      if (tt >= ntiles) break;
      mbar_wait_bounded(&bar[kk % K::NSET], (uint32_t)((kk / K::NSET) & 1));
    }
  }
}

template <class K, int KS, bool F, bool M2>
bool fused_launch_cfg(const TmaStage32* t, int ti, int num_sms, const ProbDev& P, const StageArgs* A, int im1,
                      int im2, int if0, float* o2, float* o1, int* err, cudaStream_t st)
{
  static bool attr = false;
  if (!attr)
    attr = cudaFuncSetAttribute(stage32_fused_kernel<K, KS, F, M2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                K::SMEM_BYTES) == cudaSuccess;
  if (!attr) return false;
  const CUtensorMap& mm2 = t->fz[ti][im2 >= 0 ? im2 : im1];
  const long long tiles  = ((P.nx + FOW - 1) / FOW) * ((P.ny + K::TH - 1) / K::TH);
  const long long cap    = (long long)num_sms * K::MINB;
  const int grid         = (int)(tiles < cap ? tiles : cap);
  stage32_fused_kernel<K, KS, F, M2><<<grid, K::NT, K::SMEM_BYTES, st>>>(t->fz[ti][im1], mm2, t->fzf[ti][if0], P,
                                                                          A, o2, o1, err);
  return true;
}

template <class K, int KS>
bool fused_launch_ks(const TmaStage32* t, int ti, int num_sms, const ProbDev& P, const StageArgs* A, int im1, int im2,
                     int if0, float* o2, float* o1, int* err, cudaStream_t st)
{
  const bool forced = P.kind == STS_PROBLEM_MANUFACTURED;
  if (forced)
    return (im2 >= 0) ? fused_launch_cfg<K, KS, true, true>(t, ti, num_sms, P, A, im1, im2, if0, o2, o1, err, st)
                      : fused_launch_cfg<K, KS, true, false>(t, ti, num_sms, P, A, im1, im2, if0, o2, o1, err, st);
  return (im2 >= 0) ? fused_launch_cfg<K, KS, false, true>(t, ti, num_sms, P, A, im1, im2, if0, o2, o1, err, st)
                    : fused_launch_cfg<K, KS, false, false>(t, ti, num_sms, P, A, im1, im2, if0, o2, o1, err, st);
}

template <class K>
bool fused_launch_any(const TmaStage32* t, int ti, int ks, int num_sms, const ProbDev& P, const StageArgs* A, int im1,
                      int im2, int if0, float* o2, float* o1, int* err, cudaStream_t st)
{
  switch (ks)
  {
  case 2: return fused_launch_ks<K, 2>(t, ti, num_sms, P, A, im1, im2, if0, o2, o1, err, st);
  case 3: return fused_launch_ks<K, 3>(t, ti, num_sms, P, A, im1, im2, if0, o2, o1, err, st);
  case 4: return fused_launch_ks<K, 4>(t, ti, num_sms, P, A, im1, im2, if0, o2, o1, err, st);
  default: return false;
  }
}

// fused-stage tile configurations (output rows per tile, threads, CTAs per SM, tile buffers);
// the autotuner times them on the problem's own buffers
using F0c = FCfg<32, 256, 3, 1>; // 3 x 62 KB of shared memory per SM
using F1c = FCfg<64, 256, 2, 1>; // 2 x 112 KB
using F2c = FCfg<60, 256, 2, 1>; // 2 x 105 KB: stage rows 66..60 split 9/8/8/8 over 8 warps
using F3c = FCfg<64, 384, 2, 1>; // 2 x 112 KB, 12 warps per CTA
using F4c = FCfg<58, 256, 2, 1>; // 2 x 102 KB: stage rows 64..58 split 8 per warp
using F5c = FCfg<64, 256, 1, 2>; // 1 x 224 KB, double buffered, 8 warps

} // namespace

int tma_fused_tile_rows(int ti)
{
  static const int rows[] = {F0c::TH, F1c::TH, F2c::TH, F3c::TH, F4c::TH, F5c::TH};
  return (ti >= 0 && ti < TMA_FUSED_NTILES) ? rows[ti] : 0;
}

const char* tma_fused_config_name(int ti)
{
  static const char* names[] = {"tile120x32_3cta",    "tile120x64_2cta",    "tile120x60_2cta",
                                "tile120x64_2cta384", "tile120x58_2cta",    "tile120x64_1cta256_2buf"};
  return (ti >= 0 && ti < TMA_FUSED_NTILES) ? names[ti] : "none";
}

bool tma_fused_prepare(TmaStage32* t, float* const D[4], float* const Ff[2], long long nx, long long ny)
{
  t->fz_ok = false;
  // the single-stage maps must cover D[3] too: a step's odd stage runs on any two buffers
  if (!t->ok || !D[3] || !tma_stage32_supported(nx, ny)) return false;
  for (int ti = 0; ti < TMA_FUSED_NTILES; ++ti)
  {
    const int th = tma_fused_tile_rows(ti);
    for (int b = 0; b < 4; ++b)
      if (!tma_encode_f32_2d(&t->fz[ti][b], D[b], nx, ny, FW, th + 2 * FH)) return false;
    for (int b = 0; b < 2; ++b)
      if (!tma_encode_f32_2d(&t->fzf[ti][b], Ff[b], nx, ny, FW, th + 2 * FH)) return false;
  }
  t->fz_ok = true;
  return true;
}

bool tma_fused_launch(const TmaStage32* t, int ti, int ks, int num_sms, const ProbDev& P, const StageArgs* A, int im1,
                      int im2, int if0, float* o2, float* o1, int* err, cudaStream_t st)
{
  if (!t->fz_ok || im1 < 0 || im1 > 3 || im2 > 3 || if0 < 0 || if0 > 1) return false;
  switch (ti)
  {
  case 0: return fused_launch_any<F0c>(t, ti, ks, num_sms, P, A, im1, im2, if0, o2, o1, err, st);
  case 1: return fused_launch_any<F1c>(t, ti, ks, num_sms, P, A, im1, im2, if0, o2, o1, err, st);
  case 2: return fused_launch_any<F2c>(t, ti, ks, num_sms, P, A, im1, im2, if0, o2, o1, err, st);
  case 3: return fused_launch_any<F3c>(t, ti, ks, num_sms, P, A, im1, im2, if0, o2, o1, err, st);
  case 4: return fused_launch_any<F4c>(t, ti, ks, num_sms, P, A, im1, im2, if0, o2, o1, err, st);
  case 5: return fused_launch_any<F5c>(t, ti, ks, num_sms, P, A, im1, im2, if0, o2, o1, err, st);
  default: return false;
  }
}
