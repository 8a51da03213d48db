// Mixed (FP32-increment) stage kernel with TMA tile loads and an mbarrier pipeline.
//
// Persistent CTAs (256 threads, one or two per SM) walk 128-column output tiles of 8-32 rows
// (the tile height, ring depth and CTAs per SM form the configurations the autotuner in
// lsrk.cu times on the problem's own buffers). For each tile the
// CTA's issuing thread starts three bulk tensor copies into one slot of a 3-deep shared
// memory ring: the d_{j-1} tile with a 4-column / 1-row halo (its out-of-range parts are
// zero-filled by the copy engine, which is exactly the homogeneous Dirichlet boundary), the
// d_{j-2} tile and the F_0 tile. Two tiles are always in flight while the CTA computes a
// third, so the bytes in flight per SM no longer depend on registers or occupancy. Each warp
// computes four rows: a lane owns four consecutive columns, the west/east neighbours come
// from the neighbouring lanes by shuffle (the halo columns from shared memory), and the
// rows above/below march through registers. The result goes straight to global memory with
// 16-byte stores. The arithmetic per point is the one of stage32_kernel (kernels.cuh), so
// both kernels give identical bits.
//
// Waits on the pipeline barriers are bounded: a wait that does not complete sets the
// context's error word, the CTA stops issuing, drains (again bounded) the copies it has in
// flight and returns; the host turns the error word into a failed step.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <cstring>
#include <type_traits>

#include "kernels.cuh"
#include "stage_tma.cuh"
#include "sts_internal.cuh"

namespace {

constexpr int TW = 128;                   // output tile width (floats)
constexpr int HW = TW + 8;                // halo tile width (x from x0-4 keeps 16-byte alignment)
constexpr long long WAIT_LIMIT = 1LL << 24;

// Tile / pipeline configuration: TH output rows per tile, NST slots in the shared-memory
// ring, MINB CTAs per SM. The autotuner picks one per problem size.
template <int TH_, int NST_, int MINB_>
struct Cfg {
  static constexpr int TH = TH_, NST = NST_, MINB = MINB_;
  static constexpr int HH = TH + 2;
  static constexpr int HALO_BYTES = HW * HH * 4;
  static constexpr int HALO_PAD   = (HALO_BYTES + 127) / 128 * 128;
  static constexpr int PL_BYTES   = TW * TH * 4;
  static constexpr int SLOT_BYTES = HALO_PAD + 2 * PL_BYTES;
  static constexpr int SMEM_BYTES = NST * SLOT_BYTES + 64; // + the NST pipeline barriers
  static constexpr int RPW = TH / 8;                       // rows per warp (8 warps)
  static_assert(TH % 8 == 0, "8 warps share the tile rows");
};

__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes)
{
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity)
{
  uint32_t ok;
  asm volatile(
    "{\n\t.reg .pred p;\n\t"
    "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
    "selp.u32 %0, 1, 0, p;\n\t}"
    : "=r"(ok)
    : "r"(smem_u32(bar)), "r"(parity)
    : "memory");
  return ok != 0;
}

__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, long long limit = WAIT_LIMIT)
{
  for (long long i = 0; i < limit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y)
{
  asm volatile(
    "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::"r"(
      smem_u32(dst)),
    "l"((uint64_t)map), "r"(smem_u32(bar)), "r"(x), "r"(y)
    : "memory");
}

template <class K, bool HAS_M2>
__device__ __forceinline__ void issue_tile(unsigned char* slot, uint64_t* bar, const CUtensorMap* mh,
                                           const CUtensorMap* mm2, const CUtensorMap* mf0, int tile,
                                           int tiles_x)
{
  const int x0 = (tile % tiles_x) * TW;
  const int y0 = (tile / tiles_x) * K::TH;
  mbar_expect_tx(bar, K::HALO_BYTES + (HAS_M2 ? 2 : 1) * K::PL_BYTES);
  tma_load_2d(slot, mh, bar, x0 - 4, y0 - 1);
  if (HAS_M2) tma_load_2d(slot + K::HALO_PAD, mm2, bar, x0, y0);
  tma_load_2d(slot + K::HALO_PAD + K::PL_BYTES, mf0, bar, x0, y0);
}

template <class K, bool FORCED, bool HAS_M2>
__global__ void __launch_bounds__(256, K::MINB)
  stage32_tma_kernel(const __grid_constant__ CUtensorMap mh, const __grid_constant__ CUtensorMap mm2,
                     const __grid_constant__ CUtensorMap mf0, ProbDev P, const StageArgs* __restrict__ A,
                     float* __restrict__ out, int* err)
{
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + K::NST * K::SLOT_BYTES);
  const int nx = (int)P.nx, ny = (int)P.ny;
  const int tiles_x = (nx + TW - 1) / TW;
  const int ntiles  = tiles_x * ((ny + K::TH - 1) / K::TH);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

  if (tid == 0)
  {
    for (int s = 0; s < K::NST; ++s) mbar_init(&bar[s], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (tid == 0)
    for (int k = 0; k < K::NST; ++k)
    {
      const int t = blockIdx.x + k * gridDim.x;
      if (t < ntiles) issue_tile<K, HAS_M2>(smem + k * K::SLOT_BYTES, &bar[k], &mh, &mm2, &mf0, t, tiles_x);
    }

  const float gs = A->gsf, gx = A->gxf, gy = A->gyf, gm = A->gmf, gF = A->gFf;
  const float al = A->alf, be = A->bef, ga = A->gaf;
  bool failed = false;
  int k       = 0;
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x, ++k)
  {
    const int s             = k % K::NST;
    const uint32_t parity   = (uint32_t)((k / K::NST) & 1);
    const bool ok           = mbar_wait_bounded(&bar[s], parity);
    if (__syncthreads_or(!ok))
    {
      failed = true;
      break;
    }
    const float* halo = reinterpret_cast<const float*>(smem + s * K::SLOT_BYTES);
    const float* m2s  = reinterpret_cast<const float*>(smem + s * K::SLOT_BYTES + K::HALO_PAD);
    const float* f0s  = reinterpret_cast<const float*>(smem + s * K::SLOT_BYTES + K::HALO_PAD + K::PL_BYTES);
    const int x0 = (t % tiles_x) * TW, y0 = (t / tiles_x) * K::TH;
    const int x  = x0 + lane * 4;
    const int c  = 4 + lane * 4; // column of x in the halo tile
    float Pi[4] = {0.f, 0.f, 0.f, 0.f}, Qi[4] = {0.f, 0.f, 0.f, 0.f};
    if (FORCED)
    {
#pragma unroll
      for (int v = 0; v < 4; ++v)
      {
        const bool in = x + v < nx;
        const float sx = in ? __ldg(P.Sxf + x + v) : 0.0f, sxx = in ? __ldg(P.Sxxf + x + v) : 0.0f;
        Pi[v] = __fmaf_rn(al, sx, be * sxx);
        Qi[v] = ga * sx;
      }
    }
    const int r0 = warp * K::RPW; // tile rows r0 .. r0+RPW-1 -> halo rows r0+1 ..
    float4 up  = *reinterpret_cast<const float4*>(halo + (r0 + 0) * HW + c);
    float4 cur = *reinterpret_cast<const float4*>(halo + (r0 + 1) * HW + c);
#pragma unroll
    for (int rr = 0; rr < K::RPW; ++rr)
    {
      const int r    = r0 + rr;
      const float4 dn = *reinterpret_cast<const float4*>(halo + (r + 2) * HW + c);
      float w         = __shfl_up_sync(0xffffffffu, cur.w, 1);
      float e         = __shfl_down_sync(0xffffffffu, cur.x, 1);
      if (lane == 0) w = halo[(r + 1) * HW + 3];
      if (lane == 31) e = halo[(r + 1) * HW + 4 + TW];
      float4 m2 = make_float4(0.f, 0.f, 0.f, 0.f);
      if (HAS_M2) m2 = *reinterpret_cast<const float4*>(m2s + r * TW + lane * 4);
      const float4 q0 = *reinterpret_cast<const float4*>(f0s + r * TW + lane * 4);
      const int y     = y0 + r;
      float syj = 0.0f, syyj = 0.0f;
      if (FORCED && y < ny)
      {
        syj  = __ldg(P.Syf + y);
        syyj = __ldg(P.Syyf + y);
      }
      const float cv[4]  = {cur.x, cur.y, cur.z, cur.w};
      const float uv[4]  = {up.x, up.y, up.z, up.w};
      const float dv[4]  = {dn.x, dn.y, dn.z, dn.w};
      const float mv[4]  = {m2.x, m2.y, m2.z, m2.w};
      const float qv[4]  = {q0.x, q0.y, q0.z, q0.w};
      float o[4];
#pragma unroll
      for (int v = 0; v < 4; ++v)
      {
        const float uw = (v == 0) ? w : cv[v - 1];
        const float ue = (v == 3) ? e : cv[v + 1];
        o[v] = mixed_point<FORCED>(gs, gx, gy, gm, gF, cv[v], uw, ue, uv[v], dv[v], mv[v], qv[v], syj, Pi[v], syyj,
                                   Qi[v]);
      }
      if (y < ny && x < nx && STS_IN_BOUNDS(x + 4 <= nx, err))
        *reinterpret_cast<float4*>(out + (long long)y * nx + x) = make_float4(o[0], o[1], o[2], o[3]);
      up  = cur;
      cur = dn;
    }
    __syncthreads(); // slot s fully read
    if (tid == 0)
    {
      const int tn = t + K::NST * gridDim.x;
      if (tn < ntiles)
      {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        issue_tile<K, HAS_M2>(smem + s * K::SLOT_BYTES, &bar[s], &mh, &mm2, &mf0, tn, tiles_x);
      }
    }
  }
  if (failed && tid == 0)
  {
    *(volatile int*)err = 1;
    // drain the copies this CTA still has in flight (bounded)
    for (int kk = k; kk < k + K::NST; ++kk)
    {
      const int tt = blockIdx.x + kk * gridDim.x;
      if (tt >= ntiles) break;
      mbar_wait_bounded(&bar[kk % K::NST], (uint32_t)((kk / K::NST) & 1));
    }
  }
}

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
// the step end, needs nothing else. Per point the arithmetic is mixed_point with the
// operands of the single-stage kernels, so a group gives the bits of KS single launches.
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
    if (FORCED)
      for (int r = tid; r < 2 * K::AH; r += K::NT)
      {
        const int y   = y0 - FH + (r % K::AH);
        const float v = (y >= 0 && y < ny) ? __ldg((r < K::AH ? P.Syf : P.Syyf) + y) : 0.0f;
        sys[r]        = make_float2(v, v);
      }
    const bool ok = mbar_wait_bounded(&bar[b], (uint32_t)((k / K::NSET) & 1));
    if (__syncthreads_or(!ok))
    {
      failed = true;
      break;
    }
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
          float4 up  = *reinterpret_cast<const float4*>(X + (ra - 1 + FH) * FW + c);
          float4 cur = *reinterpret_cast<const float4*>(X + (ra + FH) * FW + c);
          for (int r = ra; r < rb; ++r)
          {
            const float4 dn = *reinterpret_cast<const float4*>(X + (r + 1 + FH) * FW + c);
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
            *reinterpret_cast<float4*>(Y + (r + FH) * FW + c) = ov;
            if (l >= KS - 2 && r >= 0 && r < K::TH && (!MASK || y < ny) && store_q)
              *reinterpret_cast<float4*>((l == KS - 1 ? o1 : o2) + (long long)y * nx + x) = ov;
            up  = cur;
            cur = dn;
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

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn()
{
  static EncodeTiledFn fn = nullptr;
  if (!fn)
  {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
          cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeTiledFn)p;
  }
  return fn;
}

bool encode(CUtensorMap* m, const float* base, long long nx, long long ny, int bw, int bh)
{
  EncodeTiledFn fn = encode_fn();
  if (!fn) return false;
  cuuint64_t dims[2]    = {(cuuint64_t)nx, (cuuint64_t)ny};
  cuuint64_t strides[1] = {(cuuint64_t)nx * 4};
  cuuint32_t box[2]     = {(cuuint32_t)bw, (cuuint32_t)bh};
  cuuint32_t es[2]      = {1, 1};
  CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void*)base, dims, strides, box, es,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

template <class K, bool F, bool M2>
bool set_smem_attr()
{
  static bool done = false;
  if (!done)
    done = cudaFuncSetAttribute(stage32_tma_kernel<K, F, M2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                K::SMEM_BYTES) == cudaSuccess;
  return done;
}

template <class K, bool F, bool M2>
bool launch_cfg(const TmaStage32* t, int num_sms, const ProbDev& P, const StageArgs* A, int im1, int im2, int if0,
                float* out, int* err, cudaStream_t st)
{
  if (!set_smem_attr<K, F, M2>()) return false;
  const CUtensorMap& mm2 = (im2 >= 0) ? t->plain[K::TH][im2] : t->plain[K::TH][im1];
  const long long tiles = ((P.nx + TW - 1) / TW) * ((P.ny + K::TH - 1) / K::TH);
  const long long cap   = (long long)num_sms * K::MINB;
  const int grid        = (int)(tiles < cap ? tiles : cap);
  stage32_tma_kernel<K, F, M2><<<grid, 256, K::SMEM_BYTES, st>>>(t->halo[K::TH][im1], mm2, t->f0[K::TH][if0], P, A,
                                                                  out, err);
  return true;
}

template <class K>
bool launch_any(const TmaStage32* t, int num_sms, const ProbDev& P, const StageArgs* A, int im1, int im2, int if0,
                float* out, int* err, cudaStream_t st)
{
  const bool forced = P.kind == STS_PROBLEM_MANUFACTURED;
  if (forced)
    return (im2 >= 0) ? launch_cfg<K, true, true>(t, num_sms, P, A, im1, im2, if0, out, err, st)
                      : launch_cfg<K, true, false>(t, num_sms, P, A, im1, im2, if0, out, err, st);
  return (im2 >= 0) ? launch_cfg<K, false, true>(t, num_sms, P, A, im1, im2, if0, out, err, st)
                    : launch_cfg<K, false, false>(t, num_sms, P, A, im1, im2, if0, out, err, st);
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

// fused-stage tile configurations (output rows per tile, threads, CTAs per SM, tile buffers):
// 3 x 61 KB and 2 x 111 KB of shared memory per SM with one tile buffer per CTA; one CTA of
// 512 threads with two 111 KB (64 rows) or two 93 KB (48 rows) tile buffers
using F0c = FCfg<32, 256, 3, 1>;
using F1c = FCfg<64, 256, 2, 1>;
using F2c = FCfg<64, 512, 1, 2>;
using F3c = FCfg<48, 512, 1, 2>;

// the configurations the autotuner chooses from (rows per tile, ring depth, CTAs per SM)
using C0 = Cfg<32, 3, 1>;
using C1 = Cfg<16, 4, 2>;
using C2 = Cfg<16, 6, 1>;
using C3 = Cfg<8, 8, 2>;
using C4 = Cfg<32, 2, 2>;
using C5 = Cfg<24, 4, 1>;

} // namespace

const char* tma_stage32_variant_name(int v)
{
  static const char* names[] = {"tile128x32_ring3_1cta", "tile128x16_ring4_2cta", "tile128x16_ring6_1cta",
                                "tile128x8_ring8_2cta",  "tile128x32_ring2_2cta", "tile128x24_ring4_1cta"};
  return (v >= 0 && v < TMA_STAGE32_NVARIANTS) ? names[v] : "register_marching";
}

bool tma_stage32_supported(long long nx, long long ny)
{
  // 16-byte row pitch and 16-byte aligned x coordinates (multiples of 4 floats); the tile
  // coordinates must fit the copy engine's signed 32-bit coordinates
  return nx % 4 == 0 && nx >= 8 && ny >= 2 && nx < (1LL << 30) && ny < (1LL << 30) && encode_fn() != nullptr;
}

bool tma_stage32_prepare(TmaStage32* t, float* const D[4], float* const Ff[2], long long nx, long long ny)
{
  t->ok = false;
  if (!tma_stage32_supported(nx, ny)) return false;
  const int heights[] = {8, 16, 24, 32};
  for (int th : heights)
  {
    for (int b = 0; b < 4; ++b)
    {
      t->have[b] = false;
      if (!D[b])
      {
        if (b < 3) return false;
        continue;
      }
      if (!encode(&t->halo[th][b], D[b], nx, ny, HW, th + 2)) return false;
      if (!encode(&t->plain[th][b], D[b], nx, ny, TW, th)) return false;
    }
    for (int b = 0; b < 2; ++b)
      if (!encode(&t->f0[th][b], Ff[b], nx, ny, TW, th)) return false;
  }
  for (int b = 0; b < 4; ++b) t->have[b] = D[b] != nullptr;
  t->ok = true;
  return true;
}

int tma_fused_tile_rows(int ti)
{
  static const int rows[] = {F0c::TH, F1c::TH, F2c::TH, F3c::TH};
  return (ti >= 0 && ti < TMA_FUSED_NTILES) ? rows[ti] : 0;
}

const char* tma_fused_config_name(int ti)
{
  static const char* names[] = {"tile120x32_3cta", "tile120x64_2cta", "tile120x64_1cta512_2buf",
                                "tile120x48_1cta512_2buf"};
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
      if (!encode(&t->fz[ti][b], D[b], nx, ny, FW, th + 2 * FH)) return false;
    for (int b = 0; b < 2; ++b)
      if (!encode(&t->fzf[ti][b], Ff[b], nx, ny, FW, th + 2 * FH)) return false;
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
  default: return false;
  }
}

bool tma_stage32_launch(const TmaStage32* t, int variant, int num_sms, const ProbDev& P, const StageArgs* A, int im1,
                        int im2, int if0, float* out, int* err, cudaStream_t st)
{
  // only buffers whose maps were encoded (the caller falls back to the register kernel)
  if (im1 < 0 || im1 > 3 || !t->have[im1] || im2 > 3 || (im2 >= 0 && !t->have[im2]) || if0 < 0 || if0 > 1)
    return false;
  switch (variant)
  {
  case 0: return launch_any<C0>(t, num_sms, P, A, im1, im2, if0, out, err, st);
  case 1: return launch_any<C1>(t, num_sms, P, A, im1, im2, if0, out, err, st);
  case 2: return launch_any<C2>(t, num_sms, P, A, im1, im2, if0, out, err, st);
  case 3: return launch_any<C3>(t, num_sms, P, A, im1, im2, if0, out, err, st);
  case 4: return launch_any<C4>(t, num_sms, P, A, im1, im2, if0, out, err, st);
  case 5: return launch_any<C5>(t, num_sms, P, A, im1, im2, if0, out, err, st);
  default: return false;
  }
}

// Bounded-wait self-test. One warp arms a pipeline barrier (arrival count 1) and waits on its
// first phase with the stage kernel's try_wait loop, `limit` polls at most. With `arrive` set,
// lane 0 arrives before the wait and the phase completes; without it nothing arrives, the wait
// runs out and the kernel writes the context's error word exactly as a stalled tile pipeline
// does, then returns. No copy is in flight, so nothing is left to drain.
static __global__ void wait_selftest_kernel(int arrive, long long limit, int* err)
{
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) mbar_init(&bar, 1);
  __syncthreads();
  if (threadIdx.x == 0 && arrive)
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&bar)) : "memory");
  __syncthreads();
  const bool ok = mbar_wait_bounded(&bar, 0u, limit);
  if (!ok && threadIdx.x == 0) *(volatile int*)err = 1;
}

extern "C" int STS_WaitSelfTest(STS_Context ctx, int arrive, long long limit)
{
  if (!ctx || limit < 1 || limit > (1LL << 20))
  {
    sts_set_error("WaitSelfTest: limit must be in [1, 2^20] polls");
    return STS_ILL_INPUT;
  }
  if (!ctx_activate(ctx)) return STS_ERR_FAILURE;
  if (*(volatile int*)ctx->h_err)
  {
    sts_set_error("WaitSelfTest: the context's error word is already set");
    return STS_ERR_FAILURE;
  }
  wait_selftest_kernel<<<1, 32, 0, ctx->stream>>>(arrive ? 1 : 0, limit, ctx->d_err);
  if (!STS_CUDA_OK(cudaGetLastError()) || !STS_CUDA_OK(cudaStreamSynchronize(ctx->stream))) return STS_ERR_FAILURE;
  if (*(volatile int*)ctx->h_err)
  {
    *ctx->h_err = 0;
    sts_set_error("WaitSelfTest: the barrier wait timed out after %lld polls", limit);
    return STS_ERR_FAILURE;
  }
  return STS_SUCCESS;
}
