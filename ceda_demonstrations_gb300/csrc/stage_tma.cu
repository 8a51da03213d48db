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
#include "tma_util.cuh"

namespace {

constexpr int TW = 128;                   // output tile width (floats)
constexpr int HW = TW + 8;                // halo tile width (x from x0-4 keeps 16-byte alignment)

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

bool tma_encode_f32_2d(CUtensorMap* m, const float* base, long long nx, long long ny, int box_w, int box_h)
{
  return encode(m, base, nx, ny, box_w, box_h);
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
