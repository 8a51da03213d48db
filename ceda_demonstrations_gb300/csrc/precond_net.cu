// Learned multilevel preconditioner with hand-written training and inference kernels. The
// architecture and the gradient formulas follow the CPU reference oracle/convnet.py, against
// which the tests check the output and the gradients:
//
//   z = D (r + E^T E r)        D: Jacobi diagonal, E: 4-level linear encoder, E^T its adjoint
//   x  = [r, r s_k, r s_g] * scale                    h0 = conv(x, W_in)       (3 -> 16, n)
//   h1 = conv(pool(h0), W_1)   h2 = conv(pool(h1), W_2)   h3 = conv(pool(h2), W_3)
//   g3 = h3,  g_l = h_l + poolT(convT(g_{l+1}, W_{l+1})),  u = [1, s_k, s_g] . convT(g0, W_in)
//   z  = D (r + u / scale)
// E^T E is symmetric positive semi-definite, so the preconditioner is SPD for every system
// (an additive multilevel preconditioner with learned level operators), linear in r.
//
// Activations are NHWC BF16 with 16 channels (32 bytes per pixel). The 3x3 convolutions are
// implicit GEMMs on the tensor cores (mma.sync m16n8k16 BF16 -> FP32): a CTA stages a
// (rows+2) x (64+2) pixel tile in shared memory (16-byte halves XOR-swizzled by pixel so
// ldmatrix is conflict-free), each warp computes 16-pixel x 16-channel tiles over the nine
// taps with the weights held in registers as MMA fragments. A transposed convolution is the
// same kernel with the flipped, transposed weights; the weight gradient is a per-tile FP32
// reduction added to global memory with atomics.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <random>
#include <vector>

#include "sts_internal.cuh"

namespace net {

constexpr int CH = 16;
constexpr int NLAYER = 4; // W_in, W_1, W_2, W_3
constexpr int WSZ = CH * CH * 9; // every layer stored as 16 x 16 x 3 x 3 (zero padded)
enum { L_IN = 0, L_1, L_2, L_3 };

// convolution strip: CTA = 4 warps, 64 columns (one 16-pixel m-tile per warp)
constexpr int TC = 64;
constexpr int NTHR = 128;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// swizzled byte offset of (pixel p of a staged row, channel half h): the 16-byte halves are
// XOR-swizzled by pixel so the eight row addresses of an ldmatrix phase hit distinct banks
__device__ __forceinline__ int swz(int p, int h) { return p * 32 + ((h ^ ((p >> 2) & 1)) << 4); }

// Weight fragments: wf[(tap * 2 + nh) * 32 + lane] = {b0b1, b2b3} for n-half nh
// (B[k = ci][n = co], b0b1 = ci (lane%4)*2..+1, b2b3 = ci (lane%4)*2+8..+9, co = nh*8 + lane/4)

// Per-sample metadata of a training pair: {sk, sg, jacobi, scale, 1/(e^T M e), gamma cx, gamma cy}
// (M = I - gamma A on the crop; scale = 1/rms(r) normalises the network input)
constexpr int META = 7;
__device__ __forceinline__ double meta_out_scale(const float* meta, int img)
{
  return (double)meta[META * img + 2] / (double)meta[META * img + 3];
}

// Input of a convolution as the tile loader builds it:
//   LD_PLAIN  BF16 NHWC activations `in`;
//   LD_R64    the network input [v, v sk, v sg, 0, ...] with v = (float)(r * scale), made from
//             the FP64 residual r on the fly (the same roundings as input_kernel_t);
//   LD_UPADD  up(coarse) + in with `coarse` at half resolution (the same roundings as
//             upadd_kernel), so the skip sum is never stored.
enum { LD_PLAIN = 0, LD_R64 = 1, LD_UPADD = 2 };
struct LoadArgs {
  const double* r       = nullptr; // FP64 residual (network input / Jacobi skip)
  const float* r32      = nullptr; // FP32 residual (training batches; Jacobi skip)
  double scale          = 1.0;
  float sk = 0.f, sg    = 0.f;
  const __nv_bfloat16* coarse = nullptr;
  float cscale          = 1.f; // LD_UPADD: in + cscale * up(coarse)
};

// ---------------------------------------------------------------------------------------
// Row-marching convolution: a CTA owns a 64-column strip of one image and marches down a
// segment of rows, keeping a ring of 4 input rows (66 pixels with the halo, swizzled) in
// shared memory. Row y+2 is fetched while row y is computed (cp.async straight into the ring
// for plain BF16 input; for the FP64-residual and skip-sum loaders cp.async of the raw bytes
// three rows ahead into a raw ring, converted one iteration later), so the halo overhead is
// 2 rows per segment and the loads overlap the MMAs.
// Implicit GEMM per row: each warp computes one 16-pixel x 16-channel tile over the nine taps
// (mma.sync m16n8k16 BF16 -> FP32, A by ldmatrix.x4 from the swizzled ring, weights in
// registers as B fragments).
// ---------------------------------------------------------------------------------------
constexpr int MRING = 4;
constexpr int ROWB  = (TC + 2) * 32; // bytes of one staged row

__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src, bool valid)
{
  const int n = valid ? 16 : 0; // zero-fill when the pixel lies outside the image
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(n) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait0() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// Raw staging for the converting loaders (LD_R64, LD_UPADD): the source bytes of a row are
// copied by cp.async into a 4-row raw ring two rows ahead of use; each thread later converts
// exactly the chunks it copied (its own cp.async data needs no barrier), writing the BF16 row
// into the convolution ring. Raw row layout (contiguous, so the 16- and 8-byte accesses of a
// warp are bank-conflict free): LD_UPADD the 132 fine chunks, then the 132 coarse chunks
// above them; LD_R64 the 66 residual values.
constexpr int RAWC = (TC + 2) * 2;  // chunks per staged row
constexpr int RAWB = RAWC * 2 * 16;
__device__ __forceinline__ void cp_async8(uint32_t dst, const void* src, bool valid)
{
  const int n = valid ? 8 : 0;
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(dst), "l"(src), "r"(n) : "memory");
}

template <int LOAD>
__device__ __forceinline__ void issue_raw(unsigned char* rs, const __nv_bfloat16* in, int H, int W, int x0, int row,
                                          long long img_pix, const LoadArgs& la, int tid)
{
  for (int c = tid; c < (TC + 2) * 2; c += NTHR)
  {
    const int h = c & 1, tx = c >> 1, gx = x0 + tx - 1;
    const bool valid = row >= 0 && row < H && gx >= 0 && gx < W;
    if (LOAD == LD_R64)
    {
      if (h == 0)
        cp_async8(smem_u32(rs + tx * 8), valid ? (const void*)(la.r + img_pix + (long long)row * W + gx) : (const void*)la.r,
                  valid);
    }
    else
    {
      cp_async16(smem_u32(rs + c * 16), valid ? (const void*)(in + ((long long)row * W + gx) * CH + h * 8) : (const void*)in,
                 valid);
      cp_async16(smem_u32(rs + (RAWC + c) * 16),
                 valid ? (const void*)(la.coarse + (img_pix / 4 + (long long)(row / 2) * (W / 2) + gx / 2) * CH + h * 8)
                       : (const void*)la.coarse,
                 valid);
    }
  }
}

template <int LOAD>
__device__ __forceinline__ void convert_raw(const unsigned char* rs, unsigned char* slot, const LoadArgs& la, int tid)
{
  for (int c = tid; c < (TC + 2) * 2; c += NTHR)
  {
    const int h = c & 1, tx = c >> 1;
    uint4 v = make_uint4(0, 0, 0, 0);
    if (LOAD == LD_R64)
    {
      if (h == 0)
      {
        const double rv = *reinterpret_cast<const double*>(rs + tx * 8);
        const float xv  = (float)rv * (float)la.scale;
        __nv_bfloat162 c01 = __halves2bfloat162(__float2bfloat16_rn(xv), __float2bfloat16_rn(xv * la.sk));
        __nv_bfloat162 c23 = __halves2bfloat162(__float2bfloat16_rn(xv * la.sg), __float2bfloat16_rn(0.f));
        v.x = *reinterpret_cast<uint32_t*>(&c01);
        v.y = *reinterpret_cast<uint32_t*>(&c23);
      }
    }
    else
    {
      const uint4 f  = *reinterpret_cast<const uint4*>(rs + c * 16);
      const uint4 cc = *reinterpret_cast<const uint4*>(rs + (RAWC + c) * 16);
      const __nv_bfloat162* fb = reinterpret_cast<const __nv_bfloat162*>(&f);
      const __nv_bfloat162* cb = reinterpret_cast<const __nv_bfloat162*>(&cc);
      uint32_t o[4];
#pragma unroll
      for (int k = 0; k < 4; ++k)
      {
        const float2 a = __bfloat1622float2(fb[k]), b = __bfloat1622float2(cb[k]);
        __nv_bfloat162 t = __floats2bfloat162_rn(la.cscale * b.x + a.x, la.cscale * b.y + a.y);
        o[k] = *reinterpret_cast<uint32_t*>(&t);
      }
      v = make_uint4(o[0], o[1], o[2], o[3]);
    }
    *reinterpret_cast<uint4*>(slot + swz(tx, h)) = v;
  }
}

// Epilogue of one 16-pixel m-tile of output row y starting at column xb.
constexpr int STG = 48; // staging bytes per pixel (32 + 16 of padding: conflict-free fragment stores)
// mode 0: BF16 NHWC, 16 channels. Accumulator layout: c0,c1 -> pixel lane/4, channels
// (lane%4)*2..+1; c2,c3 -> pixel lane/4 + 8.
// mode 2: u = c0 + sk c1 + sg c2 (FP32; channel 2 sits in the next lane), redistributed so
// that lanes 0..15 own pixels 0..15, then z = (out_scale u) + (out_scale scale) r in FP64: two
// FP64 instructions per 16 pixels (GB300's FP64 issue rate is 1/64 of FP32).
// POOL: the output rows also go through 2x2 mean pooling (the next level's input, pout): the
// staged BF16 row of an even y is kept and combined with row y+1, in the order of pool_kernel.
template <int MODE, bool POOL = false>
__device__ __forceinline__ void conv_epilogue(const float (&acc)[2][4], int lane, int xb, int y, int W,
                                              long long img_pix, __nv_bfloat16* out, double* out64, double out_scale,
                                              const LoadArgs& la, unsigned char* stage, __nv_bfloat16* pout = nullptr)
{
  const int pr0 = lane >> 2;
  if (MODE == 0)
  {
    // through the warp's staging buffer, so each lane stores one full 16-byte half pixel and
    // the warp writes its 16 pixels x 32 bytes with one coalesced instruction
    unsigned char* st = stage + (POOL ? (y & 1) * 16 * STG : 0);
#pragma unroll
    for (int half = 0; half < 2; ++half)
#pragma unroll
      for (int nh = 0; nh < 2; ++nh)
      {
        const int co = nh * 8 + (lane & 3) * 2;
        __nv_bfloat162 v = __floats2bfloat162_rn(acc[nh][half * 2], acc[nh][half * 2 + 1]);
        *reinterpret_cast<__nv_bfloat162*>(st + (pr0 + half * 8) * STG + co * 2) = v;
      }
    __syncwarp();
    const int px = lane >> 1, gx = xb + px;
    const uint4 v = *reinterpret_cast<const uint4*>(st + px * STG + (lane & 1) * 16);
    if (gx < W) *reinterpret_cast<uint4*>(out + ((long long)y * W + gx) * CH + (lane & 1) * 8) = v;
    if (POOL && (y & 1) && lane < 16)
    {
      // pooled pixel k = lane / 2 of this warp's 8, channel half lane % 2
      const int k = lane >> 1, hb = (lane & 1) * 16, gxc = xb / 2 + k;
      if (2 * gxc < W)
      {
        const unsigned char* r0 = stage;            // row y - 1
        const unsigned char* r1 = stage + 16 * STG; // row y
        const uint4 a = *reinterpret_cast<const uint4*>(r0 + (2 * k) * STG + hb);
        const uint4 b = *reinterpret_cast<const uint4*>(r0 + (2 * k + 1) * STG + hb);
        const uint4 c = *reinterpret_cast<const uint4*>(r1 + (2 * k) * STG + hb);
        const uint4 d = *reinterpret_cast<const uint4*>(r1 + (2 * k + 1) * STG + hb);
        const __nv_bfloat162* A = reinterpret_cast<const __nv_bfloat162*>(&a);
        const __nv_bfloat162* B = reinterpret_cast<const __nv_bfloat162*>(&b);
        const __nv_bfloat162* Cc = reinterpret_cast<const __nv_bfloat162*>(&c);
        const __nv_bfloat162* D = reinterpret_cast<const __nv_bfloat162*>(&d);
        uint32_t o[4];
#pragma unroll
        for (int m = 0; m < 4; ++m)
        {
          const float2 fa = __bfloat1622float2(A[m]), fb = __bfloat1622float2(B[m]), fc = __bfloat1622float2(Cc[m]),
                       fd = __bfloat1622float2(D[m]);
          __nv_bfloat162 t = __floats2bfloat162_rn(0.25f * (fa.x + fb.x + fc.x + fd.x), 0.25f * (fa.y + fb.y + fc.y + fd.y));
          o[m] = *reinterpret_cast<uint32_t*>(&t);
        }
        *reinterpret_cast<uint4*>(pout + ((long long)(y / 2) * (W / 2) + gxc) * CH + (lane & 1) * 8) =
            make_uint4(o[0], o[1], o[2], o[3]);
      }
    }
    __syncwarp();
  }
  else
  {
    const float c2a = __shfl_down_sync(0xffffffffu, acc[0][0], 1);
    const float c2b = __shfl_down_sync(0xffffffffu, acc[0][2], 1);
    const float u0  = acc[0][0] + la.sk * acc[0][1] + la.sg * c2a; // pixel lane/4      (lane%4 == 0)
    const float u1  = acc[0][2] + la.sk * acc[0][3] + la.sg * c2b; // pixel lane/4 + 8
    const int src   = 4 * (lane & 7);
    const float a   = __shfl_sync(0xffffffffu, u0, src);
    const float b   = __shfl_sync(0xffffffffu, u1, src);
    const int gx    = xb + lane;
    if (lane < 16 && gx < W)
    {
      const float u       = lane < 8 ? a : b;
      const long long p   = (long long)y * W + gx;
      const double rv     = la.r ? la.r[img_pix + p] : (la.r32 ? (double)la.r32[img_pix + p] : 0.0);
      out64[p]            = __fma_rn(out_scale * la.scale, rv, (double)((float)out_scale * u));
    }
  }
}

// NARROW: the input has channels 0..7 only (the network input [r, r sk, r sg], or its
// gradient): the MMAs run with K = 8 (m16n8k8, A by ldmatrix.x2), half the tensor work.
template <int MODE, int LOAD = LD_PLAIN, bool NARROW = false, bool POOL = false>
__global__ void __launch_bounds__(NTHR) conv3x3_march_kernel(const __nv_bfloat16* __restrict__ in, int H, int W,
                                                             const uint2* __restrict__ wf,
                                                             __nv_bfloat16* __restrict__ out,
                                                             double* __restrict__ out64, double out_scale,
                                                             const float* __restrict__ meta, LoadArgs la, int rows,
                                                             __nv_bfloat16* __restrict__ pout)
{
  __shared__ __align__(128) unsigned char ring[MRING][ROWB];
  __shared__ __align__(16) unsigned char stage[NTHR / 32][(POOL ? 2 : 1) * 16 * STG]; // per-warp output staging
  __shared__ __align__(16) unsigned char rawring[LOAD == LD_PLAIN ? 1 : MRING][LOAD == LD_PLAIN ? 16 : RAWB];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int x0 = blockIdx.x * TC;
  const int ys = blockIdx.y * rows, ye = min(H, ys + rows);
  const long long img_pix = (long long)H * W * blockIdx.z;
  if (LOAD != LD_R64) in += img_pix * CH;
  if (MODE == 0)
  {
    out += img_pix * CH;
    if (POOL) pout += img_pix / 4 * CH;
  }
  else
  {
    out64 += img_pix;
    if (meta)
    {
      out_scale = meta_out_scale(meta, blockIdx.z);
      la.scale  = (double)meta[META * blockIdx.z + 3];
      la.sk     = meta[META * blockIdx.z];
      la.sg     = meta[META * blockIdx.z + 1];
    }
  }
  if (ys >= H) return;
  auto slot = [&](int r) { return &ring[(r - ys + 1) & (MRING - 1)][0]; };
  auto issue_plain = [&](int r) { // cp.async of row r (zero rows and columns outside the image)
    unsigned char* sl = slot(r);
    for (int c = tid; c < (TC + 2) * 2; c += NTHR)
    {
      const int h = c & 1, tx = c >> 1, gx = x0 + tx - 1;
      const bool valid = r >= 0 && r < H && gx >= 0 && gx < W;
      const __nv_bfloat16* src = valid ? in + ((long long)r * W + gx) * CH + h * 8 : in;
      cp_async16(smem_u32(sl + swz(tx, h)), src, valid);
    }
    cp_async_commit();
  };
  // weights into registers
  uint2 wr[9][2];
#pragma unroll
  for (int t = 0; t < 9; ++t)
#pragma unroll
    for (int nh = 0; nh < 2; ++nh) wr[t][nh] = (MODE == 0 || nh == 0) ? wf[(t * 2 + nh) * 32 + lane] : make_uint2(0, 0);
  auto rawslot = [&](int r) { return &rawring[(r - ys + 1) & (MRING - 1)][0]; };
  auto issue_conv = [&](int r) { // raw copy of row r (rows past ye are not needed: empty group)
    if (r <= ye) issue_raw<LOAD>(rawslot(r), in, H, W, x0, r, img_pix, la, tid);
    cp_async_commit();
  };
  // prologue: rows ys-1, ys, ys+1 staged (and, for the converting loaders, row ys+2 in flight)
  if (LOAD == LD_PLAIN)
  {
    issue_plain(ys - 1);
    issue_plain(ys);
    issue_plain(ys + 1);
  }
  else
  {
    issue_conv(ys - 1);
    issue_conv(ys);
    issue_conv(ys + 1);
    issue_conv(ys + 2);
    cp_async_wait1(); // all but the row ys+2 group
    for (int r = ys - 1; r <= ys + 1; ++r) convert_raw<LOAD>(rawslot(r), slot(r), la, tid);
  }
  for (int y = ys; y < ye; ++y)
  {
    // A: fetch ahead: plain rows land directly in the ring (row y+2); the converting loaders
    // copy raw row y+3 and convert raw row y+2 below
    const bool more = y + 2 <= ye;
    if (LOAD == LD_PLAIN)
    {
      if (more) issue_plain(y + 2);
      else cp_async_commit(); // empty group keeps the wait count uniform
      cp_async_wait1();       // rows up to y+1 have landed
    }
    else
    {
      issue_conv(y + 3);
      cp_async_wait1(); // raw row y+2 (this thread's copies) has landed
    }
    __syncthreads();
    // B: output row y, one 16-pixel m-tile per warp; taps in two independent accumulator
    // chains (rows y-1, y | row y+1) that are added at the end, to overlap MMA latencies
    {
      const int mt = warp;
      float acc[2][4] = {{0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}};
      float acd[2][4] = {{0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}};
#pragma unroll
      for (int t = 0; t < 9; ++t)
      {
        const int dy = t / 3, dx = t % 3;
        const int pi = (lane & 7) + ((lane >> 3) & 1) * 8;
        const int hh = lane >> 4;
        const int px = mt * 16 + pi + dx;
        float(&A)[2][4] = (t < 6) ? acc : acd;
        if constexpr (NARROW)
        {
          // lanes 0-7: pixels 0-7, lanes 8-15: pixels 8-15, channels 0-7 (half 0)
          const unsigned char* rp = slot(y - 1 + dy) + swz(mt * 16 + (lane & 15) + dx, 0);
          uint32_t a0, a1;
          asm volatile("ldmatrix.sync.aligned.m8n8.x2.shared.b16 {%0,%1}, [%2];"
                       : "=r"(a0), "=r"(a1)
                       : "r"(smem_u32(rp)));
#pragma unroll
          for (int nh = 0; nh < (MODE == 0 ? 2 : 1); ++nh)
          {
            asm volatile("mma.sync.aligned.m16n8k8.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5}, {%6}, "
                         "{%0,%1,%2,%3};"
                         : "+f"(A[nh][0]), "+f"(A[nh][1]), "+f"(A[nh][2]), "+f"(A[nh][3])
                         : "r"(a0), "r"(a1), "r"(wr[t][nh].x));
          }
        }
        else
        {
          const unsigned char* rp = slot(y - 1 + dy) + swz(px, hh);
          uint32_t a0, a1, a2, a3;
          asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];"
                       : "=r"(a0), "=r"(a1), "=r"(a2), "=r"(a3)
                       : "r"(smem_u32(rp)));
#pragma unroll
          for (int nh = 0; nh < (MODE == 0 ? 2 : 1); ++nh)
          {
            asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                         "{%0,%1,%2,%3};"
                         : "+f"(A[nh][0]), "+f"(A[nh][1]), "+f"(A[nh][2]), "+f"(A[nh][3])
                         : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(wr[t][nh].x), "r"(wr[t][nh].y));
          }
        }
      }
#pragma unroll
      for (int nh = 0; nh < 2; ++nh)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[nh][q] += acd[nh][q];
      conv_epilogue<MODE, POOL>(acc, lane, x0 + mt * 16, y, W, img_pix, out, out64, out_scale, la, stage[warp], pout);
    }
    // C: convert raw row y+2 into its ring slot (held row y-2, last read before the previous
    // barrier); its raw slot is reused by the copy of row y+6, issued after the barriers of
    // iterations y, y+1 and y+2
    if (LOAD != LD_PLAIN && more) convert_raw<LOAD>(rawslot(y + 2), slot(y + 2), la, tid);
    __syncthreads(); // D: row y's slots free for reuse, row y+2 visible
  }
  cp_async_wait0();
}

// ---------------------------------------------------------------------------------------
// Inference convolution on the 5th-generation tensor cores (tcgen05 + tensor memory).
// A CTA of 128 threads owns a 128-column strip and marches down a segment of rows, two output
// rows per round. Output row y is one UMMA tile D[128 pixels][16 channels] (FP32 in TMEM, 16
// columns; the round's two rows use columns 0-15 and 16-31) accumulated by nine
// tcgen05.mma (M 128, N 16, K 16, BF16) over the 3x3 taps, issued by one thread and
// committed to an mbarrier.
//   Input: each needed input row (130 pixels with the halo; for the skip-sum loader also the
// 66 coarse pixels under it; for the residual loader 132 FP64 values) arrives by a 1-D TMA
// bulk copy into a raw ring, four rows ahead of use, completing on the slot's mbarrier.
// Threads then convert it into the operand ring: canonical K-major layout without swizzle
// (core matrices of 8 rows x 8 channels = 128 bytes, the two channel halves 128 bytes apart,
// 8-row groups 256 bytes apart). UMMA row m stands for output pixel 16 (m % 8) + m / 8, so
// group g + 1 is group g shifted by one pixel: a staged row keeps 18 groups (pixel q = 16 r + g
// at row r of group g; the pixels that also fit as group g + 16 of row r - 1 stored twice) and
// the operand of tap dx is one descriptor moved by dx groups. The conversion's thread-to-
// (pixel, half) map keeps both the raw reads and the operand writes free of bank conflicts.
//   Output: each warp reads its 32 TMEM lanes (tcgen05.ld), the epilogue writes the rows (and
// the pooled row, or the FP64 output) into a staging buffer, and one thread stores it with
// 1-D TMA bulk stores.
// Every wait is bounded: a timeout sets the context's error flag, and the CTA waits (bounded)
// for its copies in flight, frees its tensor memory and returns.
// ---------------------------------------------------------------------------------------
namespace tc {
constexpr int COLS   = 128;            // output pixels per row tile (UMMA M)
constexpr int GROUPS = COLS / 8 + 2;   // 8-row groups of a staged row (shifts 0, 1, 2)
constexpr int SLOTB  = GROUPS * 256;   // operand ring slot: one staged row
constexpr int RING   = 6;              // operand rows: y-1 .. y+2 in use, y+3, y+4 being staged
constexpr int NRAW   = 6;              // raw rows: two being converted, four in flight
constexpr int RAWF   = (COLS + 2) * 32; // raw fine row: pixels x0-1 .. x0+128
constexpr int RAWC   = (COLS / 2 + 2) * 32; // raw coarse row: coarse pixels x0/2-1 .. x0/2+64
constexpr int RAWR   = (COLS + 4) * 8; // raw FP64 row: columns x0-2 .. x0+129
constexpr int WB     = 9 * 512;        // B operands of the nine taps (16 x 16 bf16 each)
constexpr int STAGE  = 2 * COLS * 32 + COLS * 16; // two output rows + one pooled row
template <int LOAD>
struct Cfg {
  static constexpr int RAWB = LOAD == LD_R64 ? RAWR : (LOAD == LD_UPADD ? RAWF + RAWC : RAWF);
  static constexpr int SMEM = RING * SLOTB + NRAW * RAWB + WB + STAGE;
};
// instruction descriptor, kind::f16: D F32, A and B BF16, both K-major, N 16, M 128
constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((16u >> 3) << 17) | ((128u >> 4) << 24);
constexpr long long WAIT_LIMIT = 1LL << 26;

// shared-memory matrix descriptor, K-major without swizzle: leading (channel-half) offset 128 B,
// stride (8-row group) offset 256 B, descriptor version 1 (bit 46)
__device__ __forceinline__ uint64_t sdesc(uint32_t addr)
{
  return (uint64_t)((addr & 0x3FFFF) >> 4) | ((uint64_t)(128 >> 4) << 16) | ((uint64_t)(256 >> 4) << 32) | (1ull << 46);
}
// the output pixel (column offset in the strip) of UMMA row / TMEM lane m
__device__ __forceinline__ int xpix(int m) { return 16 * (m & 7) + (m >> 3); }

__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity)
{
  uint32_t ok;
  asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
               : "=r"(ok)
               : "r"(bar), "r"(parity)
               : "memory");
  return ok != 0;
}
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity)
{
  for (long long i = 0; i < WAIT_LIMIT; ++i)
    if (mbar_try(bar, parity)) return true;
  return false;
}
__device__ __forceinline__ void mbar_init(uint32_t bar) { asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory"); }
__device__ __forceinline__ void mbar_arrive(uint32_t bar)
{
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void mbar_expect(uint32_t bar, uint32_t bytes)
{
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
// 1-D TMA: global -> shared (completes on bar), shared -> global (bulk group)
__device__ __forceinline__ void bulk_load(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar)
{
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}
__device__ __forceinline__ void bulk_store(void* dst, uint32_t src, uint32_t bytes)
{
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(src), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mma(uint32_t tmem, uint64_t a, uint64_t b, uint32_t accumulate)
{
  asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.u32 p, %4, 0;\n\t"
               "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
               "l"(a), "l"(b), "r"(IDESC), "r"(accumulate)
               : "memory");
}
__device__ __forceinline__ void commit(uint32_t bar)
{
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void ld16(uint32_t taddr, float (&v)[16])
{
  uint32_t r[16];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                 "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
               : "r"(taddr)
               : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// TMA of the in-image part of input row `row` into raw slot `raw` (thread 0); bytes issued
template <int LOAD>
__device__ __forceinline__ void issue_row(unsigned char* raw, uint32_t bar, const __nv_bfloat16* in, const LoadArgs& la,
                                          long long img_pix, int H, int W, int row, int x0)
{
  if (row < 0 || row >= H)
  {
    mbar_arrive(bar); // nothing to copy: the phase completes at once
    return;
  }
  if (LOAD == LD_R64)
  {
    const int c0 = max(x0 - 2, 0), c1 = min(x0 + COLS + 2, W); // even bounds: 16-byte aligned
    const uint32_t bytes = (uint32_t)(c1 - c0) * 8;
    mbar_expect(bar, bytes);
    bulk_load(smem_u32(raw + (c0 - (x0 - 2)) * 8), la.r + img_pix + (long long)row * W + c0, bytes, bar);
  }
  else
  {
    const int c0 = max(x0 - 1, 0), c1 = min(x0 + COLS + 1, W);
    const uint32_t fb = (uint32_t)(c1 - c0) * 32;
    uint32_t cb = 0;
    int k0 = 0, k1 = 0;
    if (LOAD == LD_UPADD)
    {
      k0 = max(x0 / 2 - 1, 0);
      k1 = min(x0 / 2 + COLS / 2 + 1, W / 2);
      cb = (uint32_t)(k1 - k0) * 32;
    }
    mbar_expect(bar, fb + cb);
    bulk_load(smem_u32(raw + (c0 - (x0 - 1)) * 32), in + ((long long)row * W + c0) * CH, fb, bar);
    if (LOAD == LD_UPADD)
      bulk_load(smem_u32(raw + RAWF + (k0 - (x0 / 2 - 1)) * 32),
                la.coarse + (img_pix / 4 + (long long)(row / 2) * (W / 2) + k0) * CH, cb, bar);
  }
}

// one 16-byte channel half h of staged pixel q of input row `row` from the raw slot, with the
// roundings of convert_raw (zero outside the image)
template <int LOAD>
__device__ __forceinline__ uint4 make_half(const unsigned char* raw, const LoadArgs& la, int H, int W, int row, int x0,
                                           int q, int h)
{
  const int c = x0 - 1 + q;
  if (row < 0 || row >= H || c < 0 || c >= W) return make_uint4(0, 0, 0, 0);
  if (LOAD == LD_PLAIN) return *reinterpret_cast<const uint4*>(raw + q * 32 + h * 16);
  if (LOAD == LD_R64)
  {
    if (h) return make_uint4(0, 0, 0, 0);
    const double rv = *reinterpret_cast<const double*>(raw + (q + 1) * 8);
    const float xv  = (float)rv * (float)la.scale;
    __nv_bfloat162 c01 = __halves2bfloat162(__float2bfloat16_rn(xv), __float2bfloat16_rn(xv * la.sk));
    __nv_bfloat162 c23 = __halves2bfloat162(__float2bfloat16_rn(xv * la.sg), __float2bfloat16_rn(0.f));
    return make_uint4(*reinterpret_cast<uint32_t*>(&c01), *reinterpret_cast<uint32_t*>(&c23), 0u, 0u);
  }
  const uint4 f  = *reinterpret_cast<const uint4*>(raw + q * 32 + h * 16);
  const uint4 cc = *reinterpret_cast<const uint4*>(raw + RAWF + (c / 2 - (x0 / 2 - 1)) * 32 + h * 16);
  const __nv_bfloat162* fb = reinterpret_cast<const __nv_bfloat162*>(&f);
  const __nv_bfloat162* cb = reinterpret_cast<const __nv_bfloat162*>(&cc);
  uint32_t w[4];
#pragma unroll
  for (int k = 0; k < 4; ++k)
  {
    const float2 a = __bfloat1622float2(fb[k]), b = __bfloat1622float2(cb[k]);
    __nv_bfloat162 t = __floats2bfloat162_rn(la.cscale * b.x + a.x, la.cscale * b.y + a.y);
    w[k] = *reinterpret_cast<uint32_t*>(&t);
  }
  return make_uint4(w[0], w[1], w[2], w[3]);
}

// raw row -> operand slot. Item i = tid + 128 j (j = 0, 1) is (pixel q = 16 r + g, half h) with
// l = i % 8, p = (i / 8) % 8, g = 4 (i / 64) + l / 2, h = l % 2, r = (l + p) % 8: the eight
// lanes of a 128-byte phase read 16-byte pieces 16 l bytes apart (mod 128) and write operand
// rows r that differ, so neither side has bank conflicts. Threads 0-3 also stage pixels 128
// and 129 (r = 7, g = 16, 17).
template <int LOAD>
__device__ __forceinline__ void convert_row(const unsigned char* raw, unsigned char* slot, const LoadArgs& la, int H,
                                            int W, int row, int x0, int tid)
{
#pragma unroll
  for (int j = 0; j < 2; ++j)
  {
    const int i = tid + COLS * j;
    const int l = i & 7, p = (i >> 3) & 7;
    const int g = 4 * (i >> 6) + (l >> 1), h = l & 1, r = (l + p) & 7;
    const int q = 16 * r + g;
    const uint4 v = make_half<LOAD>(raw, la, H, W, row, x0, q, h);
    *reinterpret_cast<uint4*>(slot + g * 256 + h * 128 + r * 16) = v;
    if (g < 2 && r >= 1) *reinterpret_cast<uint4*>(slot + (g + 16) * 256 + h * 128 + (r - 1) * 16) = v;
  }
  if (tid < 4)
  {
    const int q = COLS + (tid >> 1), h = tid & 1;
    *reinterpret_cast<uint4*>(slot + (q - 112) * 256 + h * 128 + 7 * 16) = make_half<LOAD>(raw, la, H, W, row, x0, q, h);
  }
}
} // namespace tc

// MODE 0: BF16 NHWC output (POOL: also the 2x2 means of the round's row pair into pout, in the
// order of pool_kernel); MODE 2: z = (out_scale scale) r + (double)((float)out_scale u),
// u = c0 + sk c1 + sg c2, as conv_epilogue. wu: the nine taps' B operands (tc_weight_kernel).
// Segments start on even rows and H is even, so every round has two rows.
template <int MODE, int LOAD, bool POOL>
__global__ void __launch_bounds__(tc::COLS) conv3x3_tc_kernel(const __nv_bfloat16* __restrict__ in, int H, int W,
                                                              const uint4* __restrict__ wu,
                                                              __nv_bfloat16* __restrict__ out,
                                                              double* __restrict__ out64, double out_scale, LoadArgs la,
                                                              int rows, __nv_bfloat16* __restrict__ pout, int* err)
{
  using C = tc::Cfg<LOAD>;
  extern __shared__ __align__(128) unsigned char dsm[];
  __shared__ uint32_t tbase;
  __shared__ __align__(8) uint64_t bars[1 + tc::NRAW]; // MMA completion, raw slots
  unsigned char* ring  = dsm;
  unsigned char* rawr  = ring + tc::RING * tc::SLOTB;
  unsigned char* wsm   = rawr + tc::NRAW * C::RAWB;
  unsigned char* stage = wsm + tc::WB;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int x0 = blockIdx.x * tc::COLS;
  const int ys = blockIdx.y * rows, ye = min(H, ys + rows);
  const long long img_pix = (long long)H * W * blockIdx.z;
  if (LOAD != LD_R64) in += img_pix * CH;
  if (MODE == 0)
  {
    out += img_pix * CH;
    if (POOL) pout += img_pix / 4 * CH;
  }
  else out64 += img_pix;
  if (ys >= H) return;
  const int cnt = min(tc::COLS, W - x0); // output pixels of this strip (even)
  const uint32_t mbar = smem_u32(&bars[0]);
  auto rawbar  = [&](int r) { return smem_u32(&bars[1 + (r - ys + 1) % tc::NRAW]); };
  auto rawslot = [&](int r) { return rawr + ((r - ys + 1) % tc::NRAW) * C::RAWB; };
  auto rawpar  = [&](int r) { return (uint32_t)(((r - ys + 1) / tc::NRAW) & 1); };
  auto slot    = [&](int r) { return ring + ((r - ys + 1) % tc::RING) * tc::SLOTB; };
  if (tid == 0)
  {
    for (int k = 0; k <= tc::NRAW; ++k) tc::mbar_init(smem_u32(&bars[k]));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  // raw rows ys-1 .. ys+4 in flight (rows past ye are never needed)
  int issued = ys - 2; // last input row whose copy was issued
  if (tid == 0)
    for (int r = ys - 1; r <= min(ys + 4, ye); ++r) tc::issue_row<LOAD>(rawslot(r), rawbar(r), in, la, img_pix, H, W, r, x0);
  issued = min(ys + 4, ye);
  for (int c = tid; c < 9 * 32; c += tc::COLS) reinterpret_cast<uint4*>(wsm)[c] = wu[c];
  if (warp == 0)
  {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tbase)), "r"(32)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  // operand rows ys-1 .. ys+2
  bool ok = true;
  int converted = ys - 2; // last input row converted into the operand ring
  for (int r = ys - 1; r <= min(ys + 2, ye) && ok; ++r)
  {
    ok = tc::mbar_wait(rawbar(r), rawpar(r));
    if (ok)
    {
      tc::convert_row<LOAD>(rawslot(r), slot(r), la, H, W, r, x0, tid);
      converted = r;
    }
  }
  tc::fence_async_smem();
  tc::fence_before();
  const bool bad0 = __syncthreads_or(!ok);
  tc::fence_after();
  const uint32_t tm    = tbase;
  const uint32_t taddr = tm + ((uint32_t)(warp * 32) << 16);
  const int px         = tc::xpix(tid); // this thread's output pixel offset (TMEM lane tid)
  const int gx         = x0 + px;
  bool failed          = bad0;
  int round            = 0;
  for (int y = ys; y < ye && !failed; y += 2, ++round)
  {
    const bool two = y + 1 < ye;
    // 1. MMAs of rows y, y+1 (operand rows y-1 .. y+2); the previous round's bulk stores
    //    have read the staging buffer before it is rewritten below
    if (tid == 0)
    {
#pragma unroll
      for (int t = 0; t < 9; ++t)
      {
        const int dy = t / 3, dx = t % 3;
        tc::mma(tm, tc::sdesc(smem_u32(slot(y - 1 + dy) + dx * 256)), tc::sdesc(smem_u32(wsm + t * 512)),
                t > 0 ? 1u : 0u);
      }
      if (two)
#pragma unroll
        for (int t = 0; t < 9; ++t)
        {
          const int dy = t / 3, dx = t % 3;
          tc::mma(tm + 16, tc::sdesc(smem_u32(slot(y + dy) + dx * 256)), tc::sdesc(smem_u32(wsm + t * 512)),
                  t > 0 ? 1u : 0u);
        }
      tc::commit(mbar);
      tc::bulk_wait_read();
    }
    // 2. stage operand rows y+3, y+4 (their slots held rows y-3, y-2: read by the last round)
    for (int r = y + 3; r <= min(y + 4, ye) && ok; ++r)
    {
      ok = tc::mbar_wait(rawbar(r), rawpar(r));
      if (ok)
      {
        tc::convert_row<LOAD>(rawslot(r), slot(r), la, H, W, r, x0, tid);
        converted = r;
      }
    }
    tc::fence_async_smem();
    if (__syncthreads_or(!ok))
    {
      failed = true;
      break;
    }
    // 3. raw rows y+5, y+6 into the slots of the rows just converted
    if (tid == 0)
      for (int r = issued + 1; r <= min(y + 6, ye); ++r)
        tc::issue_row<LOAD>(rawslot(r), rawbar(r), in, la, img_pix, H, W, r, x0);
    issued = max(issued, min(y + 6, ye));
    // 4. results of rows y, y+1 into the staging buffer
    ok = tc::mbar_wait(mbar, (uint32_t)(round & 1));
    tc::fence_after();
    float a0[16], a1[16];
    tc::ld16(taddr, a0);
    if (two) tc::ld16(taddr + 16, a1);
    if (MODE == 0)
    {
      uint32_t o0[8], o1[8];
#pragma unroll
      for (int k = 0; k < 8; ++k)
      {
        __nv_bfloat162 v0 = __floats2bfloat162_rn(a0[2 * k], a0[2 * k + 1]);
        __nv_bfloat162 v1 = __floats2bfloat162_rn(a1[2 * k], a1[2 * k + 1]);
        o0[k] = *reinterpret_cast<uint32_t*>(&v0);
        o1[k] = *reinterpret_cast<uint32_t*>(&v1);
      }
      uint4* s0 = reinterpret_cast<uint4*>(stage + px * 32);
      uint4* s1 = reinterpret_cast<uint4*>(stage + tc::COLS * 32 + px * 32);
      s0[0] = make_uint4(o0[0], o0[1], o0[2], o0[3]);
      s0[1] = make_uint4(o0[4], o0[5], o0[6], o0[7]);
      s1[0] = make_uint4(o1[0], o1[1], o1[2], o1[3]);
      s1[1] = make_uint4(o1[4], o1[5], o1[6], o1[7]);
      if (POOL)
      {
        // pixel px + 1 is lane tid + 8 (the next group), in the same warp for even px
        uint32_t n0[8], n1[8];
#pragma unroll
        for (int k = 0; k < 8; ++k)
        {
          n0[k] = __shfl_down_sync(0xffffffffu, o0[k], 8);
          n1[k] = __shfl_down_sync(0xffffffffu, o1[k], 8);
        }
        if (!(px & 1))
        {
          uint32_t q[8];
#pragma unroll
          for (int k = 0; k < 8; ++k)
          {
            const float2 fa = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&o0[k]));
            const float2 fb = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&n0[k]));
            const float2 fc = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&o1[k]));
            const float2 fd = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&n1[k]));
            __nv_bfloat162 t = __floats2bfloat162_rn(0.25f * (fa.x + fb.x + fc.x + fd.x),
                                                     0.25f * (fa.y + fb.y + fc.y + fd.y));
            q[k] = *reinterpret_cast<uint32_t*>(&t);
          }
          uint4* sp = reinterpret_cast<uint4*>(stage + 2 * tc::COLS * 32 + (px / 2) * 32);
          sp[0]     = make_uint4(q[0], q[1], q[2], q[3]);
          sp[1]     = make_uint4(q[4], q[5], q[6], q[7]);
        }
      }
    }
    else if (gx < W)
    {
      double* s64 = reinterpret_cast<double*>(stage);
      const float u0 = a0[0] + la.sk * a0[1] + la.sg * a0[2];
      s64[px]        = __fma_rn(out_scale * la.scale, la.r[img_pix + (long long)y * W + gx], (double)((float)out_scale * u0));
      if (two)
      {
        const float u1     = a1[0] + la.sk * a1[1] + la.sg * a1[2];
        s64[tc::COLS + px] = __fma_rn(out_scale * la.scale, la.r[img_pix + (long long)(y + 1) * W + gx],
                                      (double)((float)out_scale * u1));
      }
    }
    tc::fence_async_smem();
    tc::fence_before();
    if (__syncthreads_or(!ok))
    {
      failed = true;
      break;
    }
    tc::fence_after();
    // 5. bulk stores of the staged rows
    if (tid == 0)
    {
      if (MODE == 0)
      {
        tc::bulk_store(out + ((long long)y * W + x0) * CH, smem_u32(stage), (uint32_t)cnt * 32);
        if (two) tc::bulk_store(out + ((long long)(y + 1) * W + x0) * CH, smem_u32(stage + tc::COLS * 32), (uint32_t)cnt * 32);
        if (POOL)
          tc::bulk_store(pout + ((long long)(y / 2) * (W / 2) + x0 / 2) * CH, smem_u32(stage + 2 * tc::COLS * 32),
                         (uint32_t)cnt * 16);
      }
      else
      {
        tc::bulk_store(out64 + (long long)y * W + x0, smem_u32(stage), (uint32_t)cnt * 8);
        if (two) tc::bulk_store(out64 + (long long)(y + 1) * W + x0, smem_u32(stage + tc::COLS * 8), (uint32_t)cnt * 8);
      }
      tc::bulk_commit();
    }
  }
  if (failed)
  {
    if (tid == 0) atomicExch(err, 2);
    // bounded waits for the copies and MMAs still in flight before the memory is released
    for (int r = converted + 1; r <= issued; ++r) tc::mbar_wait(rawbar(r), rawpar(r));
    tc::mbar_wait(mbar, (uint32_t)(round & 1));
  }
  if (tid == 0) tc::bulk_wait_all();
  tc::fence_before();
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tm), "r"(32) : "memory");
}

// ---------------------------------------------------------------------------------------
// Level 0 collapsed (inference). The input layer sees x = [v, v s_k, v s_g], so
// h0 = conv(x, W_in) = conv(v, F) with F[o][t] = sum_c s_c W_in[o][c][t], and the last adjoint
// layer combined with the output weights is u = conv(g0, G), G[o][t] = F[o][8 - t], with
// g0 = h0 + 0.25 up(y1). Nothing at level 0 needs the 16-channel fine tensors:
//   p0 = pool(h0) is a stride-2 4x4 convolution of v (kernel Kp = the pooled F);
//   conv(h0, G) = conv(v, K), K = sum_o G_o * F_o the 5x5 composition, exact away from the
//     image edges; on the edge rows and columns the part through h0 outside the image is
//     removed by 5-tap 1-D corrections along the edge (and added back once at the corners);
//   conv(0.25 up(y1), G) takes, per fine pixel parity, a 2x2 coarse kernel per channel.
// So the fine level reads v (the FP64 residual) twice and y1 once and writes p0 and z: about
// 32 bytes per fine pixel instead of ~100. p0 runs on the tensor cores (TF32 MMAs), z with
// 25 + 64 FP32 FMAs per fine pixel on the CUDA cores. The folded kernels are formed on the
// host from the BF16 weights and passed as kernel parameters.
// ---------------------------------------------------------------------------------------
namespace l0 {
struct FoldA {
  float Kp[CH][16]; // [o][qy*4 + qx], offsets -1 .. 2 from (2I, 2J)
};
struct FoldB {
  float K[25];            // [sy*5 + sx], offsets -2 .. 2
  float Gc[2][2][CH][4];  // [b][a][o][cy*2 + cx]: fine parity (a, b), coarse offset (cx + a - 1, cy + b - 1)
  float CL[5], CR[5], CT[5], CB[5]; // edge corrections along the edge, offsets -2 .. 2
  float corner[4];        // (0,0), (n-1,0), (0,n-1), (n-1,n-1) add-backs
};
// Both kernels work on 2-D tiles of the coarse grid: the CTA loads its input window (with the
// halo) into shared memory, computes, stores; many small CTAs per SM hide the memory latency.
// The folded weights are kernel parameters indexed with compile-time offsets, so they are read
// from the constant bank as FMA operands and take no registers.
constexpr int PTX = 64, PTY = 4; // p0 tile: coarse columns x rows (256 threads, 8 warps of 32 coarse pixels)
constexpr int ZTX = 32, ZTY = 4; // z tile: coarse cells (128 threads, one 2 x 2 fine cell each)

// p0 = pool(conv(v, F)): stride-2 4x4 convolution as a small GEMM on the tensor cores,
// [coarse pixels x 16 taps] x [16 taps x 16 channels], mma.sync m16n8k8 TF32 -> FP32 (the
// window values and the folded weights rounded to TF32, 10-bit mantissa, below the BF16
// rounding of the output). A warp owns 32 coarse pixels of one tile row (two 16-row M tiles),
// two k steps of 8 taps and two n tiles of 8 channels: 8 MMAs instead of 512 FP32 FMA
// instructions per thread pair of pixels on the CUDA cores.
__device__ __forceinline__ uint32_t tf32_bits(float x)
{
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

__global__ void __launch_bounds__(PTX * PTY) p0_kernel(const double* __restrict__ r, double scale, int n, FoldA fa,
                                                       __nv_bfloat16* __restrict__ p0)
{
  constexpr int WR = 2 * PTY + 2, WC = 2 * PTX + 2; // fine window: rows 2J0-1 .., columns 2I0-1 ..
  __shared__ float vw[WR][WC + 2];
  __shared__ uint32_t kb[CH][16]; // folded weights as TF32 bits, [channel][tap]
  const int tid = threadIdx.x;
  const int nc = n / 2;
  const int I0 = blockIdx.x * PTX, J0 = blockIdx.y * PTY;
  const float fs = (float)scale;
  for (int e = tid; e < WR * WC; e += PTX * PTY)
  {
    const int wr = e / WC, wc = e % WC;
    const int y = 2 * J0 - 1 + wr, x = 2 * I0 - 1 + wc;
    vw[wr][wc] = (y >= 0 && y < n && x >= 0 && x < n) ? (float)__ldg(r + (long long)y * n + x) * fs : 0.f;
  }
  // the tap index is fixed per thread here (tid = c * 16 + k): a uniform constant-bank read
  // per warp and tap is not possible, so the weights go through shared memory once
  kb[tid >> 4][tid & 15] = tf32_bits(fa.Kp[tid >> 4][tid & 15]);
  __syncthreads();
  const int lane = tid & 31, warp = tid >> 5;
  const int g = lane >> 2, t = lane & 3;
  const int ty = warp >> 1;               // tile row of this warp
  const int txw = (warp & 1) * 32;        // first tile column of this warp
  // B fragments (k x n = 8 x 8, column major): b0 = B[t][g], b1 = B[t + 4][g], B[k][c] = Kp[c][k]
  uint32_t b[2][2][2]; // [k step][n tile][reg]
#pragma unroll
  for (int ks = 0; ks < 2; ++ks)
#pragma unroll
    for (int nt = 0; nt < 2; ++nt)
    {
      b[ks][nt][0] = kb[nt * 8 + g][ks * 8 + t];
      b[ks][nt][1] = kb[nt * 8 + g][ks * 8 + t + 4];
    }
  const int J = J0 + ty;
#pragma unroll
  for (int m = 0; m < 2; ++m)
  {
    const int tx0 = txw + m * 16; // tile column of M-tile row 0
    // A fragments (m x k = 16 x 8, row major): a0 = A[g][t], a1 = A[g + 8][t], a2 = A[g][t + 4],
    // a3 = A[g + 8][t + 4]; A[p][k] = v at tap k = 4 qy + qx of pixel tx0 + p
    float d[2][4] = {{0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}};
#pragma unroll
    for (int ks = 0; ks < 2; ++ks)
    {
      uint32_t a[4];
#pragma unroll
      for (int q = 0; q < 4; ++q)
      {
        const int p  = g + ((q & 1) ? 8 : 0);
        const int k  = ks * 8 + t + ((q & 2) ? 4 : 0);
        const int qy = k >> 2, qx = k & 3;
        a[q]         = tf32_bits(vw[2 * ty + qy][2 * (tx0 + p) + qx]);
      }
#pragma unroll
      for (int nt = 0; nt < 2; ++nt)
        asm volatile("mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                     "{%0,%1,%2,%3};"
                     : "+f"(d[nt][0]), "+f"(d[nt][1]), "+f"(d[nt][2]), "+f"(d[nt][3])
                     : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[ks][nt][0]), "r"(b[ks][nt][1]));
    }
    // D fragments: d0 = D[g][2t], d1 = D[g][2t + 1], d2 = D[g + 8][2t], d3 = D[g + 8][2t + 1]
#pragma unroll
    for (int h = 0; h < 2; ++h)
    {
      const int I = I0 + tx0 + g + 8 * h;
      if (I >= nc || J >= nc) continue;
      __nv_bfloat16* dst = p0 + ((long long)J * nc + I) * CH;
#pragma unroll
      for (int nt = 0; nt < 2; ++nt)
      {
        __nv_bfloat162 v = __floats2bfloat162_rn(d[nt][2 * h], d[nt][2 * h + 1]);
        *reinterpret_cast<__nv_bfloat162*>(dst + nt * 8 + 2 * t) = v;
      }
    }
  }
}

// z = (out_scale scale) r + (double)((float)out_scale u), u = conv(v, K) (+ edge corrections)
// + conv(0.25 up(y1), G); thread = one coarse cell, its 2 x 2 fine pixels
__global__ void __launch_bounds__(ZTX * ZTY) z_kernel(const double* __restrict__ r, double scale, double out_scale,
                                                      int n, const __nv_bfloat16* __restrict__ y1, FoldB fb,
                                                      double* __restrict__ z)
{
  constexpr int VR = 2 * ZTY + 4, VC = 2 * ZTX + 4; // fine window: rows 2J0-2 .., columns 2I0-2 ..
  constexpr int YR = ZTY + 2, YC = ZTX + 2;         // coarse window: rows J0-1 .., columns I0-1 ..
  __shared__ float vw[VR][VC + 1];
  __shared__ float4 yw[YR][4][YC];
  const int tid = threadIdx.x, tx = tid % ZTX, ty = tid / ZTX;
  const int nc = n / 2;
  const int I0 = blockIdx.x * ZTX, J0 = blockIdx.y * ZTY;
  const float fs = (float)scale;
  for (int e = tid; e < VR * VC; e += ZTX * ZTY)
  {
    const int wr = e / VC, wc = e % VC;
    const int y = 2 * J0 - 2 + wr, x = 2 * I0 - 2 + wc;
    vw[wr][wc] = (y >= 0 && y < n && x >= 0 && x < n) ? (float)__ldg(r + (long long)y * n + x) * fs : 0.f;
  }
  for (int e = tid; e < YR * YC * 2; e += ZTX * ZTY)
  {
    const int h = e & 1, k = (e >> 1) % YC, wr = (e >> 1) / YC;
    const int cy = J0 - 1 + wr, cx = I0 - 1 + k;
    uint4 q = make_uint4(0, 0, 0, 0);
    if (cy >= 0 && cy < nc && cx >= 0 && cx < nc)
      q = __ldg(reinterpret_cast<const uint4*>(y1 + ((long long)cy * nc + cx) * CH) + h);
    const __nv_bfloat162* bq = reinterpret_cast<const __nv_bfloat162*>(&q);
    const float2 a0 = __bfloat1622float2(bq[0]), a1 = __bfloat1622float2(bq[1]), a2 = __bfloat1622float2(bq[2]),
                 a3 = __bfloat1622float2(bq[3]);
    yw[wr][2 * h][k]     = make_float4(a0.x, a0.y, a1.x, a1.y);
    yw[wr][2 * h + 1][k] = make_float4(a2.x, a2.y, a3.x, a3.y);
  }
  __syncthreads();
  const int I = I0 + tx, J = J0 + ty;
  if (I >= nc || J >= nc) return;
  const long long row0 = (long long)(2 * J) * n;
  const double2 r0 = __ldg(reinterpret_cast<const double2*>(r + row0 + 2 * I));
  const double2 r1 = __ldg(reinterpret_cast<const double2*>(r + row0 + n + 2 * I));
  // conv(v, K): window rows 2ty .. 2ty+5, columns 2tx .. 2tx+5
  float u[2][2] = {{0.f, 0.f}, {0.f, 0.f}};
#pragma unroll
  for (int wy = 0; wy < 6; ++wy)
  {
    float wv[6];
#pragma unroll
    for (int wx = 0; wx < 6; ++wx) wv[wx] = vw[2 * ty + wy][2 * tx + wx];
#pragma unroll
    for (int b = 0; b < 2; ++b)
    {
      const int sy = wy - b;
      if (sy < 0 || sy > 4) continue;
#pragma unroll
      for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int sx = 0; sx < 5; ++sx) u[b][a] = fmaf(fb.K[sy * 5 + sx], wv[a + sx], u[b][a]);
    }
  }
  // edge corrections (image columns / rows 0 and n-1); image column 0 is window column 2 when
  // I0 = 0, image row 0 window row 2 when J0 = 0
  if (I == 0)
#pragma unroll
    for (int b = 0; b < 2; ++b)
#pragma unroll
      for (int d = 0; d < 5; ++d) u[b][0] = fmaf(-fb.CL[d], vw[2 * ty + b + d][2], u[b][0]);
  if (I == nc - 1)
#pragma unroll
    for (int b = 0; b < 2; ++b)
#pragma unroll
      for (int d = 0; d < 5; ++d) u[b][1] = fmaf(-fb.CR[d], vw[2 * ty + b + d][2 * tx + 3], u[b][1]);
  if (J == 0)
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
      for (int d = 0; d < 5; ++d) u[0][a] = fmaf(-fb.CT[d], vw[2][2 * tx + a + d], u[0][a]);
  if (J == nc - 1)
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
      for (int d = 0; d < 5; ++d) u[1][a] = fmaf(-fb.CB[d], vw[2 * ty + 3][2 * tx + a + d], u[1][a]);
  if (I == 0 && J == 0) u[0][0] = fmaf(fb.corner[0], vw[2][2], u[0][0]);
  if (I == nc - 1 && J == 0) u[0][1] = fmaf(fb.corner[1], vw[2][2 * tx + 3], u[0][1]);
  if (I == 0 && J == nc - 1) u[1][0] = fmaf(fb.corner[2], vw[2 * ty + 3][2], u[1][0]);
  if (I == nc - 1 && J == nc - 1) u[1][1] = fmaf(fb.corner[3], vw[2 * ty + 3][2 * tx + 3], u[1][1]);
  // conv(0.25 up(y1), G): coarse rows J-1 .. J+1, columns I-1 .. I+1 (window rows ty .., columns tx ..)
#pragma unroll
  for (int dJ = 0; dJ < 3; ++dJ)
#pragma unroll
    for (int dI = 0; dI < 3; ++dI)
#pragma unroll
      for (int m = 0; m < 4; ++m)
      {
        const float4 yv = yw[ty + dJ][m][tx + dI];
#pragma unroll
        for (int b = 0; b < 2; ++b)
        {
          const int cy = dJ - b;
          if (cy < 0 || cy > 1) continue;
#pragma unroll
          for (int a = 0; a < 2; ++a)
          {
            const int cx = dI - a;
            if (cx < 0 || cx > 1) continue;
            float acc = u[b][a];
            acc       = fmaf(fb.Gc[b][a][4 * m + 0][cy * 2 + cx], yv.x, acc);
            acc       = fmaf(fb.Gc[b][a][4 * m + 1][cy * 2 + cx], yv.y, acc);
            acc       = fmaf(fb.Gc[b][a][4 * m + 2][cy * 2 + cx], yv.z, acc);
            acc       = fmaf(fb.Gc[b][a][4 * m + 3][cy * 2 + cx], yv.w, acc);
            u[b][a]   = acc;
          }
        }
      }
  const double osc = out_scale * scale;
  const float fo   = (float)out_scale;
  double2 z0, z1;
  z0.x = __fma_rn(osc, r0.x, (double)(fo * u[0][0]));
  z0.y = __fma_rn(osc, r0.y, (double)(fo * u[0][1]));
  z1.x = __fma_rn(osc, r1.x, (double)(fo * u[1][0]));
  z1.y = __fma_rn(osc, r1.y, (double)(fo * u[1][1]));
  *reinterpret_cast<double2*>(z + row0 + 2 * I)     = z0;
  *reinterpret_cast<double2*>(z + row0 + n + 2 * I) = z1;
}
} // namespace l0

// The nine taps' B operands (B[n = output channel][k = input channel], K-major without
// swizzle: byte t*512 + (n/8)*256 + (k/8)*128 + (n%8)*16 + (k%8)*2) of a layer, forward or
// transposed (swapped channels, flipped taps), as frag_kernel's weights
__global__ void tc_weight_kernel(const float* __restrict__ W, __nv_bfloat16* __restrict__ wu, int transpose)
{
  const int e = blockIdx.x * blockDim.x + threadIdx.x; // 0 .. 9*256
  if (e >= 9 * 256) return;
  const int t = e >> 8, n = (e >> 4) & 15, k = e & 15;
  const float v = transpose ? W[(k * CH + n) * 9 + (8 - t)] : W[(n * CH + k) * 9 + t];
  wu[t * 256 + (n >> 3) * 128 + (k >> 3) * 64 + (n & 7) * 8 + (k & 7)] = __float2bfloat16_rn(v);
}

// Level transfers, one thread per coarse (pool) or fine (upsampling) pixel and all 16 channels
// as two 16-byte vectors; H, W are the fine level's (H counts the rows of all stacked images).
// Index arithmetic in 32 bits (at most 2^31 pixels per level).
struct V16 {
  float v[CH];
};
__device__ __forceinline__ void ld16(const __nv_bfloat16* p, V16& o)
{
  const uint4 a = *reinterpret_cast<const uint4*>(p), b = *reinterpret_cast<const uint4*>(p + 8);
  const __nv_bfloat162* x = reinterpret_cast<const __nv_bfloat162*>(&a);
  const __nv_bfloat162* y = reinterpret_cast<const __nv_bfloat162*>(&b);
#pragma unroll
  for (int k = 0; k < 4; ++k)
  {
    const float2 f = __bfloat1622float2(x[k]), g = __bfloat1622float2(y[k]);
    o.v[2 * k]         = f.x;
    o.v[2 * k + 1]     = f.y;
    o.v[8 + 2 * k]     = g.x;
    o.v[8 + 2 * k + 1] = g.y;
  }
}
__device__ __forceinline__ void st16(__nv_bfloat16* p, const V16& o)
{
  uint32_t w[8];
#pragma unroll
  for (int k = 0; k < 8; ++k)
  {
    __nv_bfloat162 t = __floats2bfloat162_rn(o.v[2 * k], o.v[2 * k + 1]);
    w[k]             = *reinterpret_cast<uint32_t*>(&t);
  }
  *reinterpret_cast<uint4*>(p)     = make_uint4(w[0], w[1], w[2], w[3]);
  *reinterpret_cast<uint4*>(p + 8) = make_uint4(w[4], w[5], w[6], w[7]);
}

// 2x2 mean pooling (FP32 arithmetic, BF16 storage)
__global__ void pool_kernel(const __nv_bfloat16* __restrict__ in, int H, int W, __nv_bfloat16* __restrict__ out)
{
  const unsigned Wc = (unsigned)W / 2, n = (unsigned)(H / 2) * Wc;
  for (unsigned q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x)
  {
    const unsigned x = q % Wc, y = q / Wc;
    const size_t f = ((size_t)(2 * y) * W + 2 * x) * CH;
    V16 a, b, c, d;
    ld16(in + f, a);
    ld16(in + f + CH, b);
    ld16(in + f + (size_t)W * CH, c);
    ld16(in + f + (size_t)W * CH + CH, d);
#pragma unroll
    for (int k = 0; k < CH; ++k) a.v[k] = 0.25f * (a.v[k] + b.v[k] + c.v[k] + d.v[k]);
    st16(out + (size_t)q * CH, a);
  }
}

// out = cscale * up(coarse) + fine (nearest-neighbour upsampling; cscale 0.25 is the adjoint
// of the 2x2 mean)
__global__ void upadd_kernel(const __nv_bfloat16* __restrict__ coarse, const __nv_bfloat16* __restrict__ fine, int H,
                             int W, float cscale, __nv_bfloat16* __restrict__ out)
{
  const unsigned n = (unsigned)H * (unsigned)W, Wc = (unsigned)W / 2;
  for (unsigned q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x)
  {
    const unsigned x = q % (unsigned)W, y = q / (unsigned)W;
    V16 c, f;
    ld16(coarse + ((size_t)(y / 2) * Wc + x / 2) * CH, c);
    ld16(fine + (size_t)q * CH, f);
#pragma unroll
    for (int k = 0; k < CH; ++k) f.v[k] = cscale * c.v[k] + f.v[k];
    st16(out + (size_t)q * CH, f);
  }
}

// g_fine += 0.25 * up(g_coarse)   (adjoint of the 2x2 mean pooling)
__global__ void poolT_add_kernel(const __nv_bfloat16* __restrict__ gcoarse, int H, int W, __nv_bfloat16* __restrict__ gf)
{
  const unsigned n = (unsigned)H * (unsigned)W, Wc = (unsigned)W / 2;
  for (unsigned q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x)
  {
    const unsigned x = q % (unsigned)W, y = q / (unsigned)W;
    V16 c, f;
    ld16(gcoarse + ((size_t)(y / 2) * Wc + x / 2) * CH, c);
    ld16(gf + (size_t)q * CH, f);
#pragma unroll
    for (int k = 0; k < CH; ++k) f.v[k] = f.v[k] + 0.25f * c.v[k];
    st16(gf + (size_t)q * CH, f);
  }
}

// Energy-norm loss of each image (n x n): d = z - e, L_img = 0.5 d^T M d / (e^T M e) with
// M = I - gamma A on the crop (zero outside). With g = (M d) * out_scale / (e^T M e) * gscale
// the gradient of the last transposed convolution's output channels is [g, sk g, sg g] (BF16);
// adds gscale * sum L_img to *acc.
__global__ void gradz_kernel(long long npix, int n, const double* __restrict__ z, const float* __restrict__ e,
                             double gscale, const float* __restrict__ meta, __nv_bfloat16* __restrict__ g,
                             double* __restrict__ acc)
{
  const long long ip = (long long)n * n;
  double lsum        = 0.0;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < npix; p += (long long)gridDim.x * blockDim.x)
  {
    const int img = (int)(p / ip);
    const int q = (int)(p % ip), i = q % n, j = q / n;
    const float* m = meta + META * img;
    const double gcx = m[5], gcy = m[6];
    auto dd = [&](long long k) { return z[k] - (double)e[k]; };
    const double dc = dd(p);
    const double dw = i > 0 ? dd(p - 1) : 0.0, de = i < n - 1 ? dd(p + 1) : 0.0;
    const double ds = j > 0 ? dd(p - n) : 0.0, dn = j < n - 1 ? dd(p + n) : 0.0;
    const double Md = (1.0 + 2.0 * (gcx + gcy)) * dc - gcx * (dw + de) - gcy * (ds + dn);
    const double inv = (double)m[4];
    lsum += 0.5 * dc * Md * inv;
    const float gv = (float)(Md * inv * meta_out_scale(meta, img) * gscale);
    __align__(16) __nv_bfloat16 o[CH];
    o[0] = __float2bfloat16_rn(gv); // dL/du expanded over the input channels [1, sk, sg]
    o[1] = __float2bfloat16_rn(gv * m[0]);
    o[2] = __float2bfloat16_rn(gv * m[1]);
#pragma unroll
    for (int c = 3; c < CH; ++c) o[c] = __float2bfloat16_rn(0.f);
    uint4* dst = reinterpret_cast<uint4*>(g + p * CH);
    dst[0]     = reinterpret_cast<uint4*>(o)[0];
    dst[1]     = reinterpret_cast<uint4*>(o)[1];
  }
  for (int m = 16; m >= 1; m >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, m);
  if ((threadIdx.x & 31) == 0 && lsum != 0.0) atomicAdd(acc, lsum * gscale);
}

// per-pair metadata from the harvested crops: scale = 1/rms(r), 1/(e^T M e); one block per pair
__global__ void __launch_bounds__(256) pair_meta_kernel(const float* __restrict__ r, const float* __restrict__ e, int n,
                                                        float sk, float sg, float jac, double gcx, double gcy,
                                                        float* __restrict__ meta)
{
  __shared__ double s1[8], s2[8];
  const long long ip = (long long)n * n;
  const float* rp    = r + ip * blockIdx.x;
  const float* ep    = e + ip * blockIdx.x;
  double a = 0.0, b = 0.0;
  for (long long q = threadIdx.x; q < ip; q += blockDim.x)
  {
    const int i = (int)(q % n), j = (int)(q / n);
    const double rv = rp[q];
    a += rv * rv;
    const double ec = ep[q];
    const double ew = i > 0 ? ep[q - 1] : 0.0, ee = i < n - 1 ? ep[q + 1] : 0.0;
    const double es = j > 0 ? ep[q - n] : 0.0, en = j < n - 1 ? ep[q + n] : 0.0;
    b += ec * ((1.0 + 2.0 * (gcx + gcy)) * ec - gcx * (ew + ee) - gcy * (es + en));
  }
  for (int m = 16; m >= 1; m >>= 1)
  {
    a += __shfl_xor_sync(0xffffffffu, a, m);
    b += __shfl_xor_sync(0xffffffffu, b, m);
  }
  if ((threadIdx.x & 31) == 0)
  {
    s1[threadIdx.x >> 5] = a;
    s2[threadIdx.x >> 5] = b;
  }
  __syncthreads();
  if (threadIdx.x == 0)
  {
    double A = 0.0, B = 0.0;
    for (int w = 0; w < 8; ++w)
    {
      A += s1[w];
      B += s2[w];
    }
    float* m = meta + META * blockIdx.x;
    m[0]     = sk;
    m[1]     = sg;
    m[2]     = jac;
    m[3]     = A > 0.0 ? (float)sqrt((double)ip / A) : 1.f;
    m[4]     = B > 0.0 ? (float)(1.0 / B) : 0.f;
    m[5]     = (float)gcx;
    m[6]     = (float)gcy;
  }
}

// weight gradient: dW[co][ci][tap] += sum_p g[p][co] * x[p + tap - 1][ci] over every image
// of the batch. Each CTA walks 16 x 16 tiles (grid-stride over tiles of all images), keeps
// its partial sums in registers and adds them to dW with one atomicAdd per weight.
__global__ void __launch_bounds__(256) wgrad_kernel(const __nv_bfloat16* __restrict__ x, const __nv_bfloat16* __restrict__ g,
                                                   int H, int W, int nimg, float* __restrict__ dW)
{
  __shared__ float xs[18][18][CH];
  __shared__ float gs[16][16][CH];
  const int tid = threadIdx.x;
  const int tx_n = (W + 15) / 16, ty_n = (H + 15) / 16;
  const long long ntiles = (long long)tx_n * ty_n * nimg;
  // 2304 weights / 256 threads = 9 per thread: thread -> (co, ci) pair, all 9 taps
  const int co = tid / CH, ci = tid % CH;
  float acc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (long long tl = blockIdx.x; tl < ntiles; tl += gridDim.x)
  {
    const int img = (int)(tl / ((long long)tx_n * ty_n));
    const int rem = (int)(tl % ((long long)tx_n * ty_n));
    const int x0 = (rem % tx_n) * 16, y0 = (rem / tx_n) * 16;
    const __nv_bfloat16* xi = x + (long long)img * H * W * CH;
    const __nv_bfloat16* gi = g + (long long)img * H * W * CH;
    __syncthreads(); // previous tile consumed
    for (int k = tid; k < 18 * 18 * CH; k += 256)
    {
      const int c = k % CH, px = (k / CH) % 18, py = k / (CH * 18);
      const int gx = x0 + px - 1, gy = y0 + py - 1;
      xs[py][px][c] = (gx >= 0 && gx < W && gy >= 0 && gy < H) ? __bfloat162float(xi[((long long)gy * W + gx) * CH + c]) : 0.f;
    }
    for (int k = tid; k < 16 * 16 * CH; k += 256)
    {
      const int c = k % CH, px = (k / CH) % 16, py = k / (CH * 16);
      const int gx = x0 + px, gy = y0 + py;
      gs[py][px][c] = (gx < W && gy < H) ? __bfloat162float(gi[((long long)gy * W + gx) * CH + c]) : 0.f;
    }
    __syncthreads();
    for (int py = 0; py < 16; ++py)
      for (int px = 0; px < 16; ++px)
      {
        const float gv = gs[py][px][co];
#pragma unroll
        for (int t = 0; t < 9; ++t) acc[t] = fmaf(gv, xs[py + t / 3][px + t % 3][ci], acc[t]);
      }
  }
#pragma unroll
  for (int t = 0; t < 9; ++t)
    if (acc[t] != 0.f) atomicAdd(&dW[(co * CH + ci) * 9 + t], acc[t]);
}

// Adam on FP32 master weights; mask keeps padded entries at zero; writes the BF16 copy
__global__ void adam_kernel(int n, float* __restrict__ w, float* __restrict__ m, float* __restrict__ v,
                            const float* __restrict__ g, const float* __restrict__ mask, float lr, float b1, float b2,
                            float eps, float bc1, float bc2, float gscale)
{
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const float gk = g[k] * gscale;
  m[k] = b1 * m[k] + (1.f - b1) * gk;
  v[k] = b2 * v[k] + (1.f - b2) * gk * gk;
  const float mh = m[k] / bc1, vh = v[k] / bc2;
  w[k] = (w[k] - lr * mh / (sqrtf(vh) + eps)) * mask[k];
}

} // namespace net

// ---------------------------------------------------------------------------------------
// host side: network state, forward / backward, training, inference
// ---------------------------------------------------------------------------------------
namespace net {

// fragment layout of one layer's weights (BF16, see conv3x3_march_kernel); transpose = 1 builds
// the input-gradient weights W'[ci][co][8 - t] = W[co][ci][t]
__global__ void frag_kernel(const float* __restrict__ W, uint2* __restrict__ wf, int transpose)
{
  const int k = blockIdx.x * blockDim.x + threadIdx.x; // 0 .. 9*2*32
  if (k >= 9 * 2 * 32) return;
  const int lane = k & 31, nh = (k >> 5) & 1, t = k >> 6;
  const int co = nh * 8 + (lane >> 2), ci0 = (lane & 3) * 2;
  auto w = [&](int o, int i) -> float {
    return transpose ? W[(i * CH + o) * 9 + (8 - t)] : W[(o * CH + i) * 9 + t];
  };
  __nv_bfloat162 lo = __floats2bfloat162_rn(w(co, ci0), w(co, ci0 + 1));
  __nv_bfloat162 hi = __floats2bfloat162_rn(w(co, ci0 + 8), w(co, ci0 + 9));
  uint2 v;
  v.x   = *reinterpret_cast<uint32_t*>(&lo);
  v.y   = *reinterpret_cast<uint32_t*>(&hi);
  wf[k] = v;
}

// x = [r, r sk, r sg] * scale (BF16 NHWC, channels 3..15 zero); with meta, sk, sg and scale
// are the image's
template <typename T>
__global__ void input_kernel_t(long long npix, long long img_pix, const T* __restrict__ r, double scale, float sk,
                               float sg, const float* __restrict__ meta, __nv_bfloat16* __restrict__ x)
{
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < npix; p += (long long)gridDim.x * blockDim.x)
  {
    if (meta)
    {
      const int img = (int)(p / img_pix);
      sk            = meta[META * img];
      sg            = meta[META * img + 1];
      scale         = (double)meta[META * img + 3];
    }
    const float v = (float)r[p] * (float)scale; // as the first convolution's tile loader
    __align__(16) __nv_bfloat16 o[CH];
    o[0] = __float2bfloat16_rn(v);
    o[1] = __float2bfloat16_rn(v * sk);
    o[2] = __float2bfloat16_rn(v * sg);
#pragma unroll
    for (int c = 3; c < CH; ++c) o[c] = __float2bfloat16_rn(0.f);
    uint4* dst = reinterpret_cast<uint4*>(x + p * CH);
    dst[0]     = reinterpret_cast<uint4*>(o)[0];
    dst[1]     = reinterpret_cast<uint4*>(o)[1];
  }
}

// dst[q] = src[idx[q]] for q < nb samples of `len` floats each (and their metadata)
__global__ void gather_kernel(const float* __restrict__ r, const float* __restrict__ e, const float* __restrict__ meta,
                              const int* __restrict__ idx, int nb, long long len, float* __restrict__ rb,
                              float* __restrict__ eb, float* __restrict__ mb)
{
  const long long n = (long long)nb * len;
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
  {
    const int q = (int)(k / len);
    const long long off = (long long)idx[q] * len + (k % len);
    rb[k] = r[off];
    eb[k] = e[off];
    if (k % len < META) mb[META * q + k % len] = meta[META * idx[q] + k % len];
  }
}

struct Level {
  __nv_bfloat16 *x = nullptr;                     // level 0: network input channels
  __nv_bfloat16 *h = nullptr, *p = nullptr;       // encoder output, pooled input (l >= 1)
  __nv_bfloat16 *g = nullptr, *y = nullptr;       // adjoint-pass sum g_l, convT output y_l (l >= 1)
  __nv_bfloat16 *dg = nullptr, *dy = nullptr, *t = nullptr; // gradients and scratch
};

} // namespace net

struct STS_Net_ {
  STS_Context ctx = nullptr;
  int nmax        = 0;
  long long cap   = 0;       // pixels the level-0 buffers hold (images x n x n)
  float* w        = nullptr; // FP32 master weights, 9 x 2304
  float* mask     = nullptr;
  float *m = nullptr, *v = nullptr, *g = nullptr;
  uint2* wf       = nullptr; // forward fragments, 9 x 576
  uint2* wt       = nullptr; // input-gradient fragments
  __nv_bfloat16* wu  = nullptr; // forward UMMA B operands (tcgen05 inference), 9 x 256 per layer
  __nv_bfloat16* wut = nullptr; // transposed UMMA B operands
  int tensor_path    = 0;       // inference convolutions: 0 mma.sync (faster here), 1 tcgen05 + TMEM
  std::vector<float> win_host;  // W_in (FP32 master) on the host, for the folded level-0 kernels
  bool win_stale     = true;
  bool collapse_l0   = true;    // inference level 0 by the collapsed kernels (l0::p0_kernel, z_kernel)
  net::Level L[4];
  double* z       = nullptr; // FP64 output at the finest level
  double* dacc    = nullptr;
  float *rb = nullptr, *eb = nullptr, *mb = nullptr; // minibatch staging
  int* idx        = nullptr;
  long long adam_t = 0;
};

using net::CH;
using net::WSZ;
using net::NLAYER;
using net::META;

static void* dalloc(size_t bytes, bool* ok)
{
  void* p = nullptr;
  if (!STS_CUDA_OK(cudaMalloc(&p, bytes))) *ok = false;
  return p;
}

static int grid_for(long long n) { return (int)std::min<long long>((n + 255) / 256, 4096); }

static void free_levels(STS_Net nt)
{
  for (auto& L : nt->L)
  {
    cudaFree(L.x);
    cudaFree(L.h);
    cudaFree(L.p);
    cudaFree(L.g);
    cudaFree(L.y);
    cudaFree(L.dg);
    cudaFree(L.dy);
    cudaFree(L.t);
    L = net::Level();
  }
  cudaFree(nt->z);
  cudaFree(nt->rb);
  cudaFree(nt->eb);
  nt->z = nullptr;
  nt->rb = nt->eb = nullptr;
  nt->cap = 0;
}

// activation buffers for `pix` level-0 pixels (a batch of images of one size)
static bool ensure_capacity(STS_Net nt, long long pix)
{
  if (pix <= nt->cap) return true;
  cudaStreamSynchronize(nt->ctx->stream);
  free_levels(nt);
  bool ok = true;
  for (int l = 0; l < 4 && ok; ++l)
  {
    const long long np = (pix >> (2 * l)) * CH * 2;
    if (l == 0) nt->L[l].x = (__nv_bfloat16*)dalloc(np, &ok);
    nt->L[l].h  = (__nv_bfloat16*)dalloc(np, &ok);
    nt->L[l].p  = (__nv_bfloat16*)dalloc(np, &ok);
    nt->L[l].g  = (__nv_bfloat16*)dalloc(np, &ok);
    nt->L[l].y  = (__nv_bfloat16*)dalloc(np, &ok);
    nt->L[l].dg = (__nv_bfloat16*)dalloc(np, &ok);
    nt->L[l].dy = (__nv_bfloat16*)dalloc(np, &ok);
    nt->L[l].t  = (__nv_bfloat16*)dalloc(np, &ok);
  }
  nt->z  = (double*)dalloc((size_t)pix * 8, &ok);
  nt->rb = (float*)dalloc((size_t)pix * 4, &ok);
  nt->eb = (float*)dalloc((size_t)pix * 4, &ok);
  if (!ok)
  {
    free_levels(nt);
    return false;
  }
  nt->cap = pix;
  return true;
}

static void refresh_frags(STS_Net nt)
{
  cudaStream_t st = nt->ctx->stream;
  for (int l = 0; l < NLAYER; ++l)
  {
    net::frag_kernel<<<3, 256, 0, st>>>(nt->w + l * WSZ, nt->wf + l * 576, 0);
    net::frag_kernel<<<3, 256, 0, st>>>(nt->w + l * WSZ, nt->wt + l * 576, 1);
    net::tc_weight_kernel<<<9, 256, 0, st>>>(nt->w + l * WSZ, nt->wu + l * 9 * 256, 0);
    net::tc_weight_kernel<<<9, 256, 0, st>>>(nt->w + l * WSZ, nt->wut + l * 9 * 256, 1);
  }
  nt->win_stale = true;
}

static float bf16_round_host(float x)
{
  uint32_t u;
  std::memcpy(&u, &x, 4);
  u = (u + 0x7FFFu + ((u >> 16) & 1u)) & 0xFFFF0000u;
  float y;
  std::memcpy(&y, &u, 4);
  return y;
}

static int floor_half(int x) { return x >= 0 ? x / 2 : -((1 - x) / 2); }

// the folded level-0 kernels of a system (features s_k, s_g) from the BF16 input-layer weights;
// host work, outside any graph capture (it may copy the weights back once after an update)
static bool l0_prepare(STS_Net nt, float sk, float sg, net::l0::FoldA* fa, net::l0::FoldB* fb)
{
  if (nt->win_stale)
  {
    nt->win_host.resize(WSZ);
    if (!STS_CUDA_OK(cudaMemcpyAsync(nt->win_host.data(), nt->w + net::L_IN * WSZ, WSZ * sizeof(float),
                                     cudaMemcpyDeviceToHost, nt->ctx->stream)) ||
        !STS_CUDA_OK(cudaStreamSynchronize(nt->ctx->stream)))
      return false;
    nt->win_stale = false;
  }
  const float* W = nt->win_host.data();
  double F[CH][9], G[CH][9];
  const double s[3] = {1.0, (double)sk, (double)sg};
  for (int o = 0; o < CH; ++o)
    for (int t = 0; t < 9; ++t)
    {
      double f = 0.0;
      for (int c = 0; c < 3; ++c) f += s[c] * (double)bf16_round_host(W[(o * CH + c) * 9 + t]);
      F[o][t] = f;
    }
  for (int o = 0; o < CH; ++o)
    for (int t = 0; t < 9; ++t) G[o][t] = F[o][8 - t];
  double Kp[CH][16] = {}, K[25] = {}, Gc[2][2][CH][4] = {}, C[4][5] = {}, corner[4] = {};
  for (int o = 0; o < CH; ++o)
    for (int dy = 0; dy < 3; ++dy)
      for (int dx = 0; dx < 3; ++dx)
      {
        const double f = F[o][dy * 3 + dx], g = G[o][dy * 3 + dx];
        for (int b = 0; b < 2; ++b)
          for (int a = 0; a < 2; ++a)
          {
            Kp[o][(b + dy) * 4 + (a + dx)] += 0.25 * f;
            const int cx = floor_half(a + dx - 1) - (a - 1), cy = floor_half(b + dy - 1) - (b - 1);
            Gc[b][a][o][cy * 2 + cx] += 0.25 * g;
          }
        for (int ey = 0; ey < 3; ++ey)
          for (int ex = 0; ex < 3; ++ex) K[(dy + ey) * 5 + (dx + ex)] += g * F[o][ey * 3 + ex];
      }
  for (int o = 0; o < CH; ++o)
  {
    for (int d = 0; d < 3; ++d)
      for (int e = 0; e < 3; ++e)
      {
        C[0][d + e] += G[o][d * 3 + 0] * F[o][e * 3 + 2]; // left edge (column 0)
        C[1][d + e] += G[o][d * 3 + 2] * F[o][e * 3 + 0]; // right edge
        C[2][d + e] += G[o][0 * 3 + d] * F[o][2 * 3 + e]; // top edge (row 0)
        C[3][d + e] += G[o][2 * 3 + d] * F[o][0 * 3 + e]; // bottom edge
      }
    corner[0] += G[o][0] * F[o][8];
    corner[1] += G[o][2] * F[o][6];
    corner[2] += G[o][6] * F[o][2];
    corner[3] += G[o][8] * F[o][0];
  }
  for (int o = 0; o < CH; ++o)
    for (int k = 0; k < 16; ++k) fa->Kp[o][k] = (float)Kp[o][k];
  for (int k = 0; k < 25; ++k) fb->K[k] = (float)K[k];
  for (int b = 0; b < 2; ++b)
    for (int a = 0; a < 2; ++a)
      for (int o = 0; o < CH; ++o)
        for (int k = 0; k < 4; ++k) fb->Gc[b][a][o][k] = (float)Gc[b][a][o][k];
  for (int d = 0; d < 5; ++d)
  {
    fb->CL[d] = (float)C[0][d];
    fb->CR[d] = (float)C[1][d];
    fb->CT[d] = (float)C[2][d];
    fb->CB[d] = (float)C[3][d];
  }
  for (int k = 0; k < 4; ++k) fb->corner[k] = (float)corner[k];
  return true;
}

extern "C" STS_Net STS_NetCreate(STS_Context ctx, int nmax, unsigned long long seed)
{
  if (!ctx || nmax < 16 || nmax % 16 != 0)
  {
    sts_set_error("STS_NetCreate: nmax must be a positive multiple of 16");
    return nullptr;
  }
  ctx_activate(ctx);
  STS_Net nt = new STS_Net_();
  nt->ctx    = ctx;
  nt->nmax   = nmax;
  bool ok    = true;
  nt->w    = (float*)dalloc(NLAYER * WSZ * 4, &ok);
  nt->mask = (float*)dalloc(NLAYER * WSZ * 4, &ok);
  nt->m    = (float*)dalloc(NLAYER * WSZ * 4, &ok);
  nt->v    = (float*)dalloc(NLAYER * WSZ * 4, &ok);
  nt->g    = (float*)dalloc(NLAYER * WSZ * 4, &ok);
  nt->wf   = (uint2*)dalloc(NLAYER * 576 * 8, &ok);
  nt->wu   = (__nv_bfloat16*)dalloc(NLAYER * 9 * 256 * 2, &ok);
  nt->wut  = (__nv_bfloat16*)dalloc(NLAYER * 9 * 256 * 2, &ok);
  nt->wt   = (uint2*)dalloc(NLAYER * 576 * 8, &ok);
  nt->dacc = (double*)dalloc(8, &ok);
  if (!ok || !ensure_capacity(nt, (long long)nmax * nmax))
  {
    STS_NetFree(&nt);
    return nullptr;
  }
  // initial weights: N(0, 1/fan_in), zero outside the real channels (W_in: 3 inputs, W_out: 1 output)
  std::vector<float> w(NLAYER * WSZ, 0.f), mask(NLAYER * WSZ, 0.f);
  std::mt19937_64 rng(seed);
  std::normal_distribution<float> nd(0.f, 1.f);
  for (int l = 0; l < NLAYER; ++l)
  {
    const int ci_n = (l == net::L_IN) ? 3 : CH, co_n = CH;
    // small initial weights: the untrained preconditioner is close to Jacobi (E^T E ~ 0.1^4)
    const float sd = std::sqrt(1.0f / (ci_n * 9)) * 0.3f;
    for (int co = 0; co < co_n; ++co)
      for (int ci = 0; ci < ci_n; ++ci)
        for (int t = 0; t < 9; ++t)
        {
          const int k = l * WSZ + (co * CH + ci) * 9 + t;
          w[k]        = nd(rng) * sd;
          mask[k]     = 1.f;
        }
  }
  cudaMemcpy(nt->w, w.data(), w.size() * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(nt->mask, mask.data(), mask.size() * 4, cudaMemcpyHostToDevice);
  cudaMemset(nt->m, 0, NLAYER * WSZ * 4);
  cudaMemset(nt->v, 0, NLAYER * WSZ * 4);
  refresh_frags(nt);
  if (!STS_CUDA_OK(cudaStreamSynchronize(ctx->stream)))
  {
    STS_NetFree(&nt);
    return nullptr;
  }
  return nt;
}

extern "C" int STS_NetFree(STS_Net* pn)
{
  if (!pn || !*pn) return 0;
  STS_Net nt = *pn;
  cudaSetDevice(nt->ctx->device);
  cudaStreamSynchronize(nt->ctx->stream);
  cudaFree(nt->w);
  cudaFree(nt->mask);
  cudaFree(nt->m);
  cudaFree(nt->v);
  cudaFree(nt->g);
  cudaFree(nt->wf);
  cudaFree(nt->wu);
  cudaFree(nt->wut);
  cudaFree(nt->wt);
  cudaFree(nt->dacc);
  cudaFree(nt->mb);
  cudaFree(nt->idx);
  free_levels(nt);
  delete nt;
  *pn = nullptr;
  return 0;
}

// Weights in the order W_in, W_d1, W_d2, W_d3, W_c, W_u2, W_u1, W_u0, W_out, each stored
// as [co][ci][3][3] with 16 x 16 entries (unused channels zero).
extern "C" int STS_NetSetWeights(STS_Net nt, const float* w)
{
  if (!nt || !w) return -1;
  ctx_activate(nt->ctx);
  std::vector<float> mask(NLAYER * WSZ);
  cudaMemcpy(mask.data(), nt->mask, mask.size() * 4, cudaMemcpyDeviceToHost);
  std::vector<float> wm(w, w + NLAYER * WSZ);
  for (size_t k = 0; k < wm.size(); ++k) wm[k] *= mask[k];
  if (!STS_CUDA_OK(cudaMemcpy(nt->w, wm.data(), wm.size() * 4, cudaMemcpyHostToDevice))) return -1;
  refresh_frags(nt);
  return STS_CUDA_OK(cudaStreamSynchronize(nt->ctx->stream)) ? 0 : -1;
}

extern "C" int STS_NetGetWeights(STS_Net nt, float* w)
{
  if (!nt || !w) return -1;
  ctx_activate(nt->ctx);
  cudaStreamSynchronize(nt->ctx->stream);
  return STS_CUDA_OK(cudaMemcpy(w, nt->w, NLAYER * WSZ * 4, cudaMemcpyDeviceToHost)) ? 0 : -1;
}

// launch shape of the row-marching convolution: 64-column strips, row segments sized so that
// the grid holds at least 4 CTAs per SM (each CTA keeps 8.4 KB of rows in flight)
struct MarchGrid {
  dim3 grid;
  int rows;
};
static MarchGrid march_grid(STS_Net nt, int n, int nimg)
{
  const int strips = (n + net::TC - 1) / net::TC;
  const long long want = 16LL * nt->ctx->num_sms; // several waves of up to 7 resident CTAs per SM
  long long segs = (want + (long long)strips * nimg - 1) / ((long long)strips * nimg);
  if (segs < 1) segs = 1;
  int rows = (int)((n + segs - 1) / segs);
  if (rows < 2) rows = 2; // short segments keep the small coarse levels from running on a few CTAs
  rows += rows & 1;       // even: row pairs stay in one CTA (fused pooling)
  MarchGrid m;
  m.rows = rows;
  m.grid = dim3((unsigned)strips, (unsigned)((n + rows - 1) / rows), (unsigned)nimg);
  return m;
}

template <int MODE, int LOAD = net::LD_PLAIN, bool NARROW = false, bool POOL = false>
static void conv_launch(STS_Net nt, const __nv_bfloat16* in, int n, int nimg, const uint2* frags, __nv_bfloat16* out,
                        double* out64, double out_scale, const float* meta, const net::LoadArgs& la,
                        __nv_bfloat16* pout = nullptr)
{
  const MarchGrid m = march_grid(nt, n, nimg);
  net::conv3x3_march_kernel<MODE, LOAD, NARROW, POOL><<<m.grid, net::NTHR, 0, nt->ctx->stream>>>(
      in, n, n, frags, out, out64, out_scale, meta, la, m.rows, pout);
}

// tcgen05 inference convolution: 128-column strips, row segments sized so that the grid is one
// full wave of resident CTAs (even, so the fused pooling's row pairs stay in one CTA)
template <int MODE, int LOAD = net::LD_PLAIN, bool POOL = false>
static void conv_tc(STS_Net nt, const __nv_bfloat16* in, int n, const __nv_bfloat16* wu, __nv_bfloat16* out,
                    double* out64, double out_scale, const net::LoadArgs& la, __nv_bfloat16* pout = nullptr)
{
  static int occ = 0; // resident CTAs per SM
  if (!occ)
  {
    cudaFuncSetAttribute(net::conv3x3_tc_kernel<MODE, LOAD, POOL>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         net::tc::Cfg<LOAD>::SMEM);
    // from the kernel's registers and shared memory (the runtime's occupancy query reports one
    // CTA per SM for kernels that allocate tensor memory; 32 TMEM columns per CTA allow 16)
    cudaFuncAttributes fa;
    occ = 4;
    if (cudaFuncGetAttributes(&fa, net::conv3x3_tc_kernel<MODE, LOAD, POOL>) == cudaSuccess)
    {
      const int regs = (fa.numRegs + 7) / 8 * 8;
      const int by_regs = regs > 0 ? 65536 / (regs * net::tc::COLS) : 16;
      const int by_smem = (227 * 1024) / (net::tc::Cfg<LOAD>::SMEM + (int)fa.sharedSizeBytes + 1024);
      occ               = std::max(1, std::min(std::min(by_regs, by_smem), 16));
    }
  }
  const int strips     = (n + net::tc::COLS - 1) / net::tc::COLS;
  const long long want = (long long)occ * nt->ctx->num_sms; // one full wave
  long long segs       = (want + strips - 1) / strips;
  int rows             = (int)((n + segs - 1) / segs);
  if (rows < 8) rows = 8;
  rows += rows & 1;
  const dim3 grid((unsigned)strips, (unsigned)((n + rows - 1) / rows), 1);
  net::conv3x3_tc_kernel<MODE, LOAD, POOL><<<grid, net::tc::COLS, net::tc::Cfg<LOAD>::SMEM, nt->ctx->stream>>>(
      in, n, n, reinterpret_cast<const uint4*>(wu), out, out64, out_scale, la, rows, pout, nt->ctx->d_err);
}

// convolution (or transposed convolution) with one layer's weights; W_in forward reads the
// 3-channel network input (or its gradient) and runs narrow
static void conv(STS_Net nt, const __nv_bfloat16* in, int n, int nimg, int layer, bool transposed, __nv_bfloat16* out,
                 __nv_bfloat16* pooled = nullptr)
{
  const uint2* frags = (transposed ? nt->wt : nt->wf) + layer * 576;
  const net::LoadArgs la;
  if (layer == net::L_IN && !transposed)
  {
    if (pooled) conv_launch<0, net::LD_PLAIN, true, true>(nt, in, n, nimg, frags, out, nullptr, 0.0, nullptr, la, pooled);
    else conv_launch<0, net::LD_PLAIN, true>(nt, in, n, nimg, frags, out, nullptr, 0.0, nullptr, la);
  }
  else if (pooled) conv_launch<0, net::LD_PLAIN, false, true>(nt, in, n, nimg, frags, out, nullptr, 0.0, nullptr, la, pooled);
  else conv_launch<0>(nt, in, n, nimg, frags, out, nullptr, 0.0, nullptr, la);
}

static void pool(STS_Net nt, const __nv_bfloat16* in, int n, int nimg, __nv_bfloat16* out)
{
  const long long cnt = (long long)n * n * nimg / 4;
  net::pool_kernel<<<grid_for(cnt), 256, 0, nt->ctx->stream>>>(in, n * nimg, n, out);
}

// out = fine + 0.25 up(coarse) (fine at n x n)
static void upadd(STS_Net nt, const __nv_bfloat16* coarse, const __nv_bfloat16* fine, int n, int nimg,
                  __nv_bfloat16* out)
{
  const long long cnt = (long long)n * n * nimg;
  net::upadd_kernel<<<grid_for(cnt), 256, 0, nt->ctx->stream>>>(coarse, fine, n * nimg, n, 0.25f, out);
}

// Training forward over nimg images of n x n (per-image meta), every intermediate stored:
// encoder h_l, p_l; adjoint pass y_l, g_l; output z = D (r + u / scale) into nt->z
template <typename T>
static void net_forward(STS_Net nt, int n, int nimg, const T* r, double scale, float sk, float sg, double out_scale,
                        const float* meta, double* zout = nullptr)
{
  cudaStream_t st = nt->ctx->stream;
  net::Level* L   = nt->L;
  const long long ip = (long long)n * n, np = ip * nimg;
  net::input_kernel_t<T><<<grid_for(np), 256, 0, st>>>(np, ip, r, scale, sk, sg, meta, L[0].x);
  conv(nt, L[0].x, n, nimg, net::L_IN, false, L[0].h, L[1].p);     // h0, p0 (level 1)
  conv(nt, L[1].p, n / 2, nimg, net::L_1, false, L[1].h, L[2].p);  // h1, p1
  conv(nt, L[2].p, n / 4, nimg, net::L_2, false, L[2].h, L[3].p);  // h2, p2
  conv(nt, L[3].p, n / 8, nimg, net::L_3, false, L[3].h);       // h3 = g3
  conv(nt, L[3].h, n / 8, nimg, net::L_3, true, L[3].y);        // y3 = convT(g3, W_3)
  upadd(nt, L[3].y, L[2].h, n / 4, nimg, L[2].g);               // g2 = h2 + poolT(y3)
  conv(nt, L[2].g, n / 4, nimg, net::L_2, true, L[2].y);        // y2
  upadd(nt, L[2].y, L[1].h, n / 2, nimg, L[1].g);               // g1
  conv(nt, L[1].g, n / 2, nimg, net::L_1, true, L[1].y);        // y1
  upadd(nt, L[1].y, L[0].h, n, nimg, L[0].g);                   // g0
  net::LoadArgs la; // Jacobi skip from the network input; sk, sg for the output combination
  if constexpr (sizeof(T) == 8) la.r = reinterpret_cast<const double*>(r);
  else la.r32 = reinterpret_cast<const float*>(r);
  la.scale = scale;
  la.sk    = sk;
  la.sg    = sg;
  conv_launch<2>(nt, L[0].g, n, nimg, nt->wt + net::L_IN * 576, nullptr, zout ? zout : nt->z, out_scale, meta, la); // z
}

// Inference of one n x n residual (FP64, device) into zout: the input channels are built in the
// first convolution's tile loader and the sums g_l = h_l + poolT(y_{l+1}) in the transposed
// convolutions' loaders, so only h_l, p_l and y_l are stored. Bitwise the output of net_forward.
static void net_forward_infer(STS_Net nt, int n, const double* r, double scale, float sk, float sg, double out_scale,
                              double* zout, const net::l0::FoldA* fa = nullptr, const net::l0::FoldB* fb = nullptr)
{
  net::Level* L = nt->L;
  net::LoadArgs la;
  la.r     = r;
  la.scale = scale;
  la.sk    = sk;
  la.sg    = sg;
  net::LoadArgs lu;
  lu.cscale            = 0.25f;
  const bool collapsed = nt->collapse_l0 && fa && fb && n % 2 == 0;
  cudaStream_t st      = nt->ctx->stream;
  if (nt->tensor_path == 1)
  { // tcgen05 + TMEM for the 16-channel levels; level 0 collapsed when it can be
    const net::LoadArgs lp;
    const int WL = 9 * 256;
    if (collapsed)
    {
      const int nc = n / 2;
      dim3 g((unsigned)((nc + net::l0::PTX - 1) / net::l0::PTX), (unsigned)((nc + net::l0::PTY - 1) / net::l0::PTY));
      net::l0::p0_kernel<<<g, net::l0::PTX * net::l0::PTY, 0, st>>>(r, scale, n, *fa, L[1].p); // p0
    }
    else
      conv_tc<0, net::LD_R64, true>(nt, nullptr, n, nt->wu + net::L_IN * WL, L[0].h, nullptr, 0.0, la, L[1].p); // h0, p0
    conv_tc<0, net::LD_PLAIN, true>(nt, L[1].p, n / 2, nt->wu + net::L_1 * WL, L[1].h, nullptr, 0.0, lp, L[2].p); // h1, p1
    conv_tc<0, net::LD_PLAIN, true>(nt, L[2].p, n / 4, nt->wu + net::L_2 * WL, L[2].h, nullptr, 0.0, lp, L[3].p); // h2, p2
    conv_tc<0>(nt, L[3].p, n / 8, nt->wu + net::L_3 * WL, L[3].h, nullptr, 0.0, lp);                             // h3
    conv_tc<0>(nt, L[3].h, n / 8, nt->wut + net::L_3 * WL, L[3].y, nullptr, 0.0, lp);                            // y3
    lu.coarse = L[3].y;
    conv_tc<0, net::LD_UPADD>(nt, L[2].h, n / 4, nt->wut + net::L_2 * WL, L[2].y, nullptr, 0.0, lu); // y2
    lu.coarse = L[2].y;
    conv_tc<0, net::LD_UPADD>(nt, L[1].h, n / 2, nt->wut + net::L_1 * WL, L[1].y, nullptr, 0.0, lu); // y1
    if (collapsed)
    {
      const int nc = n / 2;
      dim3 g((unsigned)((nc + net::l0::ZTX - 1) / net::l0::ZTX), (unsigned)((nc + net::l0::ZTY - 1) / net::l0::ZTY));
      net::l0::z_kernel<<<g, net::l0::ZTX * net::l0::ZTY, 0, st>>>(r, scale, out_scale, n, L[1].y, *fb, zout); // z
      return;
    }
    lu.coarse = L[1].y;
    lu.r      = r;
    lu.scale  = scale;
    lu.sk     = sk;
    lu.sg     = sg;
    conv_tc<2, net::LD_UPADD>(nt, L[0].h, n, nt->wut + net::L_IN * WL, nullptr, zout, out_scale, lu); // z
    return;
  }
  // level 0 collapsed (p0 straight from r, z straight from r and y1), or the mma.sync path
  if (collapsed)
  {
    const int nc = n / 2;
    dim3 g((unsigned)((nc + net::l0::PTX - 1) / net::l0::PTX), (unsigned)((nc + net::l0::PTY - 1) / net::l0::PTY));
    net::l0::p0_kernel<<<g, net::l0::PTX * net::l0::PTY, 0, st>>>(r, scale, n, *fa, L[1].p); // p0
  }
  else
    conv_launch<0, net::LD_R64, true, true>(nt, nullptr, n, 1, nt->wf + net::L_IN * 576, L[0].h, nullptr, 0.0, nullptr,
                                            la, L[1].p); // h0, p0
  conv(nt, L[1].p, n / 2, 1, net::L_1, false, L[1].h, L[2].p);                         // h1, p1
  conv(nt, L[2].p, n / 4, 1, net::L_2, false, L[2].h, L[3].p);                         // h2, p2
  conv(nt, L[3].p, n / 8, 1, net::L_3, false, L[3].h);                                                // h3
  conv(nt, L[3].h, n / 8, 1, net::L_3, true, L[3].y);                                                 // y3
  lu.coarse = L[3].y;
  conv_launch<0, net::LD_UPADD>(nt, L[2].h, n / 4, 1, nt->wt + net::L_2 * 576, L[2].y, nullptr, 0.0, nullptr, lu); // y2
  lu.coarse = L[2].y;
  conv_launch<0, net::LD_UPADD>(nt, L[1].h, n / 2, 1, nt->wt + net::L_1 * 576, L[1].y, nullptr, 0.0, nullptr, lu); // y1
  if (collapsed)
  {
    const int nc = n / 2;
    dim3 g((unsigned)((nc + net::l0::ZTX - 1) / net::l0::ZTX), (unsigned)((nc + net::l0::ZTY - 1) / net::l0::ZTY));
    net::l0::z_kernel<<<g, net::l0::ZTX * net::l0::ZTY, 0, st>>>(r, scale, out_scale, n, L[1].y, *fb, zout); // z
    return;
  }
  lu.coarse = L[1].y;
  lu.r      = r;
  lu.scale  = scale;
  lu.sk     = sk;
  lu.sg     = sg;
  conv_launch<2, net::LD_UPADD>(nt, L[0].h, n, 1, nt->wt + net::L_IN * 576, nullptr, zout, out_scale, nullptr, lu); // z
}

static void wgrad(STS_Net nt, const __nv_bfloat16* x, const __nv_bfloat16* g, int n, int nimg, int layer)
{
  const long long tiles = (long long)((n + 15) / 16) * ((n + 15) / 16) * nimg;
  const int grid        = (int)std::min<long long>(tiles, 2LL * nt->ctx->num_sms);
  net::wgrad_kernel<<<grid, 256, 0, nt->ctx->stream>>>(x, g, n, n, nimg, nt->g + layer * WSZ);
}

// out_fine += 0.25 up(coarse) (adjoint of the 2x2 mean), fine at n x n
static void poolT_add(STS_Net nt, const __nv_bfloat16* coarse, int n, int nimg, __nv_bfloat16* fine)
{
  const long long cnt = (long long)n * n * nimg;
  net::poolT_add_kernel<<<grid_for(cnt), 256, 0, nt->ctx->stream>>>(coarse, n * nimg, n, fine);
}

// Gradient of the energy-norm loss w.r.t. the weights, accumulated into nt->g (and gscale times
// the loss into nt->dacc); needs the preceding net_forward and the per-image meta. Each weight
// is used twice (encoder conv and adjoint-pass convT): a convT(a, W) layer with output
// gradient dy contributes wgrad(x = dy, g = a) and passes conv(dy, W) down; a conv(a, W) layer
// contributes wgrad(x = a, g = dh) and passes convT(dh, W) down.
static void net_backward(STS_Net nt, int n, int nimg, const float* e, double gscale, const float* meta)
{
  cudaStream_t st = nt->ctx->stream;
  net::Level* L   = nt->L;
  const long long ip = (long long)n * n, np = ip * nimg;
  const int m = nimg;
  net::gradz_kernel<<<grid_for(np), 256, 0, st>>>(np, n, nt->z, e, gscale, meta, L[0].dy, nt->dacc); // d gx (3 ch)
  // adjoint pass, top (level 0) to bottom (level 3)
  wgrad(nt, L[0].dy, L[0].g, n, m, net::L_IN);                 // W_in via convT(g0)
  conv(nt, L[0].dy, n, m, net::L_IN, false, L[0].dg);          // d g0 (= d h0 so far)
  pool(nt, L[0].dg, n, m, L[1].dy);                            // d y1
  wgrad(nt, L[1].dy, L[1].g, n / 2, m, net::L_1);
  conv(nt, L[1].dy, n / 2, m, net::L_1, false, L[1].dg);       // d g1 (= d h1 so far)
  pool(nt, L[1].dg, n / 2, m, L[2].dy);                        // d y2
  wgrad(nt, L[2].dy, L[2].g, n / 4, m, net::L_2);
  conv(nt, L[2].dy, n / 4, m, net::L_2, false, L[2].dg);       // d g2 (= d h2 so far)
  pool(nt, L[2].dg, n / 4, m, L[3].dy);                        // d y3
  wgrad(nt, L[3].dy, L[3].h, n / 8, m, net::L_3);              // g3 = h3
  conv(nt, L[3].dy, n / 8, m, net::L_3, false, L[3].dg);       // d h3
  // encoder, bottom to top
  wgrad(nt, L[3].p, L[3].dg, n / 8, m, net::L_3);
  conv(nt, L[3].dg, n / 8, m, net::L_3, true, L[3].t);
  poolT_add(nt, L[3].t, n / 4, m, L[2].dg);                    // d h2 += poolT(convT(d h3))
  wgrad(nt, L[2].p, L[2].dg, n / 4, m, net::L_2);
  conv(nt, L[2].dg, n / 4, m, net::L_2, true, L[2].t);
  poolT_add(nt, L[2].t, n / 2, m, L[1].dg);                    // d h1
  wgrad(nt, L[1].p, L[1].dg, n / 2, m, net::L_1);
  conv(nt, L[1].dg, n / 2, m, net::L_1, true, L[1].t);
  poolT_add(nt, L[1].t, n, m, L[0].dg);                        // d h0
  wgrad(nt, L[0].x, L[0].dg, n, m, net::L_IN);
}

static bool net_size_ok(STS_Net nt, int n)
{
  if (!nt || n < 16 || n % 16 != 0 || n > nt->nmax)
  {
    sts_set_error("STS_Net: size %d must be a multiple of 16 not above %d", n, nt ? nt->nmax : 0);
    return false;
  }
  return true;
}

// z = M r for one n x n residual (device pointers): z = jacobi * net(scale r) / scale
extern "C" int STS_NetSetCollapsedLevel0(STS_Net nt, int on)
{
  if (!nt) return -1;
  nt->collapse_l0 = on != 0;
  return 0;
}

extern "C" int STS_NetSetTensorPath(STS_Net nt, int path)
{
  if (!nt || (path != 0 && path != 1)) return -1;
  nt->tensor_path = path;
  return 0;
}

extern "C" int STS_NetApply(STS_Net nt, int n, const double* r, double* z, double sk, double sg, double jacobi,
                            double scale)
{
  STS_MARK_FUNCTION;
  if (!net_size_ok(nt, n) || !r || !z || !(scale > 0.0)) return -1;
  ctx_activate(nt->ctx);
  net::l0::FoldA fa;
  net::l0::FoldB fb;
  if (!l0_prepare(nt, (float)sk, (float)sg, &fa, &fb)) return -1;
  net_forward_infer(nt, n, r, scale, (float)sk, (float)sg, jacobi / scale, z, &fa, &fb);
  return STS_CUDA_OK(cudaGetLastError()) ? 0 : -1;
}

// one sample (scale 1): loss = 0.5 (z - e)^T M (z - e) / (e^T M e), M = I - gamma A on the
// n x n field with gamma cx = gcx, gamma cy = gcy, and dloss/dW (FP32, host)
extern "C" int STS_NetLossGrad(STS_Net nt, int n, const double* r, const float* e, double sk, double sg, double jacobi,
                               double gcx, double gcy, double* loss, float* grad)
{
  if (!net_size_ok(nt, n) || !r || !e) return -1;
  ctx_activate(nt->ctx);
  cudaStream_t st = nt->ctx->stream;
  const long long np = (long long)n * n;
  // e^T M e on the host (test-sized inputs)
  std::vector<float> eh(np);
  if (!STS_CUDA_OK(cudaMemcpy(eh.data(), e, np * 4, cudaMemcpyDeviceToHost))) return -1;
  double eMe = 0.0;
  for (long long q = 0; q < np; ++q)
  {
    const int i = (int)(q % n), j = (int)(q / n);
    const double c  = eh[q];
    const double w  = i > 0 ? eh[q - 1] : 0.0, ea = i < n - 1 ? eh[q + 1] : 0.0;
    const double so = j > 0 ? eh[q - n] : 0.0, no = j < n - 1 ? eh[q + n] : 0.0;
    eMe += c * ((1.0 + 2.0 * (gcx + gcy)) * c - gcx * (w + ea) - gcy * (so + no));
  }
  if (!nt->mb)
  {
    bool ok = true;
    nt->mb  = (float*)dalloc(META * 4, &ok);
    if (!ok) return -1;
  }
  const float mh[META] = {(float)sk, (float)sg, (float)jacobi, 1.f, (float)(1.0 / eMe), (float)gcx, (float)gcy};
  cudaMemcpyAsync(nt->mb, mh, sizeof(mh), cudaMemcpyHostToDevice, st);
  net_forward<double>(nt, n, 1, r, 1.0, (float)sk, (float)sg, jacobi, nt->mb);
  cudaMemsetAsync(nt->dacc, 0, 8, st);
  cudaMemsetAsync(nt->g, 0, NLAYER * WSZ * 4, st);
  net_backward(nt, n, 1, e, 1.0, nt->mb);
  double l = 0.0;
  cudaMemcpyAsync(&l, nt->dacc, 8, cudaMemcpyDeviceToHost, st);
  if (!STS_CUDA_OK(cudaStreamSynchronize(st))) return -1;
  if (loss) *loss = l;
  if (grad && !STS_CUDA_OK(cudaMemcpy(grad, nt->g, NLAYER * WSZ * 4, cudaMemcpyDeviceToHost))) return -1;
  return 0;
}

// Adam training on nsamples pairs (r_k, e_k) of n x n fields stored as FP32 on the device;
// meta[7k..7k+6] = {sk, sg, jacobi, scale, 1/(e_k^T M e_k), gamma cx, gamma cy}. Each epoch
// visits the samples in a fresh shuffled order in minibatches of `batch` images (gathered into
// a staging buffer and run as one batched forward/backward); loss = mean over the minibatch of
// 0.5 d^T M d / (e^T M e), d = z_k - e_k. Returns the mean loss of the last epoch.
extern "C" int STS_NetTrain(STS_Net nt, int n, int nsamples, const float* r, const float* e, const float* meta,
                            int epochs, int batch, float lr, unsigned long long seed, double* last_loss)
{
  if (!net_size_ok(nt, n) || nsamples < 1 || batch < 1 || epochs < 0 || !r || !e || !meta)
  {
    sts_set_error("STS_NetTrain: invalid arguments");
    return -1;
  }
  ctx_activate(nt->ctx);
  cudaStream_t st = nt->ctx->stream;
  const long long ip = (long long)n * n;
  batch = std::min(batch, nsamples);
  if (!ensure_capacity(nt, ip * batch)) return -1;
  cudaFree(nt->mb);
  cudaFree(nt->idx);
  nt->mb  = nullptr;
  nt->idx = nullptr;
  bool ok = true;
  nt->mb  = (float*)dalloc((size_t)META * batch * 4, &ok);
  nt->idx = (int*)dalloc((size_t)nsamples * 4, &ok);
  if (!ok) return -1;
  std::vector<int> order(nsamples);
  for (int k = 0; k < nsamples; ++k) order[k] = k;
  std::mt19937_64 rng(seed);
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  double epoch_loss = 0.0;
  for (int ep = 0; ep < epochs; ++ep)
  {
    std::shuffle(order.begin(), order.end(), rng);
    cudaMemcpyAsync(nt->idx, order.data(), nsamples * 4, cudaMemcpyHostToDevice, st);
    cudaMemsetAsync(nt->dacc, 0, 8, st);
    int nbatches = 0;
    for (int s0 = 0; s0 + batch <= nsamples; s0 += batch) // whole minibatches only
    {
      const long long len = ip;
      net::gather_kernel<<<grid_for(len * batch), 256, 0, st>>>(r, e, meta, nt->idx + s0, batch, len, nt->rb, nt->eb,
                                                                nt->mb);
      cudaMemsetAsync(nt->g, 0, NLAYER * WSZ * 4, st);
      net_forward<float>(nt, n, batch, nt->rb, 1.0, 0.f, 0.f, 1.0, nt->mb);
      net_backward(nt, n, batch, nt->eb, 1.0 / batch, nt->mb);
      nt->adam_t++;
      const float bc1 = 1.f - powf(b1, (float)nt->adam_t), bc2 = 1.f - powf(b2, (float)nt->adam_t);
      net::adam_kernel<<<(NLAYER * WSZ + 255) / 256, 256, 0, st>>>(NLAYER * WSZ, nt->w, nt->m, nt->v, nt->g, nt->mask, lr,
                                                                 b1, b2, eps, bc1, bc2, 1.f);
      refresh_frags(nt);
      ++nbatches;
    }
    double d2 = 0.0;
    cudaMemcpyAsync(&d2, nt->dacc, 8, cudaMemcpyDeviceToHost, st);
    if (!STS_CUDA_OK(cudaStreamSynchronize(st))) return -1;
    epoch_loss = d2 / (double)nbatches;
  }
  if (last_loss) *last_loss = epoch_loss;
  return 0;
}

// ---------------------------------------------------------------------------------------
// training data from PCG solves, and flexible CG with the network
// ---------------------------------------------------------------------------------------
#include <functional>

int sts_pcg_run(STS_Problem p, double gamma, N_Vector b, N_Vector x, double tol, int maxit, int jacobi, int* iters,
                double* relres, const std::function<void(int, const double*, const double*)>& batch_cb);

namespace net {
// dst (crop x crop FP32) = src (n-wide FP64) window at (x0, y0)
__global__ void crop_kernel(const double* __restrict__ src, long long nx, int x0, int y0, int crop,
                            float* __restrict__ dst)
{
  const long long n = (long long)crop * crop;
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
  {
    const int i = (int)(k % crop), j = (int)(k / crop);
    dst[k] = (float)src[(long long)(y0 + j) * nx + (x0 + i)];
  }
}

// e = x*_crop - e (e holds x_k crops while the solve runs)
__global__ void corr_kernel(const double* __restrict__ xs, long long nx, int x0, int y0, int crop, float* __restrict__ e)
{
  const long long n = (long long)crop * crop;
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
  {
    const int i = (int)(k % crop), j = (int)(k / crop);
    e[k] = (float)(xs[(long long)(y0 + j) * nx + (x0 + i)] - (double)e[k]);
  }
}

} // namespace net

extern "C" int STS_HarvestPCGPairs(STS_Problem p, double gamma, N_Vector b, int ncrops, int crop, int every,
                                   int max_pairs, float* r_out, float* e_out, float* meta_out,
                                   unsigned long long seed, int* npairs, int* iters)
{
  if (!p || !b || crop < 16 || crop > p->nx || crop > p->ny || ncrops < 1 || every < 1 || max_pairs < 1)
  {
    sts_set_error("STS_HarvestPCGPairs: invalid arguments");
    return -1;
  }
  STS_Context ctx = p->ctx;
  ctx_activate(ctx);
  cudaStream_t st = ctx->stream;
  N_Vector x      = N_VNew_Sts(NVL(b), ctx);
  std::mt19937_64 rng(seed);
  std::vector<int> cx(ncrops), cy(ncrops);
  for (int c = 0; c < ncrops; ++c)
  {
    cx[c] = (int)(rng() % (unsigned long long)(p->nx - crop + 1));
    cy[c] = (int)(rng() % (unsigned long long)(p->ny - crop + 1));
  }
  std::vector<int> pair_crop;
  int batch_no      = 0;
  const long long cs = (long long)crop * crop;
  auto cb = [&](int, const double* xk, const double* rk) {
    if ((batch_no++ % every) != 0) return;
    for (int c = 0; c < ncrops && (int)pair_crop.size() < max_pairs; ++c)
    {
      const long long slot = (long long)pair_crop.size();
      net::crop_kernel<<<grid_for(cs), 256, 0, st>>>(rk, p->nx, cx[c], cy[c], crop, r_out + slot * cs);
      net::crop_kernel<<<grid_for(cs), 256, 0, st>>>(xk, p->nx, cx[c], cy[c], crop, e_out + slot * cs);
      pair_crop.push_back(c);
    }
  };
  int it = 0;
  double rel;
  int rc = sts_pcg_run(p, gamma, b, x, 1e-10, 1000000, 1, &it, &rel, cb);
  for (size_t k = 0; k < pair_crop.size(); ++k)
  {
    const int c = pair_crop[k];
    net::corr_kernel<<<grid_for(cs), 256, 0, st>>>(NVD(x), p->nx, cx[c], cy[c], crop, e_out + (long long)k * cs);
  }
  if (meta_out && !pair_crop.empty())
  {
    const double sk  = (std::log10(p->ky / p->kx) + 1.5) / 1.5;
    const double sg  = std::log10(gamma / (p->dx * p->dx)) - 3.6;
    const double jac = 1.0 / (1.0 - gamma * p->cc);
    net::pair_meta_kernel<<<(unsigned)pair_crop.size(), 256, 0, st>>>(r_out, e_out, crop, (float)sk, (float)sg, (float)jac,
                                                                      gamma * p->cx, gamma * p->cy, meta_out);
  }
  STS_CUDA_OK(cudaStreamSynchronize(st));
  N_VDestroy_Sts(x);
  if (npairs) *npairs = (int)pair_crop.size();
  if (iters) *iters = it;
  return rc < 0 ? rc : 0;
}

// ---------------------------------------------------------------------------------------
// Flexible CG (one-term A-orthogonalisation of the preconditioned residual, Notay 2000):
//   z_k = M r_k,  beta_k = -(z_k . q_{k-1}) / (p_{k-1} . q_{k-1}),  p_k = z_k + beta_k p_{k-1},
//   q_k = (I - gamma A) p_k,  alpha_k = (p_k . r_k) / (p_k . q_k),
//   x += alpha_k p_k,  r -= alpha_k q_k,  stop at ||r|| <= tol ||b||.
// Fused like the PCG comparator: the scalars live on the device and come from the last block
// of each exact reduction, the network's forward pass and the three Krylov kernels of
// FCG_BATCH iterations are captured in one CUDA graph, and every kernel returns at once
// after the device-side flag says the solve has stopped.
//   KB: z . q_{k-1} -> beta                                  (16 B/DOF)
//   KP: p = z + beta p_{k-1} (also at the stencil neighbours), q = p - gamma A p,
//       p . r and p . q -> alpha                             (40 B/DOF + halo)
//   KX: x += alpha p, r -= alpha q, r . r -> stop test        (48 B/DOF)
// ---------------------------------------------------------------------------------------
#include "krylov.cuh"

namespace net {

struct FcgScal {
  double beta, alpha, pq_prev, rr, gamma, tolb, pr;
  int iters, maxit, state, pad_; // state: 0 running, 1 converged, 2 iteration limit, 3 breakdown
  unsigned long long limbs[2][xsum::NL];
  unsigned int flags[2];
  unsigned int ticket, pad2_;
};

struct FcgOut {
  int state, iters;
  double rr;
};

constexpr int FCG_BATCH = 8; // iterations per graph launch (even: p, q ping-pong)
constexpr int FCG_U     = 2; // grid-strided points per thread and trip (independent loads in flight)

__global__ void __launch_bounds__(256) fcg_beta_kernel(long long n, const double* __restrict__ z,
                                                       const double* __restrict__ qprev, FcgScal* s)
{
  if (s->state != 0) return;
  xsum::Limbs a[1];
  unsigned fl[1] = {0};
  xsum::zero(a[0]);
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long k0 = (long long)blockIdx.x * blockDim.x + threadIdx.x; k0 < n; k0 += FCG_U * stride)
  {
    double zv[FCG_U], qv[FCG_U];
#pragma unroll
    for (int u = 0; u < FCG_U; ++u)
    {
      const long long k = k0 + u * stride;
      zv[u]             = k < n ? z[k] : 0.0;
      qv[u]             = k < n ? qprev[k] : 0.0;
    }
#pragma unroll
    for (int u = 0; u < FCG_U; ++u)
      if (k0 + u * stride < n) xsum::add(a[0], zv[u] * qv[u], fl[0]);
  }
  krylov_block_finish<256, 1>(a, fl, s, [&](const double* v) {
    s->beta = (s->iters > 0) ? -v[0] / s->pq_prev : 0.0;
  });
}

// KP: p = z + beta p_prev and p.r. KQ: q = (I - gamma A) p with the coefficients folded,
// q = (1 - gamma cc) p_C - gamma cx (p_W + p_E) - gamma cy (p_S + p_N), and p.q -> alpha =
// p.r / p.q. Eight FP64 instructions per point in the two (p, stencil, the two dot products):
// GB300 issues FP64 at a small fraction of its FP32 rate (about 5e11 instructions/s
// measured), so these kernels are bounded by the FP64 pipe rather than by HBM.
__global__ void __launch_bounds__(256) fcg_p_kernel(long long n, const double* __restrict__ z,
                                                    const double* __restrict__ pp, const double* __restrict__ r,
                                                    double* __restrict__ p, FcgScal* s)
{
  if (s->state != 0) return;
  const double beta = s->beta;
  xsum::Limbs a[1];
  unsigned fl[1] = {0};
  xsum::zero(a[0]);
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long k0 = (long long)blockIdx.x * blockDim.x + threadIdx.x; k0 < n; k0 += FCG_U * stride)
  {
    double zv[FCG_U], pv[FCG_U], rv[FCG_U];
#pragma unroll
    for (int u = 0; u < FCG_U; ++u)
    {
      const long long k = k0 + u * stride;
      const bool in     = k < n;
      zv[u]             = in ? z[k] : 0.0;
      pv[u]             = in ? pp[k] : 0.0;
      rv[u]             = in ? r[k] : 0.0;
    }
#pragma unroll
    for (int u = 0; u < FCG_U; ++u)
    {
      const long long k = k0 + u * stride;
      if (k < n)
      {
        const double pk = __fma_rn(beta, pv[u], zv[u]);
        p[k]            = pk;
        xsum::add(a[0], pk * rv[u], fl[0]);
      }
    }
  }
  krylov_block_finish<256, 1>(a, fl, s, [&](const double* v) { s->pr = v[0]; });
}

__global__ void __launch_bounds__(256) fcg_q_kernel(ProbDev P, const double* __restrict__ p,
                                                    double* __restrict__ q, FcgScal* s, FcgOut* out)
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
    s->alpha   = s->pr / v[0];
    s->pq_prev = v[0];
    if (!(v[0] != 0.0) || !(v[0] == v[0]))
    {
      s->state   = 3; // breakdown: p . q = 0 or not a number
      out->state = 3;
    }
  });
}

__global__ void __launch_bounds__(256) fcg_x_kernel(long long n, const double* __restrict__ p,
                                                    const double* __restrict__ q, double* __restrict__ x,
                                                    double* __restrict__ r, FcgScal* s, FcgOut* out)
{
  if (s->state != 0) return;
  const double alpha = s->alpha;
  xsum::Limbs a[1];
  unsigned fl[1] = {0};
  xsum::zero(a[0]);
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long k0 = (long long)blockIdx.x * blockDim.x + threadIdx.x; k0 < n; k0 += FCG_U * stride)
  {
    double pv[FCG_U], qv[FCG_U], xv[FCG_U], rv[FCG_U];
#pragma unroll
    for (int u = 0; u < FCG_U; ++u)
    {
      const long long k = k0 + u * stride;
      const bool in     = k < n;
      pv[u]             = in ? p[k] : 0.0;
      qv[u]             = in ? q[k] : 0.0;
      xv[u]             = in ? x[k] : 0.0;
      rv[u]             = in ? r[k] : 0.0;
    }
#pragma unroll
    for (int u = 0; u < FCG_U; ++u)
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
    else if (!(v[0] == v[0])) s->state = 3;
    else if (s->iters >= s->maxit) s->state = 2;
    out->state = s->state;
    out->iters = s->iters;
    out->rr    = v[0];
  });
}

__global__ void axpy_kernel(long long n, double a, const double* __restrict__ xv, double* __restrict__ y)
{
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
    y[k] = __fma_rn(a, xv[k], y[k]);
}

// q = b - (I - gamma A) x (true residual of the returned iterate)
__global__ void true_residual_kernel(ProbDev P, double gamma, const double* __restrict__ x,
                                     const double* __restrict__ b, double* __restrict__ q)
{
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long j = (long long)blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= P.nx || j >= P.ny) return;
  const long long k = j * P.nx + i;
  const double pc = x[k];
  const double pw = (i > 0) ? x[k - 1] : 0.0, pe = (i < P.nx - 1) ? x[k + 1] : 0.0;
  const double ps = (j > 0) ? x[k - P.nx] : 0.0, pn = (j < P.ny - 1) ? x[k + P.nx] : 0.0;
  const double sx = pw + pe, sy = ps + pn;
  double acc = P.cc * pc;
  acc        = __fma_rn(P.cx, sx, acc);
  acc        = __fma_rn(P.cy, sy, acc);
  q[k]       = b[k] - __fma_rn(-gamma, acc, pc);
}

} // namespace net

extern "C" int STS_FCGSolve(STS_Problem p, double gamma, STS_Net nt, N_Vector b, N_Vector x, double tol, int maxit,
                            int* iters, double* relres)
{
  STS_MARK_FUNCTION;
  const bool fallback = maxit > 0; // maxit < 0: at most -maxit iterations, no fallback
  if (maxit < 0) maxit = -maxit;
  if (!p || !nt || !b || !x || p->nx != p->ny || NVL(b) != p->nx * p->ny || NVL(x) != NVL(b) || maxit < 1 ||
      p->kind == STS_PROBLEM_PERIODIC)
  {
    sts_set_error("STS_FCGSolve: invalid arguments (square Dirichlet grids, sizes a multiple of 16)");
    return -1;
  }
  const int n = (int)p->nx;
  if (!net_size_ok(nt, n)) return -1;
  if (nt->ctx != p->ctx)
  {
    sts_set_error("STS_FCGSolve: the network and the problem must share one context (stream)");
    return -1;
  }
  STS_Context ctx = p->ctx;
  ctx_activate(ctx);
  cudaStream_t st   = ctx->stream;
  const long long N = NVL(b);
  double* buf       = nullptr;
  net::FcgScal* d_s = nullptr;
  net::FcgOut *h_out = nullptr, *d_out = nullptr;
  if (!STS_CUDA_OK(cudaMalloc(&buf, 6 * N * sizeof(double))) || !STS_CUDA_OK(cudaMalloc(&d_s, sizeof(net::FcgScal))) ||
      !STS_CUDA_OK(cudaHostAlloc(&h_out, sizeof(net::FcgOut), cudaHostAllocMapped)) ||
      !STS_CUDA_OK(cudaHostGetDevicePointer(&d_out, h_out, 0)))
  {
    cudaFree(buf);
    cudaFree(d_s);
    cudaFreeHost(h_out);
    return -1;
  }
  double* r  = buf;
  double* z  = buf + N;
  double* P2[2] = {buf + 2 * N, buf + 3 * N};
  double* Q2[2] = {buf + 4 * N, buf + 5 * N};
  cudaMemsetAsync(NVD(x), 0, N * 8, st);
  cudaMemsetAsync(buf + 2 * N, 0, 4 * N * 8, st);
  cudaMemcpyAsync(r, NVD(b), N * 8, cudaMemcpyDeviceToDevice, st);
  const double bnorm = sqrt(sts_dot_exact(ctx, NVD(b), NVD(b), N, SLOT_PCG0));
  int ret = 0, it = 0;
  double tr = 0.0;
  if (bnorm > 0.0)
  {
    const double jac = 1.0 / (1.0 - gamma * p->cc);
    const double sk  = (std::log10(p->ky / p->kx) + 1.5) / 1.5;
    const double sg  = std::log10(gamma / (p->dx * p->dx)) - 3.6;
    // the network is linear in its input: any fixed scale works; 1/rms(b) keeps values O(1)
    const double scale = std::sqrt((double)N) / bnorm;
    net::FcgScal hs;
    memset(&hs, 0, sizeof(hs));
    hs.gamma   = gamma;
    hs.tolb    = tol * bnorm;
    hs.maxit   = maxit;
    hs.pq_prev = 1.0;
    memset(h_out, 0, sizeof(net::FcgOut));
    cudaMemcpyAsync(d_s, &hs, sizeof(hs), cudaMemcpyHostToDevice, st);
    // the reduction kernels run one wave of resident blocks (each block combines its exact
    // sums once), two grid-strided points per thread and trip
    auto resident = [&](auto kernel) {
      int occ = 0;
      if (!STS_CUDA_OK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, 256, 0)) || occ < 1) occ = 1;
      long long b         = (long long)ctx->num_sms * occ;
      const long long cap = (N + 256LL * net::FCG_U - 1) / (256LL * net::FCG_U);
      return (int)(b < cap ? b : (cap < 1 ? 1 : cap));
    };
    const int eb_beta = resident(net::fcg_beta_kernel), eb_p = resident(net::fcg_p_kernel),
              eb_x = resident(net::fcg_x_kernel);
    dim3 bq(256, 1);
    const unsigned gx = (unsigned)((p->nx + 255) / 256);
    int occ_q         = 0;
    if (!STS_CUDA_OK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_q, net::fcg_q_kernel, 256, 0)) || occ_q < 1)
      occ_q = 1;
    long long gy_cap = (long long)ctx->num_sms * occ_q / gx; // one wave of resident blocks
    if (gy_cap < 1) gy_cap = 1;
    dim3 gq(gx, (unsigned)(p->ny < gy_cap ? p->ny : gy_cap));
    cudaGraph_t g;
    cudaGraphExec_t ge = nullptr;
    net::l0::FoldA fa;
    net::l0::FoldB fb;
    bool ok = l0_prepare(nt, (float)sk, (float)sg, &fa, &fb) && STS_CUDA_OK(cudaStreamSynchronize(st)) &&
              STS_CUDA_OK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    if (ok)
    {
      for (int k = 0; k < net::FCG_BATCH; ++k)
      {
        double *pp = P2[k & 1], *pn = P2[(k + 1) & 1];
        double *qp = Q2[k & 1], *qn = Q2[(k + 1) & 1];
        net_forward_infer(nt, n, r, scale, (float)sk, (float)sg, jac / scale, z, &fa, &fb);
        net::fcg_beta_kernel<<<eb_beta, 256, 0, st>>>(N, z, qp, d_s);
        net::fcg_p_kernel<<<eb_p, 256, 0, st>>>(N, z, pp, r, pn, d_s);
        net::fcg_q_kernel<<<gq, bq, 0, st>>>(p->dev, pn, qn, d_s, d_out);
        net::fcg_x_kernel<<<eb_x, 256, 0, st>>>(N, pn, qn, NVD(x), r, d_s, d_out);
      }
      ok = STS_CUDA_OK(cudaStreamEndCapture(st, &g));
      if (ok)
      {
        ok = STS_CUDA_OK(cudaGraphInstantiate(&ge, g, 0));
        cudaGraphDestroy(g);
      }
    }
    ret = ok ? 1 : -1;
    // the device sets state 2 at maxit; the host bound on launches is a second guard
    for (long long launches = 0; ret == 1; ++launches)
    {
      if (launches > maxit / net::FCG_BATCH + 2)
      {
        sts_set_error("STS_FCGSolve: the device-side stop flag was not set");
        ret = -1;
        break;
      }
      if (!STS_CUDA_OK(cudaGraphLaunch(ge, st)) || !STS_CUDA_OK(cudaStreamSynchronize(st)))
      {
        ret = -1;
        break;
      }
      if (*(volatile int*)ctx->h_err)
      { // a tensor-core convolution's bounded wait timed out
        *ctx->h_err = 0;
        sts_set_error("STS_FCGSolve: a tensor-core wait timed out");
        ret = -1;
        break;
      }
      const int state = ((volatile net::FcgOut*)h_out)->state;
      if (state == 1) ret = 0;
      else if (state == 2) ret = 1;
      else if (state == 3) ret = -3;
      if (state != 0) break;
    }
    if (ge) cudaGraphExecDestroy(ge);
    it = h_out->iters;
    dim3 bb(64, 4), gg((unsigned)((p->nx + 63) / 64), (unsigned)((p->ny + 3) / 4));
    net::true_residual_kernel<<<gg, bb, 0, st>>>(p->dev, gamma, NVD(x), NVD(b), Q2[0]);
    tr = sqrt(sts_dot_exact(ctx, Q2[0], Q2[0], N, SLOT_PCG3)) / bnorm;
    if (fallback && (ret == 1 || ret == -3) && tr == tr && tr > tol)
    {
      // Jacobi-PCG fallback on the correction: (I - gamma A) d = b - (I - gamma A) x, x += d
      N_Vector qv = N_VMake_Sts(N, Q2[0], ctx);
      N_Vector dv = N_VNew_Sts(N, ctx);
      int it2     = 0;
      double rel2 = 0.0;
      int rc2     = -1;
      if (qv && dv)
        rc2 = sts_pcg_run(p, gamma, qv, dv, tol / tr, 1000000, 1, &it2, &rel2, nullptr);
      if (rc2 == 0)
      {
        net::axpy_kernel<<<grid_for(N), 256, 0, st>>>(N, 1.0, NVD(dv), NVD(x));
        net::true_residual_kernel<<<gg, bb, 0, st>>>(p->dev, gamma, NVD(x), NVD(b), Q2[0]);
        tr  = sqrt(sts_dot_exact(ctx, Q2[0], Q2[0], N, SLOT_PCG3)) / bnorm;
        ret = 2;
      }
      it += it2;
      if (qv) N_VDestroy_Sts(qv);
      if (dv) N_VDestroy_Sts(dv);
    }
  }
  cudaStreamSynchronize(st);
  cudaFree(buf);
  cudaFree(d_s);
  cudaFreeHost(h_out);
  if (iters) *iters = it;
  if (relres) *relres = tr;
  return ret;
}

// Shifted solve with a choice of method: the condition-number estimate of the Jacobi-scaled
// operator, kappa = 1 + 4 gamma (cx + cy), predicts Jacobi-PCG's iteration count (~sqrt(kappa));
// below kappa_min the network's per-iteration cost is not repaid and Jacobi-PCG runs directly,
// above it flexible CG with the network (falling back to Jacobi-PCG itself if needed).
extern "C" int STS_ImplicitSolveLearned(STS_Problem p, double gamma, STS_Net nt, N_Vector b, N_Vector x, double tol,
                                        int maxit, double kappa_min, int* iters, double* relres, int* used_net)
{
  STS_MARK_FUNCTION;
  if (!p || !b || !x)
  {
    sts_set_error("STS_ImplicitSolveLearned: invalid arguments");
    return -1;
  }
  if (!(kappa_min > 0.0)) kappa_min = 1500.0;
  const double kappa = 1.0 + 4.0 * gamma * (p->cx + p->cy);
  const bool net_ok  = nt && p->nx == p->ny && p->kind != STS_PROBLEM_PERIODIC && p->nx % 16 == 0 && p->nx <= nt->nmax;
  if (used_net) *used_net = 0;
  if (net_ok && kappa >= kappa_min)
  {
    if (used_net) *used_net = 1;
    return STS_FCGSolve(p, gamma, nt, b, x, tol, maxit, iters, relres);
  }
  return STS_ImplicitSolvePCG(p, gamma, b, x, tol, maxit, 1, iters, relres);
}

// ---------------------------------------------------------------------------------------
// The network as a preconditioner object behind the reference's PSetup / PSolve interface
// (diffusion_2D/preconditioner_jacobi.cpp:9-61 signatures), for the generic Krylov solvers:
// PSetup takes gamma and folds the system features into the level-0 weights, PSolve applies
// z = M r with the input scaled by 1/rms(r) (the network is linear in r, the scale only keeps
// the BF16 / FP32 activations in range). Flexible GMRES (SUNLinSol_SPFGMR) is the safe outer
// method: the BF16 network is linear in exact arithmetic but its rounding is not.
// ---------------------------------------------------------------------------------------
struct STS_NetPrec_ {
  STS_Net net       = nullptr;
  STS_Problem p     = nullptr;
  double gamma      = -1.0;
  double sk = 0.0, sg = 0.0, jac = 1.0;
  net::l0::FoldA fa;
  net::l0::FoldB fb;
  bool ready        = false;
};

extern "C" int STS_NetPrecCreate(STS_Net nt, STS_Problem p, STS_NetPrec* out)
{
  if (!out) return -1;
  *out = nullptr;
  if (!nt || !p || p->nx != p->ny || p->kind == STS_PROBLEM_PERIODIC || nt->ctx != p->ctx)
  {
    sts_set_error("STS_NetPrecCreate: square Dirichlet grid on the network's context required");
    return -1;
  }
  if (!net_size_ok(nt, (int)p->nx)) return -1;
  STS_NetPrec P = new STS_NetPrec_();
  P->net        = nt;
  P->p          = p;
  *out          = P;
  return 0;
}

extern "C" int STS_NetPrecFree(STS_NetPrec* P)
{
  if (!P || !*P) return 0;
  delete *P;
  *P = nullptr;
  return 0;
}

extern "C" int STS_NetPSetup(double t, N_Vector u, N_Vector f, int jok, int* jcurPtr, double gamma, void* user_data)
{
  STS_MARK_FUNCTION;
  (void)t;
  (void)u;
  (void)f;
  (void)jok;
  STS_NetPrec P = (STS_NetPrec)user_data;
  if (!P || !(gamma > 0.0)) return -1;
  STS_Problem p = P->p;
  ctx_activate(p->ctx);
  P->gamma = gamma;
  P->jac   = 1.0 / (1.0 - gamma * p->cc);
  P->sk    = (std::log10(p->ky / p->kx) + 1.5) / 1.5;
  P->sg    = std::log10(gamma / (p->dx * p->dx)) - 3.6;
  P->ready = l0_prepare(P->net, (float)P->sk, (float)P->sg, &P->fa, &P->fb);
  if (jcurPtr) *jcurPtr = 1;
  return P->ready ? 0 : -1;
}

extern "C" int STS_NetPrecSolve(void* P_data, N_Vector r, N_Vector z, double tol, int lr)
{
  STS_MARK_FUNCTION;
  (void)tol;
  (void)lr;
  STS_NetPrec P = (STS_NetPrec)P_data;
  if (!P || !P->ready || !r || !z || NVL(r) != P->p->nx * P->p->ny || NVL(z) != NVL(r))
  {
    sts_set_error("STS_NetPrecSolve: call STS_NetPSetup first; vectors of the problem's size");
    return -1;
  }
  STS_Context ctx = P->p->ctx;
  const long long N = NVL(r);
  const double rn   = sqrt(sts_dot_exact(ctx, NVD(r), NVD(r), N, SLOT_PCG3));
  if (!(rn > 0.0) || !(rn < INFINITY))
  {
    if (!(rn == 0.0)) return -1; // non-finite input
    return STS_CUDA_OK(cudaMemsetAsync(NVD(z), 0, N * sizeof(double), ctx->stream)) ? 0 : -1;
  }
  const double scale = std::sqrt((double)N) / rn;
  net_forward_infer(P->net, (int)P->p->nx, NVD(r), scale, (float)P->sk, (float)P->sg, P->jac / scale, NVD(z), &P->fa,
                    &P->fb);
  return STS_CUDA_OK(cudaGetLastError()) ? 0 : -1;
}

extern "C" int STS_NetPSolve(double t, N_Vector u, N_Vector f, N_Vector r, N_Vector z, double gamma, double delta,
                             int lr, void* user_data)
{
  (void)t;
  (void)u;
  (void)f;
  STS_NetPrec P = (STS_NetPrec)user_data;
  if (!P) return -1;
  if (!P->ready || P->gamma != gamma)
    if (STS_NetPSetup(0.0, nullptr, nullptr, 0, nullptr, gamma, P) != 0) return -1;
  return STS_NetPrecSolve(P, r, z, delta, lr);
}
