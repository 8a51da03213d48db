// Device-side reductions shared by the fused Krylov solvers (PCG and flexible CG): exact
// dot products whose last block produces the solver's scalars without a host round trip.
#pragma once
#include "kernels.cuh"
#include "sts_internal.cuh"

// Block combine of up to two exact accumulators into s->limbs (device scalar block S with
// limbs[2][NL], flags[2] and ticket); the last block to arrive finalises the sums, resets
// the accumulators and runs `fin` on the results.
template <int NT, int NACC, typename S, typename Fin>
__device__ __forceinline__ void krylov_block_finish(xsum::Limbs* a, unsigned* fl, S* s, Fin fin)
{
  __shared__ long long sm[NT / 32][NACC][xsum::NL];
  __shared__ unsigned sflags[NACC];
  __shared__ bool last;
  const int tid  = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  const int lane = tid & 31, warp = tid >> 5;
  if (tid < NACC) sflags[tid] = 0;
#pragma unroll
  for (int c = 0; c < NACC; ++c)
#pragma unroll
    for (int k = 0; k < xsum::NL; ++k)
    {
      long long v = a[c].l[k];
#pragma unroll
      for (int m = 16; m >= 1; m >>= 1) v += shfl_xor_ll(v, m);
      if (lane == 0) sm[warp][c][k] = v;
    }
  __syncthreads();
#pragma unroll
  for (int c = 0; c < NACC; ++c)
    if (fl[c]) atomicOr(&sflags[c], fl[c]);
  if (warp == 0)
  {
#pragma unroll
    for (int c = 0; c < NACC; ++c)
#pragma unroll
      for (int k = 0; k < xsum::NL; ++k)
      {
        long long v = (lane < NT / 32) ? sm[lane][c][k] : 0LL;
#pragma unroll
        for (int m = 16; m >= 1; m >>= 1) v += shfl_xor_ll(v, m);
        if (lane == 0 && v != 0) atomicAdd(&s->limbs[c][k], (unsigned long long)v);
      }
  }
  __syncthreads();
  if (tid == 0)
  {
#pragma unroll
    for (int c = 0; c < NACC; ++c)
      if (sflags[c]) atomicOr(&s->flags[c], sflags[c]);
    __threadfence();
    unsigned t = atomicAdd(&s->ticket, 1u);
    last       = (t == gridDim.x * gridDim.y - 1);
  }
  __syncthreads();
  if (last && tid == 0)
  {
    __threadfence();
    double v[NACC];
#pragma unroll
    for (int c = 0; c < NACC; ++c)
    {
      long long tot[xsum::NL];
#pragma unroll
      for (int k = 0; k < xsum::NL; ++k)
      {
        tot[k]         = (long long)atomicAdd(&s->limbs[c][k], 0ULL);
        s->limbs[c][k] = 0ULL;
      }
      v[c]        = xsum::finalize(tot, atomicOr(&s->flags[c], 0u));
      s->flags[c] = 0u;
    }
    fin(v);
    s->ticket = 0u;
    __threadfence();
  }
}

