// Allocation-free WRMS norm.
//
// Some callers cannot allocate GPU or pinned host memory at the point where they need a
// norm: code that runs while another runtime is recording a CUDA graph or owns a fixed
// memory pool, real-time loops that must not touch the allocator after start-up, or a
// foreign vector library (for example a SUNDIALS NVECTOR wrapping arrays it does not own)
// that has raw device pointers but no STS_Context. STS_WrmsNormNoAlloc serves them: it is
// the exact-WRMS reduction of N_VWrmsNorm_Sts with its scratch space in a fixed array in
// device global memory instead of a context's cudaMalloc'd workspace, and it writes its
// result to a device location the caller provides.
//
// The scratch array is small (one accumulator block: ten 64-bit limbs, a word, flags and a
// ticket, 96 bytes) and lives for as long as the library is loaded, on every device that
// loads it. Host code cannot use the array's name as a device address, so the first call
// on each device, with that device current, looks the address up with cudaGetSymbolAddress
// and caches it; make that first call outside any stream capture. Every call on a device
// shares the one array: the call clears it with cudaMemsetAsync before its kernel, and
// calls whose kernels overlap on the GPU (different streams, no ordering) race on it.
#include <cuda_runtime.h>

#include <mutex>

#include "kernels.cuh"
#include "sts_internal.cuh"

static constexpr int NOALLOC_MAX_DEVICES = 64;

// The shared scratch: one exact-accumulator block per device (zero at module load).
static __device__ __align__(256) RedWork g_noalloc_scratch[1];

static RedWork* g_scratch_addr[NOALLOC_MAX_DEVICES] = {};
static int g_num_sms[NOALLOC_MAX_DEVICES]           = {};
static std::mutex g_setup_mu;

// once per device, with that device current
static int noalloc_setup(int dev)
{
  std::lock_guard<std::mutex> lk(g_setup_mu);
  if (g_scratch_addr[dev]) return 0;
  void* p       = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || !p)
  {
    sts_set_error("STS_WrmsNormNoAlloc: cudaGetSymbolAddress failed on device %d: %s", dev,
                  cudaGetErrorString(e));
    return -1;
  }
  int sms = 0;
  e       = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess || sms < 1)
  {
    sts_set_error("STS_WrmsNormNoAlloc: cannot query device %d: %s", dev, cudaGetErrorString(e));
    return -1;
  }
  g_num_sms[dev]      = sms;
  g_scratch_addr[dev] = (RedWork*)p;
  return 0;
}

extern "C" int STS_WrmsNormNoAlloc(const double* x, const double* w, sts_index n, double* result,
                                   void* stream)
{
  if (!x || !w || !result)
  {
    sts_set_error("STS_WrmsNormNoAlloc: NULL pointer argument");
    return -1;
  }
  if (n < 1 || n > STS_NOALLOC_MAX_N)
  {
    sts_set_error("STS_WrmsNormNoAlloc: length %lld outside [1, %lld] (the accumulator's term limit)",
                  (long long)n, (long long)STS_NOALLOC_MAX_N);
    return -1;
  }
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= NOALLOC_MAX_DEVICES)
  {
    sts_set_error("STS_WrmsNormNoAlloc: no usable current device");
    return -1;
  }
  if (!g_scratch_addr[dev] && noalloc_setup(dev)) return -1;
  cudaStream_t s = (cudaStream_t)stream;
  RedWork* work  = g_scratch_addr[dev];
  e              = cudaMemsetAsync(work, 0, sizeof(RedWork), s);
  if (e != cudaSuccess)
  {
    sts_set_error("STS_WrmsNormNoAlloc: clearing the scratch failed: %s", cudaGetErrorString(e));
    return -1;
  }
  long long blocks = (n + 256 * 4 - 1) / (256 * 4);
  long long cap    = (long long)g_num_sms[dev] * 8;
  if (blocks > cap) blocks = cap;
  xred_kernel<1><<<(unsigned)blocks, 256, 0, s>>>(n, x, w, work, result);
  e = cudaGetLastError();
  if (e != cudaSuccess)
  {
    sts_set_error("STS_WrmsNormNoAlloc: launch failed: %s", cudaGetErrorString(e));
    return -1;
  }
  return 0;
}
