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
// ticket, 96 bytes) and lives for as long as the library is loaded, in every CUDA context
// that loads it. Host code cannot use the array's name as a device address: each call looks
// the address up with cudaGetSymbolAddress in the context current on the calling thread
// (the lookup allocates nothing). A stream being captured into a CUDA graph may not trigger
// that lookup (it can load the module), so a call on a capturing stream uses the address
// found by an earlier call in the same context and fails with a clear error if there was
// none: make the first call in each context outside any stream capture. The cache is keyed by
// the context, not the device number, so a driver-API context made current on the same device
// or the new primary context after cudaDeviceReset gets its own lookup. Every call in a context
// shares the one array: the call clears it with cudaMemsetAsync before its kernel, and calls
// whose kernels overlap on the GPU (different streams, no ordering) race on it.
#include <cuda.h>
#include <cuda_runtime.h>

#include <mutex>

#include "kernels.cuh"
#include "sts_internal.cuh"

static constexpr int NOALLOC_MAX_DEVICES = 64;

// The shared scratch: one exact-accumulator block per context (zero at module load).
static __device__ __align__(256) RedWork g_noalloc_scratch[1];

// Address of the scratch and the SM count, per device, for the context they were found in.
// Written and read under g_mu (an uncontended lock per call, next to a kernel launch).
struct ScratchSlot {
  CUcontext ctx = nullptr;
  RedWork* addr = nullptr;
  int sms       = 0;
};
static ScratchSlot g_slot[NOALLOC_MAX_DEVICES];
static std::mutex g_mu;

// cuCtxGetCurrent through the runtime's driver entry point (the library links no libcuda)
static CUresult (*g_ctx_get_current)(CUcontext*) = nullptr;
static std::once_flag g_ctx_fn_once;

static bool current_context(CUcontext* out)
{
  std::call_once(g_ctx_fn_once, [] {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      g_ctx_get_current = reinterpret_cast<CUresult (*)(CUcontext*)>(fn);
  });
  *out = nullptr;
  return g_ctx_get_current && g_ctx_get_current(out) == CUDA_SUCCESS && *out;
}

// the scratch address and SM count for the current context of device `dev`
static int noalloc_scratch(int dev, bool capturing, RedWork** addr, int* sms)
{
  CUcontext cur = nullptr;
  if (!current_context(&cur))
  {
    sts_set_error("STS_WrmsNormNoAlloc: no current CUDA context on device %d", dev);
    return -1;
  }
  std::lock_guard<std::mutex> lk(g_mu);
  ScratchSlot& sl = g_slot[dev];
  if (capturing)
  {
    if (sl.ctx != cur || !sl.addr)
    {
      sts_set_error("STS_WrmsNormNoAlloc: first call in this CUDA context made during stream capture; "
                    "make one call outside capture first");
      return -1;
    }
  }
  else
  {
    void* p       = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
    {
      sts_set_error("STS_WrmsNormNoAlloc: cudaGetSymbolAddress failed on device %d: %s", dev, cudaGetErrorString(e));
      return -1;
    }
    if (sl.ctx != cur || sl.sms < 1)
    {
      int n = 0;
      e     = cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
      if (e != cudaSuccess || n < 1)
      {
        sts_set_error("STS_WrmsNormNoAlloc: cannot query device %d: %s", dev, cudaGetErrorString(e));
        return -1;
      }
      sl.sms = n;
    }
    sl.ctx  = cur;
    sl.addr = (RedWork*)p;
  }
  *addr = sl.addr;
  *sms  = sl.sms;
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
  cudaStream_t s = (cudaStream_t)stream;
  cudaStreamCaptureStatus cap_status = cudaStreamCaptureStatusNone;
  e = cudaStreamIsCapturing(s, &cap_status);
  if (e != cudaSuccess)
  {
    sts_set_error("STS_WrmsNormNoAlloc: invalid stream: %s", cudaGetErrorString(e));
    return -1;
  }
  RedWork* work = nullptr;
  int sms       = 0;
  if (noalloc_scratch(dev, cap_status != cudaStreamCaptureStatusNone, &work, &sms)) return -1;
  e = cudaMemsetAsync(work, 0, sizeof(RedWork), s);
  if (e != cudaSuccess)
  {
    sts_set_error("STS_WrmsNormNoAlloc: clearing the scratch failed: %s", cudaGetErrorString(e));
    return -1;
  }
  long long blocks = (n + 256 * 4 - 1) / (256 * 4);
  long long cap    = (long long)sms * 8;
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
