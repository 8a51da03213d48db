// Internal declarations shared by the translation units of libstsgpu.so.
#pragma once
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <string>

#include "../../include/stsgpu.h"
#include "xsum.cuh"

#include <nvtx3/nvToolsExt.h>

// NVTX range over one API call: the regions the reference marks for its profiler (the RHS,
// the preconditioner, Evolve) plus the solvers. Without an attached tool a push / pop costs a
// test of a null function pointer.
struct StsRange {
  explicit StsRange(const char* name) { nvtxRangePushA(name); }
  ~StsRange() { nvtxRangePop(); }
  StsRange(const StsRange&)            = delete;
  StsRange& operator=(const StsRange&) = delete;
};
#define STS_MARK_FUNCTION StsRange sts_range_(__func__)
#define STS_MARK_REGION(name) StsRange sts_range_(name)

// ---------------------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------------------
void sts_set_error(const char* fmt, ...);

#define STS_CUDA_OK(call)                                                                  \
  ([&]() -> bool {                                                                         \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess)                                                                 \
    {                                                                                      \
      sts_set_error("%s:%d %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(e_));    \
      return false;                                                                        \
    }                                                                                      \
    return true;                                                                           \
  }())

// ---------------------------------------------------------------------------------------
// context: stream + reduction workspace. Each reduction kernel adds its per-block partial
// limbs into `limbs` with integer atomics, takes a ticket, and the last block converts the
// total into a double written to a result slot (mapped pinned host memory) and clears the
// workspace for the next reduction on the stream.
// ---------------------------------------------------------------------------------------
constexpr int STS_NSLOTS = 64;
enum ResultSlot {
  SLOT_GENERIC = 0,
  SLOT_DSM     = 1,
  SLOT_D0      = 2,
  SLOT_D1      = 3,
  SLOT_D2      = 4,
  SLOT_LAM     = 5,
  SLOT_NRM     = 6,
  SLOT_PCG0    = 8,
  SLOT_PCG1    = 9,
  SLOT_PCG2    = 10,
  SLOT_PCG3    = 11,
  SLOT_MULTI   = 16, // N_VDotProdMulti: slots 16 .. 63
};

struct RedWork {
  unsigned long long limbs[xsum::NL];
  unsigned long long maxbits;
  unsigned int flags;
  unsigned int ticket;
};

struct STS_Context_ {
  int device        = 0;
  int num_sms       = 0;
  cudaStream_t stream = nullptr;
  RedWork* d_work   = nullptr;    // device
  double* h_slots   = nullptr;    // pinned, mapped
  double* d_slots   = nullptr;    // device alias of h_slots
  int* h_err        = nullptr;    // pinned, mapped: kernels report a bounded wait that timed out
  int* d_err        = nullptr;
};

bool ctx_activate(STS_Context ctx);

// grid size for grid-stride elementwise / reduction kernels
inline int ew_blocks(STS_Context ctx, long long n, int per_block)
{
  long long b = (n + per_block - 1) / per_block;
  long long cap = (long long)ctx->num_sms * 8;
  if (b > cap) b = cap;
  if (b < 1) b = 1;
  return (int)b;
}

// Dense output: ARKODE's Hermite interpolation module (ARKodeGetDky with k = 0), degree
// min(q - 1, 5) for a method of order q, here 1 to 3. On the last step [t - h, t], with
// tau = (tout - t) / h in [-1, 0]:
//   degree 1: p = -tau y_old + (1 + tau) y_new
//   degree 2: p = tau^2 y_old + (1 - tau^2) y_new + h (tau^2 + tau) f_new
//   degree 3: p = (3 tau^2 + 2 tau^3) y_old + (1 - 3 tau^2 - 2 tau^3) y_new
//               + h (tau^2 + tau^3) f_old + h (tau + 2 tau^2 + tau^3) f_new
// Elementwise out = a0 y_old, then FMAs in the order y_new, f_old, f_new (the oracle's
// orc_hermite does the same). fold / fnew may be null where the degree does not use them.
void sts_hermite_coeffs(int deg, double tau, double h, double a[4]);
void sts_hermite(STS_Context ctx, long long n, int deg, double tau, double h, const double* yold,
                 const double* ynew, const double* fold, const double* fnew, double* out);

// ---------------------------------------------------------------------------------------
// device-side reduction helpers
// ---------------------------------------------------------------------------------------
#ifdef __CUDACC__
__device__ __forceinline__ long long shfl_xor_ll(long long v, int m)
{
  return (long long)__shfl_xor_sync(0xffffffffu, (unsigned long long)v, m);
}

// Block-level combine of per-thread limbs, then global atomics + last-block finalisation.
// Every thread of the block must call it. `post` selects the final transform:
//   0: value, 1: sqrt(value / n) (WRMS). The result goes to slot_out.
template <int NT>
__device__ __forceinline__ void xsum_block_finish(xsum::Limbs& a, unsigned flags, RedWork* w,
                                                  double* slot_out, int post, double n)
{
  __shared__ long long sm[NT / 32][xsum::NL];
  __shared__ unsigned sflags;
  __shared__ bool last;
  // linear thread index: blocks may be 1-D or 2-D (NT threads in total)
  const int tid  = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  const int lane = tid & 31, warp = tid >> 5;
  if (tid == 0) sflags = 0;
#pragma unroll
  for (int k = 0; k < xsum::NL; ++k)
  {
    long long v = a.l[k];
#pragma unroll
    for (int m = 16; m >= 1; m >>= 1) v += shfl_xor_ll(v, m);
    if (lane == 0) sm[warp][k] = v;
  }
  __syncthreads();
  if (flags) atomicOr(&sflags, flags);
  if (warp == 0)
  {
#pragma unroll
    for (int k = 0; k < xsum::NL; ++k)
    {
      long long v = (lane < NT / 32) ? sm[lane][k] : 0LL;
#pragma unroll
      for (int m = 16; m >= 1; m >>= 1) v += shfl_xor_ll(v, m);
      if (lane == 0 && v != 0) atomicAdd(&w->limbs[k], (unsigned long long)v);
    }
  }
  __syncthreads();
  if (tid == 0)
  {
    if (sflags) atomicOr(&w->flags, sflags);
    __threadfence();
    unsigned t = atomicAdd(&w->ticket, 1u);
    last       = (t == gridDim.x * gridDim.y * gridDim.z - 1);
  }
  __syncthreads();
  if (last && tid == 0)
  {
    __threadfence();
    long long tot[xsum::NL];
#pragma unroll
    for (int k = 0; k < xsum::NL; ++k)
    {
      tot[k]       = (long long)atomicAdd(&w->limbs[k], 0ULL);
      w->limbs[k]  = 0ULL;
    }
    unsigned f = atomicOr(&w->flags, 0u);
    double v   = xsum::finalize(tot, f);
    if (post == 1) v = sqrt(v / n);
    *slot_out = v;
    w->flags  = 0u;
    w->ticket = 0u;
    __threadfence();
  }
}
#endif

// ---------------------------------------------------------------------------------------
// problem
// ---------------------------------------------------------------------------------------
struct ProbDev {
  long long nx, ny;
  int kind, inhom;
  double kx, ky, cx, cy, cc;
  const double *Sx, *Sxx, *Sy, *Syy;
  const float *Sxf, *Sxxf, *Syf, *Syyf;
  const double *Dxw, *Dxe, *Dys, *Dyn;
  int* err; // the context's error word (bounded waits, debug-bounds checks)
};

// Debug-bounds build (-DSTS_DEBUG_BOUNDS): before touching memory a kernel checks the index
// range the thread (or the CTA) is about to use; a violation stores STS_ERR_WORD_BOUNDS in the
// context's error word and the work is skipped, never trapped. The product build compiles the
// checks to `true`.
constexpr int STS_ERR_WORD_WAIT = 1, STS_ERR_WORD_TC_WAIT = 2, STS_ERR_WORD_BOUNDS = 3;
inline const char* sts_err_word_text(int w)
{
  return w == STS_ERR_WORD_BOUNDS ? "an index range check failed (debug-bounds build)"
                                  : "a pipeline wait timed out";
}
#ifdef STS_DEBUG_BOUNDS
#ifdef __CUDACC__
__device__ __forceinline__ bool sts_in_bounds(bool ok, int* err)
{
  if (!ok && err) atomicExch(err, STS_ERR_WORD_BOUNDS);
  return ok;
}
#endif
#define STS_IN_BOUNDS(cond, err) sts_in_bounds((cond), (err))
#else
#define STS_IN_BOUNDS(cond, err) true
#endif

struct STS_Problem_ {
  STS_Context ctx = nullptr;
  int kind = 0, inhom = 0;
  long long nx = 0, ny = 0;
  double kx = 1, ky = 1, xl = 0, xu = 1, yl = 0, yu = 1, dx = 0, dy = 0, cx = 0, cy = 0, cc = 0;
  double* d_tab   = nullptr; // Sx | Sxx | Sy | Syy | Dxw | Dxe | Dys | Dyn (doubles)
  float* d_tabf   = nullptr; // Sxf | Sxxf | Syf | Syyf
  double* d_jacobi = nullptr; // PSetup output (constant Jacobi scale, 1 entry)
  double jacobi_scale = 1.0;
  ProbDev dev{};
};

static inline double sts_c(double t)
{
  double cs = cos(2.0 * 3.14159265358979323846 * t);
  return cs * cs;
}
static inline double sts_cdot(double t) { return -2.0 * 3.14159265358979323846 * sin(4.0 * 3.14159265358979323846 * t); }

// N_Vector content
struct NVContent {
  long long length = 0;
  long long nx = 0, ny = 0;
  bool own = false;
  int device = 0; // owner device: destroying a vector must not need its context
  double* data = nullptr;
};
inline NVContent* NVC(N_Vector v) { return (NVContent*)v->content; }
inline double* NVD(N_Vector v) { return NVC(v)->data; }
inline long long NVL(N_Vector v) { return NVC(v)->length; }

// problem-level kernels used by the integrator and the solvers (diffusion.cu)
int sts_rhs_launch(STS_Problem p, double t, const double* u, double* f, bool forcing, cudaStream_t s);
double sts_dot_exact(STS_Context ctx, const double* x, const double* y, long long n, int slot);
double sts_wrms_ewt(STS_Context ctx, const double* a, const double* b, const double* y, long long n,
                    double rtol, double atol, int slot);

// Integrator handles (void* arkode_mem) start with a kind word: LSRKStep (lsrk.cu) or ARKStep
// (arkstep.cu); the ARKode* entry points of lsrk.cu dispatch on it.
#include <cstdint>
constexpr uint32_t STS_MEM_LSRK    = 0x4B52534Cu;
constexpr uint32_t STS_MEM_ARKSTEP = 0x534B5241u;
inline uint32_t sts_mem_kind(const void* mem) { return *(const uint32_t*)mem; }
// the step-size controllers of lsrk.cu for an error estimate of order ord
double sts_controller_estimate(int controller, double h, double dsm, double ep1, double ep2, double hp,
                               long long nhist, double ord);
int arkstep_sstolerances(void* mem, double rtol, double atol);
int arkstep_set_user_data(void* mem, void* ud);
int arkstep_set_controller(void* mem, int c);
int arkstep_set_fixed_step(void* mem, double h);
int arkstep_set_max_steps(void* mem, long long mx);
int arkstep_set_stop_time(void* mem, double ts);
int arkstep_evolve(void* mem, double tout, N_Vector yout, double* tret, int itask);
int arkstep_reset(void* mem, double t, N_Vector y);
int arkstep_get_stats(void* mem, STS_Stats* s);
int arkstep_print_stats(void* mem, char* buf, int buflen);
void arkstep_free(void* mem);
