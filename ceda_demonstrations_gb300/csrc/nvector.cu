// Device N_Vector for the GB300 STS path: context, ops table, elementwise kernels and
// exact reductions. Ops mirror gkeyll_diffusion/src/nvector_gkylzero.c:45-514 (the LSRKStep
// subset) plus N_VProd (preconditioner_jacobi.cpp:58) and N_VLinearCombination.
#include <cuda_runtime.h>

#include <cmath>
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <mutex>

#include "kernels.cuh"
#include "sts_internal.cuh"

// ---------------------------------------------------------------------------------------
// error state
// ---------------------------------------------------------------------------------------
static thread_local char g_err[512] = "";

void sts_set_error(const char* fmt, ...)
{
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

extern "C" const char* STS_GetLastError(void) { return g_err; }

extern "C" int STS_DeviceCount(void)
{
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) return 0;
  return n;
}

// ---------------------------------------------------------------------------------------
// context
// ---------------------------------------------------------------------------------------
bool ctx_activate(STS_Context ctx)
{
  int cur = -1;
  if (cudaGetDevice(&cur) != cudaSuccess) return false;
  if (cur != ctx->device) return STS_CUDA_OK(cudaSetDevice(ctx->device));
  return true;
}

extern "C" int STS_ContextCreate(int device, STS_Context* out)
{
  if (!out) return -1;
  *out = nullptr;
  int ndev = 0;
  if (!STS_CUDA_OK(cudaGetDeviceCount(&ndev))) return -1;
  if (device < 0 || device >= ndev)
  {
    sts_set_error("STS_ContextCreate: device %d out of range (%d devices)", device, ndev);
    return -1;
  }
  if (!STS_CUDA_OK(cudaSetDevice(device))) return -1;
  STS_Context c = new STS_Context_();
  c->device     = device;
  cudaDeviceProp prop;
  if (!STS_CUDA_OK(cudaGetDeviceProperties(&prop, device))) goto fail;
  c->num_sms = prop.multiProcessorCount;
  if (!STS_CUDA_OK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking))) goto fail;
  if (!STS_CUDA_OK(cudaMalloc(&c->d_work, sizeof(RedWork)))) goto fail;
  if (!STS_CUDA_OK(cudaMemset(c->d_work, 0, sizeof(RedWork)))) goto fail;
  if (!STS_CUDA_OK(cudaHostAlloc(&c->h_slots, STS_NSLOTS * sizeof(double), cudaHostAllocMapped)))
    goto fail;
  if (!STS_CUDA_OK(cudaHostGetDevicePointer(&c->d_slots, c->h_slots, 0))) goto fail;
  memset(c->h_slots, 0, STS_NSLOTS * sizeof(double));
  if (!STS_CUDA_OK(cudaHostAlloc(&c->h_err, sizeof(int), cudaHostAllocMapped))) goto fail;
  if (!STS_CUDA_OK(cudaHostGetDevicePointer(&c->d_err, c->h_err, 0))) goto fail;
  *c->h_err = 0;
  *out = c;
  return 0;
fail:
  STS_ContextFree(&c);
  return -1;
}

extern "C" int STS_ContextFree(STS_Context* pc)
{
  if (!pc || !*pc) return 0;
  STS_Context c = *pc;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  if (c->d_work) cudaFree(c->d_work);
  if (c->h_slots) cudaFreeHost(c->h_slots);
  if (c->h_err) cudaFreeHost(c->h_err);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
  *pc = nullptr;
  return 0;
}

extern "C" int STS_ContextSynchronize(STS_Context ctx)
{
  if (!ctx) return -1;
  return STS_CUDA_OK(cudaStreamSynchronize(ctx->stream)) ? 0 : -1;
}

extern "C" void* STS_ContextGetStream(STS_Context ctx) { return ctx ? (void*)ctx->stream : nullptr; }

// ---------------------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------------------
enum EwOp { EW_LINSUM, EW_CONST, EW_PROD, EW_DIV, EW_SCALE, EW_ABS, EW_INV, EW_ADDCONST };

template <int OP>
__device__ __forceinline__ double ew_apply(double a, double b, double x, double y)
{
  if constexpr (OP == EW_LINSUM) return __fma_rn(a, x, __dmul_rn(b, y));
  else if constexpr (OP == EW_CONST) return a;
  else if constexpr (OP == EW_PROD) return __dmul_rn(x, y);
  else if constexpr (OP == EW_DIV) return __ddiv_rn(x, y);
  else if constexpr (OP == EW_SCALE) return __dmul_rn(a, x);
  else if constexpr (OP == EW_ABS) return fabs(x);
  else if constexpr (OP == EW_INV) return __drcp_rn(x);
  else return __dadd_rn(x, b);
}

template <int OP>
__global__ void __launch_bounds__(256) ew_kernel(long long n, double a, double b,
                                                 const double* __restrict__ x,
                                                 const double* __restrict__ y, double* z)
{
  const long long stride = (long long)gridDim.x * blockDim.x;
  long long i            = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  // two elements per thread per iteration (16-byte accesses when aligned)
  const long long n2 = n / 2;
  const bool aligned = ((((uintptr_t)x) | ((uintptr_t)y) | ((uintptr_t)z)) & 15) == 0;
  if (aligned)
  {
    for (long long k = i; k < n2; k += stride)
    {
      double2 xv = x ? reinterpret_cast<const double2*>(x)[k] : make_double2(0, 0);
      double2 yv = y ? reinterpret_cast<const double2*>(y)[k] : make_double2(0, 0);
      double2 r;
      r.x                                  = ew_apply<OP>(a, b, xv.x, yv.x);
      r.y                                  = ew_apply<OP>(a, b, xv.y, yv.y);
      reinterpret_cast<double2*>(z)[k]     = r;
    }
    if (i == 0 && (n & 1))
    {
      long long k = n - 1;
      z[k] = ew_apply<OP>(a, b, x ? x[k] : 0.0, y ? y[k] : 0.0);
    }
  }
  else
  {
    for (long long k = i; k < n; k += stride)
      z[k] = ew_apply<OP>(a, b, x ? x[k] : 0.0, y ? y[k] : 0.0);
  }
}

// z = sum_i c_i X_i, evaluated as fma chains in index order
constexpr int LC_MAX = 8;
struct LCArgs {
  double c[LC_MAX];
  const double* X[LC_MAX];
};

__global__ void __launch_bounds__(256) lincomb_kernel(long long n, int nvec, LCArgs args, double* z)
{
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += stride)
  {
    double acc = __dmul_rn(args.c[0], args.X[0][k]);
    for (int v = 1; v < nvec; ++v) acc = __fma_rn(args.c[v], args.X[v][k], acc);
    z[k] = acc;
  }
}

__global__ void __launch_bounds__(256) maxnorm_kernel(long long n, const double* __restrict__ x,
                                                      RedWork* w, double* slot)
{
  unsigned long long m   = 0;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += stride)
  {
    unsigned long long b = (unsigned long long)__double_as_longlong(fabs(x[k]));
    m                    = b > m ? b : m;
  }
#pragma unroll
  for (int s = 16; s >= 1; s >>= 1)
  {
    unsigned long long o = __shfl_xor_sync(0xffffffffu, m, s);
    m                    = o > m ? o : m;
  }
  __shared__ bool last;
  if ((threadIdx.x & 31) == 0 && m) atomicMax(&w->maxbits, m);
  __syncthreads();
  if (threadIdx.x == 0)
  {
    __threadfence();
    unsigned t = atomicAdd(&w->ticket, 1u);
    last       = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (last && threadIdx.x == 0)
  {
    __threadfence();
    unsigned long long b = atomicMax(&w->maxbits, 0ULL);
    *slot                = __longlong_as_double((long long)b);
    w->maxbits           = 0ULL;
    w->ticket            = 0u;
    __threadfence();
  }
}

// ---------------------------------------------------------------------------------------
// host wrappers
// ---------------------------------------------------------------------------------------
template <int OP>
static void ew_launch(STS_Context ctx, long long n, double a, double b, const double* x, const double* y,
                      double* z)
{
  if (n <= 0) return;
  ctx_activate(ctx);
  ew_kernel<OP><<<ew_blocks(ctx, n / 2 + 1, 256), 256, 0, ctx->stream>>>(n, a, b, x, y, z);
}

static double read_slot(STS_Context ctx, int slot)
{
  if (!STS_CUDA_OK(cudaStreamSynchronize(ctx->stream))) return NAN;
  return ((volatile double*)ctx->h_slots)[slot];
}

double sts_dot_exact(STS_Context ctx, const double* x, const double* y, long long n, int slot)
{
  ctx_activate(ctx);
  xred_kernel<0><<<ew_blocks(ctx, n, 256 * 4), 256, 0, ctx->stream>>>(n, x, y, ctx->d_work,
                                                                       ctx->d_slots + slot);
  return read_slot(ctx, slot);
}

// ---------------------------------------------------------------------------------------
// N_Vector
// ---------------------------------------------------------------------------------------
static N_Vector_Ops make_ops()
{
  N_Vector_Ops o          = (N_Vector_Ops)calloc(1, sizeof(struct _generic_N_Vector_Ops));
  o->nvclone              = N_VClone_Sts;
  o->nvcloneempty         = N_VCloneEmpty_Sts;
  o->nvdestroy            = N_VDestroy_Sts;
  o->nvspace              = N_VSpace_Sts;
  o->nvgetarraypointer    = N_VGetDeviceArrayPointer_Sts;
  o->nvgetlength          = N_VGetLength_Sts;
  o->nvlinearsum          = N_VLinearSum_Sts;
  o->nvconst              = N_VConst_Sts;
  o->nvprod               = N_VProd_Sts;
  o->nvdiv                = N_VDiv_Sts;
  o->nvscale              = N_VScale_Sts;
  o->nvabs                = N_VAbs_Sts;
  o->nvinv                = N_VInv_Sts;
  o->nvaddconst           = N_VAddConst_Sts;
  o->nvdotprod            = N_VDotProd_Sts;
  o->nvmaxnorm            = N_VMaxNorm_Sts;
  o->nvwrmsnorm           = N_VWrmsNorm_Sts;
  o->nvlinearcombination  = N_VLinearCombination_Sts;
  o->nvdotprodmulti       = N_VDotProdMulti_Sts;
  return o;
}

extern "C" N_Vector N_VNewEmpty_Sts(STS_Context ctx)
{
  if (!ctx)
  {
    sts_set_error("N_VNewEmpty_Sts: NULL context");
    return nullptr;
  }
  N_Vector v = (N_Vector)calloc(1, sizeof(struct _generic_N_Vector));
  v->ops     = make_ops();
  v->content = new NVContent();
  v->sunctx  = ctx;
  NVC(v)->device = ctx->device;
  return v;
}

extern "C" N_Vector N_VNew_Sts(sts_index length, STS_Context ctx)
{
  if (length < 0)
  {
    sts_set_error("N_VNew_Sts: negative length");
    return nullptr;
  }
  N_Vector v = N_VNewEmpty_Sts(ctx);
  if (!v) return nullptr;
  ctx_activate(ctx);
  NVContent* c = NVC(v);
  c->length    = length;
  c->nx        = length;
  c->ny        = 1;
  c->own       = true;
  size_t bytes = (size_t)(length > 0 ? length : 1) * sizeof(double);
  if (!STS_CUDA_OK(cudaMalloc(&c->data, bytes)) ||
      !STS_CUDA_OK(cudaMemsetAsync(c->data, 0, bytes, ctx->stream)) ||
      !STS_CUDA_OK(cudaStreamSynchronize(ctx->stream)))
  {
    N_VDestroy_Sts(v);
    return nullptr;
  }
  return v;
}

extern "C" N_Vector N_VMake_Sts(sts_index length, double* device_data, STS_Context ctx)
{
  N_Vector v = N_VNewEmpty_Sts(ctx);
  if (!v) return nullptr;
  NVContent* c = NVC(v);
  c->length    = length;
  c->nx        = length;
  c->ny        = 1;
  c->own       = false;
  c->data      = device_data;
  return v;
}

extern "C" N_Vector N_VCloneEmpty_Sts(N_Vector w)
{
  if (!w) return nullptr;
  N_Vector v = N_VNewEmpty_Sts(w->sunctx);
  if (!v) return nullptr;
  memcpy(v->ops, w->ops, sizeof(struct _generic_N_Vector_Ops)); // ops copied (N_VCopyOps)
  NVContent* c = NVC(v);
  c->length    = NVL(w);
  c->nx        = NVC(w)->nx;
  c->ny        = NVC(w)->ny;
  return v;
}

extern "C" N_Vector N_VClone_Sts(N_Vector w)
{
  if (!w) return nullptr;
  N_Vector v = N_VNew_Sts(NVL(w), w->sunctx);
  if (!v) return nullptr;
  memcpy(v->ops, w->ops, sizeof(struct _generic_N_Vector_Ops));
  NVC(v)->nx = NVC(w)->nx;
  NVC(v)->ny = NVC(w)->ny;
  return v;
}

extern "C" void N_VDestroy_Sts(N_Vector v)
{
  if (!v) return;
  NVContent* c = NVC(v);
  if (c)
  {
    if (c->own && c->data)
    { // cudaFree waits for work using the buffer; the context is not touched, so a vector
      // may outlive the context that made it
      int cur = -1;
      cudaGetDevice(&cur);
      if (cur != c->device) cudaSetDevice(c->device);
      cudaFree(c->data);
    }
    delete c;
  }
  free(v->ops);
  free(v);
}

extern "C" double* N_VGetDeviceArrayPointer_Sts(N_Vector v) { return v ? NVD(v) : nullptr; }
extern "C" sts_index N_VGetLength_Sts(N_Vector v) { return v ? NVL(v) : 0; }

extern "C" void N_VSpace_Sts(N_Vector v, sts_index* lrw, sts_index* liw)
{
  *lrw = v ? NVL(v) : 0;
  *liw = 0;
}

extern "C" int N_VSetShape_Sts(N_Vector v, sts_index nx, sts_index ny)
{
  if (!v || nx * ny != NVL(v)) return -1;
  NVC(v)->nx = nx;
  NVC(v)->ny = ny;
  return 0;
}

extern "C" int N_VCopyFromHost_Sts(N_Vector v, const double* host)
{
  if (!v || !host) return -1;
  ctx_activate(v->sunctx);
  if (!STS_CUDA_OK(cudaMemcpyAsync(NVD(v), host, NVL(v) * sizeof(double), cudaMemcpyHostToDevice,
                                   v->sunctx->stream)))
    return -1;
  return STS_CUDA_OK(cudaStreamSynchronize(v->sunctx->stream)) ? 0 : -1;
}

extern "C" int N_VCopyToHost_Sts(N_Vector v, double* host)
{
  if (!v || !host) return -1;
  ctx_activate(v->sunctx);
  if (!STS_CUDA_OK(cudaMemcpyAsync(host, NVD(v), NVL(v) * sizeof(double), cudaMemcpyDeviceToHost,
                                   v->sunctx->stream)))
    return -1;
  return STS_CUDA_OK(cudaStreamSynchronize(v->sunctx->stream)) ? 0 : -1;
}

extern "C" void N_VLinearSum_Sts(double a, N_Vector x, double b, N_Vector y, N_Vector z)
{
  ew_launch<EW_LINSUM>(z->sunctx, NVL(z), a, b, NVD(x), NVD(y), NVD(z));
}
extern "C" void N_VConst_Sts(double c, N_Vector z)
{
  ew_launch<EW_CONST>(z->sunctx, NVL(z), c, 0.0, nullptr, nullptr, NVD(z));
}
extern "C" void N_VProd_Sts(N_Vector x, N_Vector y, N_Vector z)
{
  ew_launch<EW_PROD>(z->sunctx, NVL(z), 0.0, 0.0, NVD(x), NVD(y), NVD(z));
}
extern "C" void N_VDiv_Sts(N_Vector x, N_Vector y, N_Vector z)
{
  ew_launch<EW_DIV>(z->sunctx, NVL(z), 0.0, 0.0, NVD(x), NVD(y), NVD(z));
}
extern "C" void N_VScale_Sts(double c, N_Vector x, N_Vector z)
{
  ew_launch<EW_SCALE>(z->sunctx, NVL(z), c, 0.0, NVD(x), nullptr, NVD(z));
}
extern "C" void N_VAbs_Sts(N_Vector x, N_Vector z)
{
  ew_launch<EW_ABS>(z->sunctx, NVL(z), 0.0, 0.0, NVD(x), nullptr, NVD(z));
}
extern "C" void N_VInv_Sts(N_Vector x, N_Vector z)
{
  ew_launch<EW_INV>(z->sunctx, NVL(z), 0.0, 0.0, NVD(x), nullptr, NVD(z));
}
extern "C" void N_VAddConst_Sts(N_Vector x, double b, N_Vector z)
{
  ew_launch<EW_ADDCONST>(z->sunctx, NVL(z), 0.0, b, NVD(x), nullptr, NVD(z));
}

extern "C" double N_VDotProd_Sts(N_Vector x, N_Vector y)
{
  return sts_dot_exact(x->sunctx, NVD(x), NVD(y), NVL(x), SLOT_GENERIC);
}

extern "C" double N_VWrmsNorm_Sts(N_Vector x, N_Vector w)
{
  STS_Context ctx = x->sunctx;
  long long n     = NVL(x);
  ctx_activate(ctx);
  xred_kernel<1><<<ew_blocks(ctx, n, 256 * 4), 256, 0, ctx->stream>>>(n, NVD(x), NVD(w), ctx->d_work,
                                                                       ctx->d_slots + SLOT_GENERIC);
  return read_slot(ctx, SLOT_GENERIC);
}

extern "C" double N_VMaxNorm_Sts(N_Vector x)
{
  STS_Context ctx = x->sunctx;
  long long n     = NVL(x);
  ctx_activate(ctx);
  maxnorm_kernel<<<ew_blocks(ctx, n, 256 * 4), 256, 0, ctx->stream>>>(n, NVD(x), ctx->d_work,
                                                                       ctx->d_slots + SLOT_GENERIC);
  return read_slot(ctx, SLOT_GENERIC);
}

// N_VDotProdMulti: the exact dot products of x with Y[0..nvec-1], each written to its own
// result slot; one stream synchronisation per STS_NSLOTS - SLOT_MULTI products
extern "C" int N_VDotProdMulti_Sts(int nvec, N_Vector x, N_Vector* Y, double* dots)
{
  if (nvec < 1 || !x || !Y || !dots) return -1;
  STS_Context ctx = x->sunctx;
  long long n     = NVL(x);
  ctx_activate(ctx);
  constexpr int CH = STS_NSLOTS - SLOT_MULTI;
  for (int c0 = 0; c0 < nvec; c0 += CH)
  {
    const int cnt = std::min(CH, nvec - c0);
    for (int k = 0; k < cnt; ++k)
    {
      if (NVL(Y[c0 + k]) != n) return -1;
      xred_kernel<0><<<ew_blocks(ctx, n, 256 * 4), 256, 0, ctx->stream>>>(n, NVD(x), NVD(Y[c0 + k]), ctx->d_work,
                                                                           ctx->d_slots + SLOT_MULTI + k);
    }
    if (!STS_CUDA_OK(cudaStreamSynchronize(ctx->stream))) return -1;
    for (int k = 0; k < cnt; ++k) dots[c0 + k] = ((volatile double*)ctx->h_slots)[SLOT_MULTI + k];
  }
  return 0;
}

extern "C" int N_VLinearCombination_Sts(int nvec, double* c, N_Vector* X, N_Vector z)
{
  if (nvec < 1) return -1;
  STS_Context ctx = z->sunctx;
  long long n     = NVL(z);
  ctx_activate(ctx);
  // chunks of LC_MAX vectors: z = sum_{first chunk}; then z += further chunks
  int done = 0;
  while (done < nvec)
  {
    LCArgs a{};
    int cnt = 0;
    if (done > 0)
    {
      a.c[0] = 1.0;
      a.X[0] = NVD(z);
      cnt    = 1;
    }
    while (cnt < LC_MAX && done < nvec)
    {
      a.c[cnt] = c[done];
      a.X[cnt] = NVD(X[done]);
      ++cnt;
      ++done;
    }
    lincomb_kernel<<<ew_blocks(ctx, n, 256), 256, 0, ctx->stream>>>(n, cnt, a, NVD(z));
  }
  return STS_CUDA_OK(cudaGetLastError()) ? 0 : -1;
}

// host-side exact sum (same limb arithmetic as the device reductions)
extern "C" double STS_ExactSumHost(const double* x, sts_index n)
{
  xsum::Limbs a;
  xsum::zero(a);
  unsigned f = 0;
  for (long long i = 0; i < n; ++i) xsum::add(a, x[i], f);
  return xsum::finalize(a.l, f);
}
