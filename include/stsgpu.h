/* stsgpu.h — C ABI of the GB300 (sm_103a) diffusion_2D super-time-stepping library.
 *
 * The entry points mirror the interfaces through which the reference's diffusion_2D
 * driver reaches its hot path (SUNDIALS ARKODE/LSRKStep, NVECTOR, SUNLinearSolver and the
 * problem callbacks). Each declaration names the reference interface it replaces
 * (file:line, paths relative to the sundials-codes/ceda-demonstrations tree). SUNDIALS is
 * an empty submodule there, so SUNDIALS functions are cited at their call sites in
 * diffusion_2D/main.cpp and the gkeyll_diffusion C sources.
 *
 * Conventions
 *   - plain C types only: double, float, int, long long, opaque handles, raw pointers;
 *   - all vector data lives in device (HBM) memory; N_Vector ops are asynchronous on the
 *     context's CUDA stream except reductions, which synchronise and return host doubles;
 *   - functions returning int use 0 = success, > 0 = recoverable, < 0 = failure
 *     (the ARKODE / callback convention of diffusion_2D.cpp:900-933);
 *   - constructors return NULL on failure; STS_GetLastError() gives the reason.
 */
#ifndef STSGPU_H
#define STSGPU_H

#ifdef __cplusplus
extern "C" {
#endif

typedef long long sts_index; /* sunindextype (64-bit index build) */

/* ------------------------------------------------------------------------------------
 * Context. Replaces SUNContext (SUNContext_Create, diffusion_2D/main.cpp:79): owns the
 * CUDA stream and the reduction workspace of one device.
 * ----------------------------------------------------------------------------------*/
typedef struct STS_Context_* STS_Context;
int STS_ContextCreate(int device, STS_Context* ctx);
int STS_ContextFree(STS_Context* ctx);
int STS_ContextSynchronize(STS_Context ctx);
void* STS_ContextGetStream(STS_Context ctx); /* cudaStream_t */
const char* STS_GetLastError(void);
int STS_DeviceCount(void);
/* Failure-detection self-test (no reference counterpart; the reference has no device-side
 * waits). Every spin on a pipeline barrier in this library is bounded: a wait that runs out
 * sets the context's error word, the kernel drains what it has in flight and returns, and the
 * host turns the word into STS_ERR_FAILURE with the context still usable. This entry point
 * runs that path on one barrier: with `arrive` nonzero the barrier completes and the call
 * returns STS_SUCCESS; with `arrive` 0 nothing arrives, the wait gives up after `limit` polls
 * (1 .. 2^20) and the call returns STS_ERR_FAILURE and clears the word. */
int STS_WaitSelfTest(STS_Context ctx, int arrive, long long limit);

/* ------------------------------------------------------------------------------------
 * N_Vector (device). Layout {content, ops, sunctx} as SUNDIALS' generic N_Vector; the ops
 * table holds the subset LSRKStep, the PCG solver and the Jacobi PSolve use
 * (gkeyll_diffusion/src/nvector_gkylzero.c:45-60, + nvprod for
 * diffusion_2D/preconditioner_jacobi.cpp:58, + nvlinearcombination and nvdotprodmulti).
 * ----------------------------------------------------------------------------------*/
typedef struct _generic_N_Vector* N_Vector;
typedef struct _generic_N_Vector_Ops* N_Vector_Ops;

struct _generic_N_Vector_Ops {
  N_Vector (*nvclone)(N_Vector);
  N_Vector (*nvcloneempty)(N_Vector);
  void (*nvdestroy)(N_Vector);
  void (*nvspace)(N_Vector, sts_index*, sts_index*);
  double* (*nvgetarraypointer)(N_Vector);
  sts_index (*nvgetlength)(N_Vector);
  void (*nvlinearsum)(double, N_Vector, double, N_Vector, N_Vector);
  void (*nvconst)(double, N_Vector);
  void (*nvprod)(N_Vector, N_Vector, N_Vector);
  void (*nvdiv)(N_Vector, N_Vector, N_Vector);
  void (*nvscale)(double, N_Vector, N_Vector);
  void (*nvabs)(N_Vector, N_Vector);
  void (*nvinv)(N_Vector, N_Vector);
  void (*nvaddconst)(N_Vector, double, N_Vector);
  double (*nvdotprod)(N_Vector, N_Vector);
  double (*nvmaxnorm)(N_Vector);
  double (*nvwrmsnorm)(N_Vector, N_Vector);
  int (*nvlinearcombination)(int, double*, N_Vector*, N_Vector);
  int (*nvdotprodmulti)(int, N_Vector, N_Vector*, double*);
};

struct _generic_N_Vector {
  void* content;
  N_Vector_Ops ops;
  STS_Context sunctx;
};

/* N_VNew_Parallel (diffusion_2D/main.cpp:176): owned device vector, zero-filled */
N_Vector N_VNew_Sts(sts_index length, STS_Context ctx);
/* N_VNewEmpty_Gkylzero (nvector_gkylzero.c:32-82) */
N_Vector N_VNewEmpty_Sts(STS_Context ctx);
/* N_VMake_Gkylzero (nvector_gkylzero.c:85-99): wrap caller-owned device memory */
N_Vector N_VMake_Sts(sts_index length, double* device_data, STS_Context ctx);
/* N_VCloneEmpty/Clone/Destroy_Gkylzero (nvector_gkylzero.c:111-203) */
N_Vector N_VCloneEmpty_Sts(N_Vector w);
N_Vector N_VClone_Sts(N_Vector w);
void N_VDestroy_Sts(N_Vector v);
/* N_VGetArrayPointer (diffusion_2D/diffusion.cpp:24,27): DEVICE pointer */
double* N_VGetDeviceArrayPointer_Sts(N_Vector v);
sts_index N_VGetLength_Sts(N_Vector v);
/* N_VSpace_Gkylzero (nvector_gkylzero.c:407-411) */
void N_VSpace_Sts(N_Vector v, sts_index* lrw, sts_index* liw);
/* 2-D shape (nx fastest, IDX(i,j,nx) = nx*j + i, diffusion_2D.hpp:55); informational */
int N_VSetShape_Sts(N_Vector v, sts_index nx, sts_index ny);
/* host <-> device copies (synchronous on the context stream) */
int N_VCopyFromHost_Sts(N_Vector v, const double* host);
int N_VCopyToHost_Sts(N_Vector v, double* host);

/* nvector_gkylzero.c:205-514 */
void N_VLinearSum_Sts(double a, N_Vector x, double b, N_Vector y, N_Vector z);
void N_VConst_Sts(double c, N_Vector z);
void N_VProd_Sts(N_Vector x, N_Vector y, N_Vector z);
void N_VDiv_Sts(N_Vector x, N_Vector y, N_Vector z);
void N_VScale_Sts(double c, N_Vector x, N_Vector z);
void N_VAbs_Sts(N_Vector x, N_Vector z);
void N_VInv_Sts(N_Vector x, N_Vector z);
void N_VAddConst_Sts(N_Vector x, double b, N_Vector z);
/* reductions: exact, order-independent accumulation (terms truncated to 2^-160, summed
 * exactly, rounded once); the values do not depend on the launch shape */
double N_VDotProd_Sts(N_Vector x, N_Vector y);
double N_VMaxNorm_Sts(N_Vector x);
double N_VWrmsNorm_Sts(N_Vector x, N_Vector w);
int N_VLinearCombination_Sts(int nvec, double* c, N_Vector* X, N_Vector z);
/* N_VDotProdMulti (SUNDIALS fused op, used by SPGMR's classical Gram-Schmidt): dots[k] =
 * exact x . Y[k]; returns 0, or -1 on a length mismatch or a CUDA error */
int N_VDotProdMulti_Sts(int nvec, N_Vector x, N_Vector* Y, double* dots);

/* Allocation-free WRMS norm. No counterpart in the reference: it exists for callers that
 * cannot allocate device or pinned memory when they need a norm (work recorded into another
 * runtime's CUDA graph or fixed memory pool, real-time loops, foreign vector libraries that
 * hold raw device pointers but no STS_Context). Computes the same exact value as
 * N_VWrmsNorm_Sts: sqrt(sum_i (x_i w_i)^2 / n) over device arrays x, w of length n, written
 * to the device location `result`, asynchronously on `stream` (a cudaStream_t, NULL = the
 * default stream). It calls no cudaMalloc/cudaFree: its scratch is one fixed 96-byte block
 * per CUDA context in a static device array held until the library is unloaded. A call on
 * a stream that is not being captured looks that block up (cudaGetSymbolAddress, in the
 * context current on the calling thread); a call on a capturing stream reuses the address
 * found by an earlier call in the same context, so the first call in each context (also the
 * new context after a cudaDeviceReset) must come before any stream capture. Each call clears
 * the block first; calls that overlap on the GPU race on it.
 * n must lie in [1, STS_NOALLOC_MAX_N]; otherwise -1 and STS_GetLastError() says why. */
#define STS_NOALLOC_MAX_N 2147483647LL
int STS_WrmsNormNoAlloc(const double* x, const double* w, sts_index n, double* result,
                        void* stream);

/* ------------------------------------------------------------------------------------
 * Problem and callbacks (diffusion_2D). STS_Problem replaces UserData
 * (diffusion_2D/diffusion_2D.hpp:66-214) for the single-device case.
 * ----------------------------------------------------------------------------------*/
#define STS_PROBLEM_MANUFACTURED 0 /* [0,1]^2 Dirichlet, u = sin^2(pi x) sin^2(pi y) cos^2(2 pi t) */
#define STS_PROBLEM_UNFORCED 1     /* [0,1]^2 Dirichlet, no forcing */
#define STS_PROBLEM_PERIODIC 2     /* reference mode: periodic, initial.cpp:42-43 IC */

typedef struct STS_Problem_* STS_Problem;
STS_Problem STS_ProblemCreate(STS_Context ctx, int kind, sts_index nx, sts_index ny, double kx,
                              double ky, int inhomogeneous, double xl, double xu, double yl,
                              double yu);
int STS_ProblemFree(STS_Problem* p);
int STS_ProblemGetInfo(STS_Problem p, double* dx, double* dy, double* cx, double* cy);
/* Initial (diffusion_2D/initial.cpp:20-47) */
int STS_Initial(double t, N_Vector u, STS_Problem p);
/* sum_k a_k sin(p_k pi x) sin(q_k pi y) (batched initial condition) */
int STS_InitialModes(N_Vector u, STS_Problem p, int nmodes, const int* pm, const int* qm,
                     const double* amp);
int STS_Exact(double t, N_Vector u, STS_Problem p);
/* ARKRhsFn diffusion (diffusion_2D/diffusion_2D.cpp:23-35 -> diffusion.cpp:9-209) */
int STS_Diffusion(double t, N_Vector u, N_Vector f, void* user_data);
/* J v = A v (the RHS is affine) */
int STS_JacTimes(N_Vector v, N_Vector Jv, double t, N_Vector y, N_Vector fy, void* user_data,
                 N_Vector tmp);
/* ARKDomEigFn dom_eig (diffusion_2D/main.cpp:536-550) */
int STS_DomEig(double t, N_Vector y, N_Vector fn, double* lambdaR, double* lambdaI,
               void* user_data, N_Vector temp1, N_Vector temp2, N_Vector temp3);
/* SUNDomEigEstimator_Power (diffusion_2D/main.cpp:344): power iteration on A from v */
int STS_PowerIteration(STS_Problem p, N_Vector v, int maxiters, double reltol, double* lambda,
                       int* iters);
/* ARKLsPrecSetupFn / ARKLsPrecSolveFn (diffusion_2D/preconditioner_jacobi.cpp:9-61) */
int STS_PSetup(double t, N_Vector u, N_Vector f, int jok, int* jcurPtr, double gamma,
               void* user_data);
int STS_PSolve(double t, N_Vector u, N_Vector f, N_Vector r, N_Vector z, double gamma,
               double delta, int lr, void* user_data);

/* ------------------------------------------------------------------------------------
 * LSRKStep STS integrator (ARKODE). Replaces LSRKStepCreateSTS and the ARKode* calls of
 * diffusion_2D/main.cpp:257-400,442,486. When the RHS is STS_Diffusion with an STS_Problem
 * as user data, stages run as fused stencil+stage kernels; any other ARKRhsFn runs through
 * the N_Vector ops (generic path).
 * ----------------------------------------------------------------------------------*/
typedef int (*STS_ARKRhsFn)(double t, N_Vector y, N_Vector ydot, void* user_data);
typedef int (*STS_ARKDomEigFn)(double t, N_Vector y, N_Vector fn, double* lambdaR,
                               double* lambdaI, void* user_data, N_Vector temp1,
                               N_Vector temp2, N_Vector temp3);

#define STS_LSRK_RKC_2 0 /* ARKODE_LSRK_RKC_2 */
#define STS_LSRK_RKL_2 1 /* ARKODE_LSRK_RKL_2 */
#define STS_LSRK_SSP_S_2 2  /* ARKODE_LSRK_SSP_S_2 */
#define STS_LSRK_SSP_S_3 3  /* ARKODE_LSRK_SSP_S_3 */
#define STS_LSRK_SSP_10_4 4 /* ARKODE_LSRK_SSP_10_4 */
#define STS_ADAPT_PID 0  /* ARK_ADAPT_PID */
#define STS_ADAPT_PI 1   /* ARK_ADAPT_PI */
#define STS_ADAPT_I 2    /* ARK_ADAPT_I */
#define STS_ADAPT_EXP_GUS 3  /* ARK_ADAPT_EXP_GUS */
#define STS_ADAPT_IMP_GUS 4  /* ARK_ADAPT_IMP_GUS */
#define STS_ADAPT_IMEX_GUS 5 /* ARK_ADAPT_IMEX_GUS */
#define STS_NORMAL 1     /* ARK_NORMAL */
#define STS_ONE_STEP 2   /* ARK_ONE_STEP */
#define STS_SUCCESS 0
#define STS_TSTOP_RETURN 1
#define STS_TOO_MUCH_WORK -1
#define STS_ERR_FAILURE -3
#define STS_RHSFUNC_FAIL -8
#define STS_ILL_INPUT -22
#define STS_MEM_NULL -21

typedef struct STS_Stats {
  long long nst, nst_attempts, netf, nfe, nfe_dee, ndee, nst_exp, stage_max, stages_total;
  double t, hlast, hnext, spectral_radius;
} STS_Stats;

void* STS_LSRKStepCreateSTS(STS_ARKRhsFn rhs, double t0, N_Vector y0, STS_Context ctx); /* main.cpp:257 */
int STS_LSRKStepSetSTSMethod(void* mem, int method);
/* LSRKStepCreateSSP / LSRKStepSetSSPMethod / LSRKStepSetNumSSPStages (diffusion_2D/main.cpp:
 * 250-294): SSP(s,2) (s >= 2, default 10), SSP(s,3) (s = n^2 >= 4, default 9), SSP(10,4);
 * integrated through the N_Vector ops with an embedded error estimate (first / second / third
 * order) and the same step-size controllers */
void* STS_LSRKStepCreateSSP(STS_ARKRhsFn rhs, double t0, N_Vector y0, STS_Context ctx);
int STS_LSRKStepSetSSPMethod(void* arkode_mem, int type);
int STS_LSRKStepSetNumSSPStages(void* arkode_mem, int num_stages);
/* host helper: weights b, stage times c, error weights w = b - bhat of an SSP method */
int STS_LSRKSSPWeights(int type, int s, double* b, double* c, double* w);                 /* main.cpp:336-338 */
int STS_ARKodeSStolerances(void* mem, double rtol, double atol);      /* main.cpp:262 */
int STS_ARKodeSetUserData(void* mem, void* user_data);                /* main.cpp:266 */
int STS_LSRKStepSetDomEigFn(void* mem, STS_ARKDomEigFn fn);           /* main.cpp:352 */
int STS_LSRKStepSetDomEigEstimatorPower(void* mem, int maxiters, double reltol);
/* LSRKStepSetNumDomEigEstInitPreprocessIters / ...PreprocessIters
 * (gkeyll_diffusion/gk_diffusion_1x1v_p1.c:873-885): warm-up power iterations before the
 * first / every later estimate of the power-iteration estimator */
int STS_LSRKStepSetNumDomEigEstInitPreprocessIters(void* arkode_mem, int iters);
int STS_LSRKStepSetNumDomEigEstPreprocessIters(void* arkode_mem, int iters); /* main.cpp:344-348 */
int STS_LSRKStepSetDomEigFrequency(void* mem, long long nsteps);      /* gk_diffusion_1x1v_p1.c / analytic_CR_test.c:320 */
int STS_LSRKStepSetMaxNumStages(void* mem, int smax);                 /* analytic_CR_test.c:324 */
int STS_LSRKStepSetDomEigSafetyFactor(void* mem, double safety);      /* analytic_CR_test.c:332 */
int STS_ARKodeSetAdaptController(void* mem, int controller);          /* main.cpp:366-376 */
int STS_ARKodeSetFixedStep(void* mem, double h);                      /* main.cpp:361 */
int STS_ARKodeSetMaxNumSteps(void* mem, long long mxsteps);           /* main.cpp:380 */
/* the step that would pass tstop ends on it; the call returns STS_TSTOP_RETURN there and the
 * stop time is cleared (set it again for the next one, main.cpp:437-441) */
int STS_ARKodeSetStopTime(void* mem, double tstop);                   /* main.cpp:384 */
/* new: FP32 stage increments relative to the FP64 step-start state (fused path only) */
int STS_LSRKStepSetMixedPrecision(void* mem, int on);
/* new: mixed-stage kernel selection: 0 = autotuned at the first step among the TMA +
 * mbarrier pipelined tile configurations (rows per tile, ring depth, CTAs per SM; row length
 * a multiple of 4) and the register-marching kernel (default), 1 = register-marching kernel,
 * 2 + k = TMA configuration k (k < 6). All variants give identical bits. */
int STS_LSRKStepSetStageKernel(void* mem, int variant);
/* new: the autotuner's choice (-1 = register-marching), its time per launch and its name */
int STS_LSRKStepGetStageKernelInfo(void* mem, int* variant, double* ms_per_launch, char* name,
                                   int namelen);
/* new: mixed form, several stages per launch (temporal blocking on 120-column tiles in shared
   memory, the same bits as one launch per stage). ks: 0 = autotuned (default: four stages per
   launch when the autotuner times that faster than one), 1 = off, 2..4 = that many; config:
   0 = autotuned, 1..6 = tile configuration (1: 120 x 32, three CTAs per SM; 2, 3, 5: 120 x 64,
   120 x 60 and 120 x 58, two CTAs of 256 threads per SM; 4: 120 x 64, two CTAs of 384 threads;
   6: 120 x 64, one CTA of 256 threads per SM with two tile buffers).
   Applies with the autotuned stage kernel (STS_LSRKStepSetStageKernel variant 0). */
int STS_LSRKStepSetStageFusion(void* mem, int ks, int config);
/* new: the stages per launch in use (1: none), the tile configuration (0: none) and its rows,
   and the autotuner's time per four-stage launch */
int STS_LSRKStepGetStageFusion(void* mem, int* ks, int* config, int* tile_rows, double* ms_per_launch);
/* new: capture the fixed-s stage loop of the fused path in CUDA graphs (default on) */
int STS_LSRKStepSetUseGraphs(void* mem, int on);
/* new: reference mode (STS_PROBLEM_PERIODIC with STS_Diffusion): fused stage and step-end
 * kernels (default on) or the plain RHS + N_Vector sequence; both give identical bits */
int STS_LSRKStepSetFusedPeriodic(void* mem, int on);
/* ARKodeEvolve (main.cpp:442). STS_NORMAL steps until t_n >= tout (only a stop time clips a
 * step) and returns the dense output at tret = tout: ARKODE's Hermite interpolant on the last
 * step, degree min(q - 1, 5) for a method of order q (RKC2, RKL2, SSP(s,2), DIRK2, ERK2: 1;
 * SSP(s,3), DIRK3, ERK3: 2; SSP(10,4), ERK4: 3); a tout the last step already passed is
 * answered without stepping. STS_ONE_STEP takes one step and returns y_n, t_n. A reached stop
 * time returns y_n with STS_TSTOP_RETURN. */
int STS_ARKodeEvolve(void* mem, double tout, N_Vector yout, double* tret, int itask);
/* ARKodeReset: restart from (t, y) keeping options, counters and the step size; F(t, y) is
 * re-evaluated on the next step */
int STS_ARKodeReset(void* mem, double t, N_Vector y);
/* Checkpoint / restart (new; the reference writes only text snapshots of u,
 * diffusion_2D.cpp:729-842): the full integrator state (t, step-size and controller history,
 * eigenvalue estimate and refresh counter, statistics, y_n, the FSAL F_n, the mixed path's
 * FP32 copy of F_n and the power-iteration vector) to one binary file. Reading it into an
 * integrator created for the same problem size, method and precision continues the run
 * with the same step sequence and bits as the uninterrupted one. */
int STS_LSRKStepWriteCheckpoint(void* arkode_mem, const char* path);
int STS_LSRKStepReadCheckpoint(void* arkode_mem, const char* path);
/* CUDA-event timing of the fused stage kernel on the integrator's current buffers (after at
 * least one evolve): average milliseconds per launch over nlaunch launches of stage j = s/2
 * of the last step (with several stages per launch: of the group starting there), launched
 * on the context stream exactly as the integrator does */
int STS_LSRKStepTimeStageKernel(void* mem, int nlaunch, double* ms_per_launch);
int STS_ARKodeGetStats(void* mem, STS_Stats* stats);                  /* ARKodePrintAllStats main.cpp:486 */
int STS_ARKodePrintAllStats(void* mem, char* buf, int buflen);
void STS_ARKodeFree(void** mem);                                     /* main.cpp:505 */

/* ------------------------------------------------------------------------------------
 * ARKStep (ARKODE's additive RK stepper) in the two forms diffusion_2D/main.cpp:239-253
 * creates: ARKStepCreate(nullptr, fi, ...) -> implicit DIRK (--integrator dirk) with a
 * Newton iteration on each stage, its linear systems solved by a SUNLinearSolver with the
 * user's PSetup / PSolve (main.cpp:199-231, 296-330); ARKStepCreate(fe, nullptr, ...) ->
 * explicit ERK (--integrator erk with --order >= 0). Methods (ARKodeSetOrder): implicit
 * 2 = ARKODE_SDIRK_2_1_2, 3 = ARKODE_ARK324L2SA_DIRK_4_2_3 (the default); explicit
 * 2 = ARKODE_HEUN_EULER_2_1_2, 3 = ARKODE_BOGACKI_SHAMPINE_4_2_3, 4 = ARKODE_ZONNEVELD_5_3_4
 * (the default). The returned handle takes the ARKode* calls above (tolerances, user data,
 * controller, fixed step, max steps, stop time, Evolve, Reset, GetStats, PrintAllStats, Free).
 * ----------------------------------------------------------------------------------*/
#define STS_CONV_FAILURE -4 /* ARK_CONV_FAILURE */
typedef int (*STS_ARKLsPrecSetupFn)(double t, N_Vector y, N_Vector fy, int jok, int* jcurPtr,
                                    double gamma, void* user_data);
typedef int (*STS_ARKLsPrecSolveFn)(double t, N_Vector y, N_Vector fy, N_Vector r, N_Vector z,
                                    double gamma, double delta, int lr, void* user_data);
void* STS_ARKStepCreate(STS_ARKRhsFn fe, STS_ARKRhsFn fi, double t0, N_Vector y0,
                        STS_Context ctx);                                   /* main.cpp:239-248 */
int STS_ARKodeSetOrder(void* mem, int order);                               /* main.cpp:272, 297 */
int STS_ARKodeSetLinearSolver(void* mem, void* LS, void* A);               /* main.cpp:305 */
int STS_ARKodeSetPreconditioner(void* mem, STS_ARKLsPrecSetupFn psetup,
                                STS_ARKLsPrecSolveFn psolve);               /* main.cpp:311 */
/* new: the user data PSetup / PSolve receive, where it differs from the RHS's (the reference
 * keeps both in one UserData; here e.g. an STS_PFMG beside the STS_Problem). NULL: the RHS's */
int STS_ARKStepSetPrecData(void* mem, void* pdata);
int STS_ARKodeSetLSetupFrequency(void* mem, int msbp);                     /* main.cpp:315 */
int STS_ARKodeSetEpsLin(void* mem, double eplifac);                        /* main.cpp:320 */
int STS_ARKodeSetLinear(void* mem, int timedepend);                        /* main.cpp:326 */
int STS_ARKodeSetNonlinear(void* mem); /* the --nonlinear default of ARKODE (main.cpp:630) */
typedef struct STS_ARKStepStats {
  long long nst, nst_attempts, netf, ncfn, nfe, nfi, nfe_ls, nni, nnf, nli, nlcf, npe, nps, njv,
      nsetups;
  double t, h0, hlast, hnext;
} STS_ARKStepStats;
int STS_ARKStepGetStats(void* mem, STS_ARKStepStats* stats); /* ARKodePrintAllStats main.cpp:486 */
/* host helper: the Butcher table (A row-major s x s, b, embedding d, c) of a method */
int STS_ARKStepTable(int implicit, int order, int* s, int* q, int* p, double* A, double* b,
                     double* d, double* c);

/* new (measurement): the FP64 FMA rate of the current device in TFLOP/s (2 flops per FMA),
 * from a probe kernel of independent FMA chains timed with CUDA events; the denominator the
 * FP64 stage kernel's rate is reported against */
int STS_ProbeFP64Rate(STS_Context ctx, double* tflops);

/* host-only helpers (no device work): the integrator's coefficient and step-size rules */
int STS_LSRKStageCoeffs(int method, int s, double* mu, double* nu, double* mus, double* ajm1,
                        double* cjm1);
int STS_LSRKStagesNeeded(int method, double h, double rho, int smax, double* hmax);
double STS_AdaptControllerEstimate(int controller, double h, double dsm, double ep1, double ep2,
                                   double hp, long long nhist);
int STS_ManufacturedTables(sts_index n, double d, double* S, double* Sdd);
double STS_ExactSumHost(const double* x, sts_index n);

/* ------------------------------------------------------------------------------------
 * Implicit comparator: SUNLinSol_PCG with the Jacobi preconditioner
 * (diffusion_2D/main.cpp:207-212, 305-316; preconditioner_jacobi.cpp). The fused solver
 * solves (I - gamma A) x = b for the problem's operator A with x0 = 0.
 * ----------------------------------------------------------------------------------*/
#define STS_PREC_NONE 0  /* SUN_PREC_NONE */
#define STS_PREC_RIGHT 2 /* SUN_PREC_RIGHT */
typedef int (*STS_ATimesFn)(void* A_data, N_Vector v, N_Vector z);
typedef int (*STS_PSolveFn)(void* P_data, N_Vector r, N_Vector z, double tol, int lr);

void* STS_SUNLinSol_PCG(N_Vector y, int pretype, int maxl, STS_Context ctx); /* main.cpp:211 */
/* SUNLinSol_SPGMR (main.cpp:216, --ls gmres): restarted GMRES(maxl), right preconditioning,
 * maxl <= 1000; SUNLinSol_SPGMRSetMaxRestarts (default 0) / SetGSType (default modified) */
#define STS_MODIFIED_GS 1  /* SUN_MODIFIED_GS */
#define STS_CLASSICAL_GS 2 /* SUN_CLASSICAL_GS (with one re-orthogonalisation pass) */
void* STS_SUNLinSol_SPGMR(N_Vector y, int pretype, int maxl, STS_Context ctx);
int STS_SUNLinSol_SPGMRSetMaxRestarts(void* LS, int maxrs);
int STS_SUNLinSol_SPGMRSetGSType(void* LS, int gstype);
/* SUNLinSol_SPFGMR (SUNDIALS' flexible GMRES, the Krylov method for a preconditioner that may
 * change between applications, e.g. the learned network below): restarted FGMRES(maxl), right
 * preconditioning only (any other nonzero pretype is taken as right), maxl <= 1000; it keeps
 * the preconditioned basis and updates x += Z y. SetMaxRestarts / SetGSType as for SPGMR. */
void* STS_SUNLinSol_SPFGMR(N_Vector y, int pretype, int maxl, STS_Context ctx);
int STS_SUNLinSol_SPFGMRSetMaxRestarts(void* LS, int maxrs);
int STS_SUNLinSol_SPFGMRSetGSType(void* LS, int gstype);
int STS_SUNLinSolSetATimes(void* LS, void* A_data, STS_ATimesFn atimes);
int STS_SUNLinSolSetPreconditioner(void* LS, void* P_data, STS_PSolveFn psolve);
/* solve A x = b from x0 = 0 through the callbacks; stop when ||r||_2 <= delta ||b||_2 (PCG:
 * the recurrence residual; SPGMR: the Givens residual estimate). Returns 0 converged, 1 not
 * converged within maxl iterations (SPGMR: maxl (max_restarts + 1)) or a callback failed,
 * -1 illegal input */
int STS_SUNLinSolSolve(void* LS, N_Vector x, N_Vector b, double delta);
int STS_SUNLinSolNumIters(void* LS);
double STS_SUNLinSolResNorm(void* LS);
int STS_SUNLinSolFree(void* LS);
/* fused (I - gamma A) x = b solve with Jacobi (jacobi=1) or no preconditioner */
int STS_ImplicitSolvePCG(STS_Problem p, double gamma, N_Vector b, N_Vector x, double tol,
                         int maxit, int jacobi, int* iters, double* relres);
/* fixed-step SDIRK2 with fused Jacobi-PCG stage solves (ARKStep DIRK, main.cpp:242,272) */
int STS_SDIRK2Evolve(STS_Problem p, N_Vector y, double t0, double h, int nsteps, double tol,
                     int maxit, long long* total_iters);
/* fixed-step SDIRK2 whose stage systems (I - gamma h A) d = rhs are solved by a generic
 * SUNLinearSolver (STS_SUNLinSol_PCG or STS_SUNLinSol_SPGMR), as ARKodeSetLinearSolver +
 * ARKodeSetPreconditioner attach one (main.cpp:302-316): the driver sets the solver's ATimes
 * to v - gamma h A v (STS_JacTimes) and, when `precond` is 1, its PSolve to the Jacobi
 * STS_PSolve (used when the solver was created with STS_PREC_RIGHT). The solver's own
 * callbacks are replaced. Returns 0, or -1 on illegal input or a failed solve (rc < 0). */
int STS_SDIRK2EvolveLS(STS_Problem p, void* LS, int precond, N_Vector y, double t0, double h,
                       int nsteps, double tol, long long* total_iters);
/* One shifted system (I - gamma A) x = b with a generic solver object (PCG, SPGMR or SPFGMR):
 * the driver sets ATimes to the shifted operator and the preconditioner to none (prec 0), the
 * Jacobi STS_PSolve (1) or the caller's (2: P_data + psolve, e.g. STS_PFMGPrecSolve or
 * STS_NetPrecSolve after their PSetup); a preconditioner needs a solver made with
 * STS_PREC_RIGHT. Returns the solver's code (0 converged, 1 not converged) or -1. */
int STS_ImplicitSolveLS(STS_Problem p, double gamma, void* LS, int prec, void* P_data,
                        STS_PSolveFn psolve, N_Vector b, N_Vector x, double tol, int* iters,
                        double* relres);
/* SDIRK2 with each stage solved by STS_ImplicitSolveLearned (declared below); STS_Net is the
 * learned preconditioner's handle */
typedef struct STS_Net_* STS_Net;
int STS_SDIRK2EvolveLearned(STS_Problem p, STS_Net net, N_Vector y, double t0, double h, int nsteps,
                            double tol, int maxit, long long* total_iters);

/* ------------------------------------------------------------------------------------
 * Structured multigrid preconditioner in the role of hypre PFMG
 * (diffusion_2D/preconditioner_hypre.cpp; --pfmg_relax, --pfmg_nrelax of
 * diffusion_2D.cpp:138-150): one V-cycle per PSolve, semicoarsening in the direction of the
 * stronger coupling, non-Galerkin coarse operators, weighted Jacobi (relax_type 1),
 * symmetric red/black Gauss-Seidel (2, the reference's default) or nonsymmetric red/black
 * Gauss-Seidel (3, red then black before and after: not symmetric, so a preconditioner for
 * GMRES or flexible methods; runtests-diffusion2d.py:60,62 pass it) with nrelax pre and post
 * sweeps. Dirichlet problems (constant couplings, coarse coupling a/4) and the periodic problem
 * (per-face couplings, including k (1 + 0.99 sin); coarse faces two fine faces in series,
 * 0.5 a1 a2 / (a1 + a2); an odd direction is not coarsened).
 * ----------------------------------------------------------------------------------*/
typedef struct STS_PFMG_* STS_PFMG;
STS_PFMG STS_PFMGCreate(STS_Problem p, int relax_type, int nrelax);
void STS_PFMGFree(STS_PFMG* mg);
/* PSetup / PSolve (preconditioner_hypre.cpp:13-180), user_data = the STS_PFMG */
int STS_PFMGPSetup(double t, N_Vector u, N_Vector f, int jok, int* jcurPtr, double gamma,
                   void* user_data);
int STS_PFMGPSolve(double t, N_Vector u, N_Vector f, N_Vector r, N_Vector z, double gamma,
                   double delta, int lr, void* user_data);
/* the SUNLinSol PSolve callback form, for a PFMG set up with STS_PFMGPSetup */
int STS_PFMGPrecSolve(void* P_data, N_Vector r, N_Vector z, double tol, int lr);
int STS_PFMGNumLevels(STS_PFMG mg);
long long STS_PFMGNumVCycles(STS_PFMG mg);
/* (I - gamma A) x = b by CG (SUNLinSol_PCG through the callbacks) with the PFMG
 * preconditioner, x0 = 0, stop at ||r||_2 <= tol ||b||_2; returns as STS_SUNLinSolSolve */
int STS_ImplicitSolvePFMG(STS_Problem p, double gamma, STS_PFMG mg, N_Vector b, N_Vector x,
                          double tol, int maxit, int* iters, double* relres);
/* fixed-step SDIRK2 with each stage solved by CG + PFMG (the DIRK runs of a hypre build) */
int STS_SDIRK2EvolvePFMG(STS_Problem p, STS_PFMG mg, N_Vector y, double t0, double h, int nsteps,
                         double tol, int maxit, long long* total_iters);

/* ------------------------------------------------------------------------------------
 * Batched STS (new; the reference integrates one problem per run): many independent
 * homogeneous-Dirichlet unforced heat problems, each with its own n x n grid and kx, ky,
 * integrated from t = 0 to tf in one persistent launch with per-instance step control on
 * the device (same method, controller and step rules as the single-problem integrator).
 * States are concatenated in instance order, each row-major n x n.
 * ----------------------------------------------------------------------------------*/
typedef struct STS_Batch_* STS_Batch;
STS_Batch STS_BatchCreate(STS_Context ctx, int ninst, const int* n, const double* kx,
                          const double* ky);
int STS_BatchFree(STS_Batch* b);
long long STS_BatchTotalDOF(STS_Batch b);
int STS_BatchSetState(STS_Batch b, const double* host_y);
int STS_BatchGetState(STS_Batch b, double* host_y);
/* nmodes sine modes per instance: arrays of ninst*nmodes (p, q integers, a amplitudes) */
int STS_BatchSetInitialModes(STS_Batch b, int nmodes, const int* p, const int* q,
                             const double* a);
int STS_BatchEvolve(STS_Batch b, double tf, int method, double rtol, double atol, int smax,
                    int controller, long long maxsteps);
double STS_BatchLastMilliseconds(STS_Batch b);
int STS_BatchGetInstanceStats(STS_Batch b, int inst, STS_Stats* stats);
/* launch shape: threads per CTA (256 or 512) and CTAs per SM */
int STS_BatchSetLaunch(STS_Batch b, int threads, int ctas_per_sm);
/* mixed = 1: stages as FP32 increments relative to the FP64 step start (the single-problem
 * integrator's mixed form: FP32 copy of F_n, FP64 step update, error estimate and exact WRMS);
 * 0 (default): FP64 stages */
int STS_BatchSetMixed(STS_Batch b, int mixed);
/* autotuner: time every launch shape on the probe horizon [0, tf_probe], keep the fastest */
int STS_BatchAutotune(STS_Batch b, double tf_probe, int method, double rtol, double atol,
                      int smax, int* threads, int* ctas_per_sm, double* ms_best);
/* instances with n >= big_n are integrated by thread-block clusters of `cluster` CTAs (1, 2,
 * 4, 8, or 16 where the device schedules that non-portable size; rows split between the
 * CTAs, cluster barriers between sweeps, the exact reductions combined through distributed
 * shared memory), concurrently with the single-CTA group */
int STS_BatchSetCluster(STS_Batch b, int cluster, int big_n);
int STS_BatchGetLaunch(STS_Batch b, int* threads, int* ctas_per_sm, int* cluster, int* big_n);

/* ------------------------------------------------------------------------------------
 * Learned multilevel preconditioner (new; the reference's multilevel alternative to Jacobi
 * is hypre PFMG, diffusion_2D/preconditioner_hypre.cpp). z = D (r + E^T E r): D the Jacobi
 * diagonal, E a 4-level linear convolutional encoder (16 channels, 3x3 kernels, 2x2 mean
 * pooling, BF16 weights, FP32 accumulation, tensor-core implicit GEMM) on the input channels
 * [r, r sk, r sg] (sk = normalised log10(ky/kx), sg = normalised log10(gamma/dx^2)), E^T its
 * exact adjoint: an SPD additive multilevel preconditioner with learned level operators.
 * Sizes: multiples of 16.
 * ----------------------------------------------------------------------------------*/
STS_Net STS_NetCreate(STS_Context ctx, int nmax, unsigned long long seed);
int STS_NetFree(STS_Net* net);
/* weights: 4 layers (W_in, W_1, W_2, W_3) x [16][16][3][3] FP32 (W_in: 3 input channels) */
int STS_NetSetWeights(STS_Net net, const float* w);
int STS_NetGetWeights(STS_Net net, float* w);
/* z = jacobi * (r + E^T E (scale r) / scale) on device arrays of n x n doubles */
/* inference convolutions: 0 = the row-marching mma.sync kernels the training uses (default,
 * the faster of the two at 2048^2), 1 = tcgen05 tensor cores with TMEM accumulators, 1-D TMA
 * bulk loads and stores; both compute the same network */
int STS_NetSetTensorPath(STS_Net net, int path);
/* inference level 0 collapsed (default 1): p0 as a stride-2 4x4 convolution of the input and
 * z from a 5x5 convolution of the input plus a coarse-parity convolution of y1, with the
 * system features folded into the weights, so no 16-channel fine-level tensor is formed;
 * 0 = the layer-by-layer kernels. The same network either way. */
int STS_NetSetCollapsedLevel0(STS_Net net, int on);
int STS_NetApply(STS_Net net, int n, const double* r, double* z, double sk, double sg, double jacobi,
                 double scale);
/* one sample (scale 1): loss = 0.5 (z - e)^T M (z - e) / (e^T M e) with M = I - gamma A on the
 * n x n field (zero outside; gcx = gamma kx/dx^2, gcy = gamma ky/dy^2) and its weight
 * gradient (host FP32 array); z = jacobi (r + E^T E r) */
int STS_NetLossGrad(STS_Net net, int n, const double* r, const float* e, double sk, double sg,
                    double jacobi, double gcx, double gcy, double* loss, float* grad);
/* Adam over device samples r, e (nsamples x n x n FP32) with per-sample
 * meta = {sk, sg, jacobi, scale, 1/(e^T M e), gcx, gcy} (7 floats, as STS_HarvestPCGPairs
 * writes it), minibatches of `batch` samples run batched */
int STS_NetTrain(STS_Net net, int n, int nsamples, const float* r, const float* e, const float* meta,
                 int epochs, int batch, float lr, unsigned long long seed, double* last_loss);
/* residual/correction pairs from a converged fused Jacobi-PCG solve of (I - gamma A) x = b:
 * after every `every`-th batch of 8 iterations, `ncrops` crops (crop x crop, seeded fixed
 * positions) of r_k and of e_k = x* - x_k are appended to r_out / e_out (device FP32,
 * capacity max_pairs), and their training metadata (7 floats each) to meta_out (device,
 * may be NULL) */
int STS_HarvestPCGPairs(STS_Problem p, double gamma, N_Vector b, int ncrops, int crop, int every,
                        int max_pairs, float* r_out, float* e_out, float* meta_out,
                        unsigned long long seed, int* npairs, int* iters);
/* flexible CG with the network as preconditioner, x0 = 0, stop at ||r|| <= tol ||b||; on
 * stagnation (maxit) or breakdown it falls back to Jacobi-PCG on the remaining correction.
 * Returns 0 converged, 2 converged through the fallback, 1 not converged, < 0 error; iters
 * counts FCG plus fallback iterations; relres is the true FP64 residual of the returned x.
 * maxit < 0 runs at most -maxit FCG iterations without the fallback. */
int STS_FCGSolve(STS_Problem p, double gamma, STS_Net net, N_Vector b, N_Vector x, double tol,
                 int maxit, int* iters, double* relres);
/* Learned-or-Jacobi shifted solve: FCG with the network when kappa = 1 + 4 gamma (cx + cy)
 * >= kappa_min (<= 0: 1500, the measured break-even of the network's per-iteration cost on
 * GB300), otherwise the fused Jacobi-PCG; used_net reports the choice. Same return codes. */
int STS_ImplicitSolveLearned(STS_Problem p, double gamma, STS_Net net, N_Vector b, N_Vector x,
                             double tol, int maxit, double kappa_min, int* iters, double* relres,
                             int* used_net);
/* The network as a preconditioner object with the reference's PSetup / PSolve signatures
 * (diffusion_2D/preconditioner_jacobi.cpp:9-10,49-50) for the generic solvers: PSetup takes
 * gamma and folds the system features (ky/kx, gamma/dx^2) into the level-0 weights; PSolve
 * applies z = M r (input scaled by 1/rms(r)); STS_NetPrecSolve is the SUNLinSol PSolve form.
 * Square Dirichlet grids with n a multiple of 16, on the network's context. Use with
 * STS_SUNLinSol_SPFGMR (the BF16 network is linear only up to rounding). */
typedef struct STS_NetPrec_* STS_NetPrec;
int STS_NetPrecCreate(STS_Net net, STS_Problem p, STS_NetPrec* P);
int STS_NetPrecFree(STS_NetPrec* P);
int STS_NetPSetup(double t, N_Vector u, N_Vector f, int jok, int* jcurPtr, double gamma,
                  void* user_data);
int STS_NetPSolve(double t, N_Vector u, N_Vector f, N_Vector r, N_Vector z, double gamma,
                  double delta, int lr, void* user_data);
int STS_NetPrecSolve(void* P_data, N_Vector r, N_Vector z, double tol, int lr);

#ifdef __cplusplus
}
#endif
#endif
