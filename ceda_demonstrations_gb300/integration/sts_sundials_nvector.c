/* SUNDIALS N_Vector over libstsgpu's device vector: the forwarding shim a real SUNDIALS build
 * of the reference uses to drive this library's vector with its own integrators
 * (LSRKStepCreateSTS, ARKStepCreate, SUNLinSol_PCG: diffusion_2D/main.cpp:176-257). The
 * SUNDIALS vector's content is this library's N_Vector; each op forwards to the C ABI, as
 * gkeyll_diffusion/src/nvector_gkylzero.c:32-82 forwards to gkylzero arrays.
 *
 * Build against SUNDIALS' headers and link with -lstsgpu:
 *   cc -c sts_sundials_nvector.c -I<sundials>/include -I<repo>/include
 *
 * Index widths: libstsgpu's sts_index is 64-bit; SUNDIALS' sunindextype is 32-bit in the
 * reference's build (SUNDIALS_INDEX_SIZE=32, README.md:147). Lengths pass from the narrower to
 * the wider type; a vector longer than 2^31 - 1 cannot exist in a 32-bit SUNDIALS build, and
 * sts_nvspace clamps nothing because it never sees one. */
#include <stdlib.h>

#include <sundials/sundials_nvector.h>

/* the library's own vector type; its struct lives in stsgpu.h with the same member names as
 * SUNDIALS', so it is kept under another name here */
#define N_Vector STS_N_Vector
#define _generic_N_Vector _sts_generic_N_Vector
#define _generic_N_Vector_Ops _sts_generic_N_Vector_Ops
#define N_Vector_Ops STS_N_Vector_Ops
#include "stsgpu.h"
#undef N_Vector
#undef _generic_N_Vector
#undef _generic_N_Vector_Ops
#undef N_Vector_Ops

#define STS(v) ((STS_N_Vector)((v)->content))

N_Vector sts_sundials_wrap(STS_N_Vector inner, SUNContext sctx);

static N_Vector sh_clone(N_Vector w) { return sts_sundials_wrap(N_VClone_Sts(STS(w)), w->sunctx); }
static void sh_destroy(N_Vector v)
{
  if (!v) return;
  if (v->content) N_VDestroy_Sts(STS(v));
  v->content = NULL;
  N_VFreeEmpty(v);
}
static void sh_space(N_Vector v, sunindextype* lrw, sunindextype* liw)
{
  sts_index r = 0, i = 0;
  N_VSpace_Sts(STS(v), &r, &i);
  *lrw = (sunindextype)r;
  *liw = (sunindextype)i;
}
static sunrealtype* sh_devptr(N_Vector v) { return (sunrealtype*)N_VGetDeviceArrayPointer_Sts(STS(v)); }
static sunindextype sh_length(N_Vector v) { return (sunindextype)N_VGetLength_Sts(STS(v)); }
static void sh_linearsum(sunrealtype a, N_Vector x, sunrealtype b, N_Vector y, N_Vector z)
{
  N_VLinearSum_Sts(a, STS(x), b, STS(y), STS(z));
}
static void sh_const(sunrealtype c, N_Vector z) { N_VConst_Sts(c, STS(z)); }
static void sh_prod(N_Vector x, N_Vector y, N_Vector z) { N_VProd_Sts(STS(x), STS(y), STS(z)); }
static void sh_div(N_Vector x, N_Vector y, N_Vector z) { N_VDiv_Sts(STS(x), STS(y), STS(z)); }
static void sh_scale(sunrealtype c, N_Vector x, N_Vector z) { N_VScale_Sts(c, STS(x), STS(z)); }
static void sh_abs(N_Vector x, N_Vector z) { N_VAbs_Sts(STS(x), STS(z)); }
static void sh_inv(N_Vector x, N_Vector z) { N_VInv_Sts(STS(x), STS(z)); }
static void sh_addconst(N_Vector x, sunrealtype b, N_Vector z) { N_VAddConst_Sts(STS(x), b, STS(z)); }
static sunrealtype sh_dot(N_Vector x, N_Vector y) { return N_VDotProd_Sts(STS(x), STS(y)); }
static sunrealtype sh_maxnorm(N_Vector x) { return N_VMaxNorm_Sts(STS(x)); }
static sunrealtype sh_wrms(N_Vector x, N_Vector w) { return N_VWrmsNorm_Sts(STS(x), STS(w)); }
static int sh_lincomb(int nvec, sunrealtype* c, N_Vector* X, N_Vector z)
{
  STS_N_Vector Xs[64];
  if (nvec < 1 || nvec > 64) return -1;
  for (int k = 0; k < nvec; ++k) Xs[k] = STS(X[k]);
  return N_VLinearCombination_Sts(nvec, c, Xs, STS(z));
}
static int sh_dotmulti(int nvec, N_Vector x, N_Vector* Y, sunrealtype* d)
{
  STS_N_Vector Ys[64];
  if (nvec < 1 || nvec > 64) return -1;
  for (int k = 0; k < nvec; ++k) Ys[k] = STS(Y[k]);
  return N_VDotProdMulti_Sts(nvec, STS(x), Ys, d);
}

N_Vector sts_sundials_wrap(STS_N_Vector inner, SUNContext sctx)
{
  if (!inner) return NULL;
  N_Vector v = N_VNewEmpty(sctx);
  if (!v) return NULL;
  v->content                       = inner;
  v->ops->nvclone                  = sh_clone;
  v->ops->nvdestroy                = sh_destroy;
  v->ops->nvspace                  = sh_space;
  v->ops->nvgetdevicearraypointer  = sh_devptr;
  v->ops->nvgetlength              = sh_length;
  v->ops->nvgetlocallength         = sh_length;
  v->ops->nvlinearsum              = sh_linearsum;
  v->ops->nvconst                  = sh_const;
  v->ops->nvprod                   = sh_prod;
  v->ops->nvdiv                    = sh_div;
  v->ops->nvscale                  = sh_scale;
  v->ops->nvabs                    = sh_abs;
  v->ops->nvinv                    = sh_inv;
  v->ops->nvaddconst               = sh_addconst;
  v->ops->nvdotprod                = sh_dot;
  v->ops->nvmaxnorm                = sh_maxnorm;
  v->ops->nvwrmsnorm               = sh_wrms;
  v->ops->nvlinearcombination      = sh_lincomb;
  v->ops->nvdotprodmulti           = sh_dotmulti;
  return v;
}

/* the reference's ARKRhsFn / PSetup / PSolve over the wrapped vectors; user_data carries the
 * STS_Problem (diffusion_2D.cpp:23-35, preconditioner_jacobi.cpp:9-61) */
int sts_sundials_diffusion(sunrealtype t, N_Vector u, N_Vector f, void* ud)
{
  return STS_Diffusion(t, STS(u), STS(f), ud);
}
int sts_sundials_psetup(sunrealtype t, N_Vector u, N_Vector f, sunbooleantype jok, sunbooleantype* jcur,
                        sunrealtype gamma, void* ud)
{
  int j  = 0;
  int rc = STS_PSetup(t, u ? STS(u) : NULL, f ? STS(f) : NULL, jok, &j, gamma, ud);
  if (jcur) *jcur = j;
  return rc;
}
int sts_sundials_psolve(sunrealtype t, N_Vector u, N_Vector f, N_Vector r, N_Vector z, sunrealtype gamma,
                        sunrealtype delta, int lr, void* ud)
{
  return STS_PSolve(t, u ? STS(u) : NULL, f ? STS(f) : NULL, STS(r), STS(z), gamma, delta, lr, ud);
}
