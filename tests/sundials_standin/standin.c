/* Stand-ins for the two SUNDIALS constructors the vector shim calls (N_VNewEmpty allocates a
 * vector and a zeroed operations table, N_VFreeEmpty frees both), and a driver that wraps a
 * vector and checks every operation the shim forwards is in place. No device work: the
 * wrapped inner vector is never touched. TEST INFRASTRUCTURE ONLY. */
#include <stdio.h>
#include <stdlib.h>

#include <sundials/sundials_nvector.h>

N_Vector N_VNewEmpty(SUNContext sunctx)
{
  N_Vector v = (N_Vector)calloc(1, sizeof(*v));
  if (!v) return NULL;
  v->ops    = (N_Vector_Ops)calloc(1, sizeof(*v->ops));
  v->sunctx = sunctx;
  return v;
}

void N_VFreeEmpty(N_Vector v)
{
  if (!v) return;
  free(v->ops);
  free(v);
}

N_Vector sts_sundials_wrap(void* inner, SUNContext sctx);
int sts_sundials_diffusion(sunrealtype t, N_Vector u, N_Vector f, void* ud);

int main(void)
{
  int fake    = 0;
  N_Vector v  = sts_sundials_wrap(&fake, NULL);
  int missing = 0;
  void* ops[] = {(void*)v->ops->nvclone,    (void*)v->ops->nvdestroy,  (void*)v->ops->nvlinearsum,
                 (void*)v->ops->nvconst,    (void*)v->ops->nvprod,     (void*)v->ops->nvdiv,
                 (void*)v->ops->nvscale,    (void*)v->ops->nvabs,      (void*)v->ops->nvinv,
                 (void*)v->ops->nvaddconst, (void*)v->ops->nvdotprod,  (void*)v->ops->nvmaxnorm,
                 (void*)v->ops->nvwrmsnorm, (void*)v->ops->nvspace,    (void*)v->ops->nvgetlength,
                 (void*)v->ops->nvlinearcombination, (void*)v->ops->nvdotprodmulti,
                 (void*)v->ops->nvgetdevicearraypointer};
  for (size_t k = 0; k < sizeof(ops) / sizeof(ops[0]); ++k) missing += ops[k] == NULL;
  if (v->content != &fake) missing++;
  v->content = NULL;
  N_VFreeEmpty(v);
  printf("%s\n", missing ? "missing ops" : "ok");
  return missing ? 1 : 0;
}
