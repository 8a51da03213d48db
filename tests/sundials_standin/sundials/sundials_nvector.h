/* Stand-in for SUNDIALS' public <sundials/sundials_nvector.h> (v7), for compiling the
 * library's SUNDIALS vector shim in a CPU test where SUNDIALS is absent (the reference's
 * deps/sundials submodule is empty). TEST INFRASTRUCTURE ONLY.
 *
 * It declares the generic vector { content, ops, sunctx }, an operations table with the
 * public member names of SUNDIALS' _generic_N_Vector_Ops (the ones the shim assigns and the
 * rest of the standard set), sunrealtype / sunindextype (32-bit, the reference's
 * SUNDIALS_INDEX_SIZE=32 build, README.md:147) and N_VNewEmpty / N_VFreeEmpty. The shim
 * touches the table only by member name, so the order of the members here is not a claim
 * about SUNDIALS' binary layout. */
#ifndef STS_STANDIN_SUNDIALS_NVECTOR_H
#define STS_STANDIN_SUNDIALS_NVECTOR_H
#include <stdint.h>

typedef double sunrealtype;
typedef int32_t sunindextype;
typedef int sunbooleantype;
typedef struct SUNContext_* SUNContext;
typedef int N_Vector_ID;

typedef struct _generic_N_Vector_Ops* N_Vector_Ops;
typedef struct _generic_N_Vector* N_Vector;

struct _generic_N_Vector_Ops {
  N_Vector_ID (*nvgetvectorid)(N_Vector);
  N_Vector (*nvclone)(N_Vector);
  N_Vector (*nvcloneempty)(N_Vector);
  void (*nvdestroy)(N_Vector);
  void (*nvspace)(N_Vector, sunindextype*, sunindextype*);
  sunrealtype* (*nvgetarraypointer)(N_Vector);
  sunrealtype* (*nvgetdevicearraypointer)(N_Vector);
  void (*nvsetarraypointer)(sunrealtype*, N_Vector);
  void* (*nvgetcommunicator)(N_Vector);
  sunindextype (*nvgetlength)(N_Vector);
  sunindextype (*nvgetlocallength)(N_Vector);
  void (*nvlinearsum)(sunrealtype, N_Vector, sunrealtype, N_Vector, N_Vector);
  void (*nvconst)(sunrealtype, N_Vector);
  void (*nvprod)(N_Vector, N_Vector, N_Vector);
  void (*nvdiv)(N_Vector, N_Vector, N_Vector);
  void (*nvscale)(sunrealtype, N_Vector, N_Vector);
  void (*nvabs)(N_Vector, N_Vector);
  void (*nvinv)(N_Vector, N_Vector);
  void (*nvaddconst)(N_Vector, sunrealtype, N_Vector);
  sunrealtype (*nvdotprod)(N_Vector, N_Vector);
  sunrealtype (*nvmaxnorm)(N_Vector);
  sunrealtype (*nvwrmsnorm)(N_Vector, N_Vector);
  sunrealtype (*nvwrmsnormmask)(N_Vector, N_Vector, N_Vector);
  sunrealtype (*nvmin)(N_Vector);
  sunrealtype (*nvwl2norm)(N_Vector, N_Vector);
  sunrealtype (*nvl1norm)(N_Vector);
  void (*nvcompare)(sunrealtype, N_Vector, N_Vector);
  sunbooleantype (*nvinvtest)(N_Vector, N_Vector);
  sunbooleantype (*nvconstrmask)(N_Vector, N_Vector, N_Vector);
  sunrealtype (*nvminquotient)(N_Vector, N_Vector);
  int (*nvlinearcombination)(int, sunrealtype*, N_Vector*, N_Vector);
  int (*nvscaleaddmulti)(int, sunrealtype*, N_Vector, N_Vector*, N_Vector*);
  int (*nvdotprodmulti)(int, N_Vector, N_Vector*, sunrealtype*);
};

struct _generic_N_Vector {
  void* content;
  N_Vector_Ops ops;
  SUNContext sunctx;
};

N_Vector N_VNewEmpty(SUNContext sunctx);
void N_VFreeEmpty(N_Vector v);

#endif
