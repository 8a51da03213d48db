/* Minimal stand-in for the SUNDIALS headers the reference's diffusion_2D sources include,
 * so that those sources compile unmodified into oracle/_ref (TEST INFRASTRUCTURE ONLY).
 *
 * It declares only what diffusion_2D/{diffusion_2D,diffusion,initial,buffers,
 * preconditioner_jacobi}.cpp use: the scalar and index types, SUN_RCONST, the profiler
 * marker, and a serial N_Vector with N_VGetArrayPointer / N_VConst / N_VProd / N_VDotProd /
 * N_VDestroy (semantics of SUNDIALS' serial vector). sunindextype is 32-bit, as in the
 * reference's SUNDIALS build (SUNDIALS_INDEX_SIZE=32, README.md:147). */
#ifndef REF_SHIM_SUNDIALS_CORE_HPP
#define REF_SHIM_SUNDIALS_CORE_HPP
#include <cstdint>

typedef double sunrealtype;
typedef int32_t sunindextype;
typedef int sunbooleantype;
#define SUN_RCONST(x) (x)
#define SUNTRUE 1
#define SUNFALSE 0

typedef void* SUNProfiler;
typedef void* SUNContext;
#define SUNDIALS_CXX_MARK_FUNCTION(prof) ((void)(prof))

/* sundials_mpi_types.h: the MPI datatype of sunrealtype */
#define MPI_SUNREALTYPE MPI_DOUBLE

struct RefShimVector {
  sunrealtype* data;
  sunindextype length;
  int own_data;
};
typedef RefShimVector* N_Vector;

sunrealtype* N_VGetArrayPointer(N_Vector v);
void N_VConst(sunrealtype c, N_Vector z);
void N_VProd(N_Vector x, N_Vector y, N_Vector z);
sunrealtype N_VDotProd(N_Vector x, N_Vector y);
void N_VDestroy(N_Vector v);

#endif
