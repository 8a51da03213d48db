// Driver around the reference's own diffusion_2D sources, compiled unmodified into
// oracle/_ref/libdiffusion_ref.so by oracle/Makefile (target `ref`). TEST INFRASTRUCTURE
// ONLY: it lets the CPU tests compare the oracle's restatement (oracle/sts_oracle.c) with
// the reference's code on the reference's own periodic problem.
//
// Compiled from the reference: diffusion_2D/diffusion_2D.cpp (UserData::parse_args, setup,
// start_exchange / end_exchange, Diffusion_Coeff_X/Y, check_flag, diffusion), diffusion.cpp
// (laplacian), initial.cpp (Initial), buffers.cpp (halo buffers), preconditioner_jacobi.cpp
// (PSetup / PSolve). This file supplies what those sources take from SUNDIALS and MPI: a
// serial N_Vector (sundials_core.hpp in ref_shim/include) and a single-rank MPI whose
// periodic 1 x 1 Cartesian grid makes every neighbour rank 0 (ref_shim/include/mpi.h).
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "diffusion_2D.hpp"

// ---------------------------------------------------------------- serial N_Vector
sunrealtype* N_VGetArrayPointer(N_Vector v) { return v ? v->data : nullptr; }

void N_VConst(sunrealtype c, N_Vector z)
{
  for (sunindextype i = 0; i < z->length; ++i) z->data[i] = c;
}

void N_VProd(N_Vector x, N_Vector y, N_Vector z)
{
  for (sunindextype i = 0; i < z->length; ++i) z->data[i] = x->data[i] * y->data[i];
}

sunrealtype N_VDotProd(N_Vector x, N_Vector y)
{
  sunrealtype s = 0.0;
  for (sunindextype i = 0; i < x->length; ++i) s += x->data[i] * y->data[i];
  return s;
}

void N_VDestroy(N_Vector v)
{
  if (!v) return;
  if (v->own_data) delete[] v->data;
  delete v;
}

static N_Vector wrap(double* data, sunindextype n)
{
  return new RefShimVector{data, n, 0};
}

// ---------------------------------------------------------------- single-rank MPI
namespace {
struct Posted {
  void* buf;
  int count;
  int tag;
};
std::vector<Posted> g_posted; // receives waiting for the matching send
int g_mpi_errors = 0;
} // namespace

int MPI_Comm_size(MPI_Comm, int* size)
{
  *size = 1;
  return MPI_SUCCESS;
}
int MPI_Comm_rank(MPI_Comm, int* rank)
{
  *rank = 0;
  return MPI_SUCCESS;
}
int MPI_Dims_create(int, int ndims, int* dims)
{
  for (int d = 0; d < ndims; ++d)
    if (dims[d] <= 0) dims[d] = 1;
  return MPI_SUCCESS;
}
int MPI_Cart_create(MPI_Comm, int, const int*, const int*, int, MPI_Comm* cart)
{
  *cart = 2;
  return MPI_SUCCESS;
}
int MPI_Cart_get(MPI_Comm, int maxdims, int* dims, int* periods, int* coords)
{
  for (int d = 0; d < maxdims; ++d)
  {
    dims[d]    = 1;
    periods[d] = 1;
    coords[d]  = 0;
  }
  return MPI_SUCCESS;
}
int MPI_Cart_rank(MPI_Comm, const int*, int* rank)
{
  *rank = 0; // periodic 1 x 1 grid: every coordinate wraps to rank 0
  return MPI_SUCCESS;
}
int MPI_Irecv(void* buf, int count, MPI_Datatype, int, int tag, MPI_Comm, MPI_Request* req)
{
  g_posted.push_back({buf, count, tag});
  req->tag = tag;
  return MPI_SUCCESS;
}
int MPI_Isend(const void* buf, int count, MPI_Datatype, int, int tag, MPI_Comm, MPI_Request* req)
{
  req->tag = tag;
  for (size_t k = 0; k < g_posted.size(); ++k)
    if (g_posted[k].tag == tag && g_posted[k].count == count)
    {
      std::memcpy(g_posted[k].buf, buf, sizeof(double) * (size_t)count);
      g_posted.erase(g_posted.begin() + (long)k);
      return MPI_SUCCESS;
    }
  ++g_mpi_errors; // a send with no posted receive: the exchange pattern changed
  return 1;
}
int MPI_Wait(MPI_Request*, MPI_Status*) { return MPI_SUCCESS; }

// ---------------------------------------------------------------- C API for the tests
extern "C" {

// UserData of the reference for an nx x ny periodic problem on the default domain
// [-pi, pi] x [-6, 6], set up by the reference's own parse_args (dx = (xu-xl)/(nx-1)) and
// setup (single rank). kx, ky are passed as 17-digit decimals, which round-trip exactly.
void* ref_create(int nx, int ny, double kx, double ky, int inhomogeneous)
{
  char b[64];
  std::vector<std::string> args;
  args.push_back("--nx");
  args.push_back(std::to_string(nx));
  args.push_back("--ny");
  args.push_back(std::to_string(ny));
  std::snprintf(b, sizeof b, "%.17g", kx);
  args.push_back("--kx");
  args.push_back(b);
  std::snprintf(b, sizeof b, "%.17g", ky);
  args.push_back("--ky");
  args.push_back(b);
  if (inhomogeneous) args.push_back("--inhomogeneous");
  UserData* ud = new UserData(nullptr);
  if (ud->parse_args(args, false) != 0 || ud->setup() != 0)
  {
    delete ud;
    return nullptr;
  }
  return ud;
}

void ref_free(void* ud) { delete (UserData*)ud; }

void ref_grid(void* p, double* dx, double* dy, double* xl, double* yl)
{
  UserData* ud = (UserData*)p;
  *dx          = ud->dx;
  *dy          = ud->dy;
  *xl          = ud->xl;
  *yl          = ud->yl;
}

// the ARKRhsFn diffusion (diffusion_2D.cpp:23-35 -> laplacian, diffusion.cpp:9-209)
int ref_rhs(void* p, double t, double* u, double* f)
{
  UserData* ud = (UserData*)p;
  N_Vector U = wrap(u, ud->nodes_loc), F = wrap(f, ud->nodes_loc);
  g_mpi_errors = 0;
  int rc       = diffusion(t, U, F, ud);
  N_VDestroy(U);
  N_VDestroy(F);
  return (rc != 0 || g_mpi_errors || !g_posted.empty()) ? -1 : 0;
}

// Initial (initial.cpp:20-47)
int ref_initial(void* p, double* u)
{
  UserData* ud = (UserData*)p;
  N_Vector U   = wrap(u, ud->nodes_loc);
  int rc       = Initial(0.0, U, ud);
  N_VDestroy(U);
  return rc;
}

// PSetup (preconditioner_jacobi.cpp:9-43) into `diag`, then PSolve z = diag * r (:49-61)
int ref_jacobi(void* p, double gamma, double* diag, double* r, double* z)
{
  UserData* ud = (UserData*)p;
  ud->diag     = wrap(diag, ud->nodes_loc);
  sunbooleantype jcur = 0;
  int rc              = PSetup(0.0, nullptr, nullptr, 0, &jcur, gamma, ud);
  if (rc == 0)
  {
    N_Vector R = wrap(r, ud->nodes_loc), Z = wrap(z, ud->nodes_loc);
    rc         = PSolve(0.0, nullptr, nullptr, R, Z, gamma, 0.0, 2, ud);
    N_VDestroy(R);
    N_VDestroy(Z);
  }
  N_VDestroy(ud->diag);
  ud->diag = nullptr;
  return rc;
}

// Diffusion_Coeff_X / _Y (diffusion_2D.cpp:887-897)
double ref_coeff_x(void* p, double x) { return Diffusion_Coeff_X(x, (UserData*)p); }
double ref_coeff_y(void* p, double y) { return Diffusion_Coeff_Y(y, (UserData*)p); }
}
