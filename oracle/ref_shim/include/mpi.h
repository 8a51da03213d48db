/* Single-rank stand-in for the MPI calls of diffusion_2D/diffusion_2D.cpp (TEST
 * INFRASTRUCTURE ONLY). One process, a 1 x 1 periodic Cartesian grid: every neighbour of
 * rank 0 is rank 0, so the halo exchange of UserData::start_exchange / end_exchange
 * (diffusion_2D.cpp:400-584) becomes the periodic wrap of the local field: a send is copied
 * into the posted receive with the same tag. */
#ifndef REF_SHIM_MPI_H
#define REF_SHIM_MPI_H

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef struct {
  int tag;
} MPI_Request;
typedef struct {
  int status;
} MPI_Status;

#define MPI_SUCCESS 0
#define MPI_COMM_NULL 0
#define MPI_COMM_WORLD 1
#define MPI_DOUBLE 1

int MPI_Comm_size(MPI_Comm comm, int* size);
int MPI_Comm_rank(MPI_Comm comm, int* rank);
int MPI_Dims_create(int nnodes, int ndims, int* dims);
int MPI_Cart_create(MPI_Comm comm, int ndims, const int* dims, const int* periods, int reorder, MPI_Comm* cart);
int MPI_Cart_get(MPI_Comm comm, int maxdims, int* dims, int* periods, int* coords);
int MPI_Cart_rank(MPI_Comm comm, const int* coords, int* rank);
int MPI_Irecv(void* buf, int count, MPI_Datatype type, int source, int tag, MPI_Comm comm, MPI_Request* req);
int MPI_Isend(const void* buf, int count, MPI_Datatype type, int dest, int tag, MPI_Comm comm, MPI_Request* req);
int MPI_Wait(MPI_Request* req, MPI_Status* status);

#endif
