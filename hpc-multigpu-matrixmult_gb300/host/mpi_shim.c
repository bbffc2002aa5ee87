/*
 * Single-rank implementation of the MPI calls used by the SUMMA layer and the
 * driver (see include/mpi_shim/mpi.h). Each call checks its arguments the way
 * a one-process MPI job would see them: rank arguments must be 0, the only
 * valid root is 0, point-to-point calls have no peer and fail.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "mpi.h"

#define SHIM_MAX_COMMS 64
#define SHIM_MAX_TYPES 64

static int g_initialized;
static int g_next_comm = 2;
static int g_comm_live[SHIM_MAX_COMMS] = {0, 1};
static int g_comm_ndims[SHIM_MAX_COMMS];

/* Derived vector types: count blocks of blocklength elements, stride apart. */
static struct {
  int live, count, blocklength, stride, base_size;
} g_types[SHIM_MAX_TYPES];

static int base_size(MPI_Datatype t) {
  switch (t) {
    case MPI_FLOAT: return 4;
    case MPI_DOUBLE: return 8;
    case MPI_INT: return 4;
    default:
      if (t >= 16 && t < 16 + SHIM_MAX_TYPES && g_types[t - 16].live) return -1; /* derived */
      return 0;
  }
}

static int comm_ok(MPI_Comm c) { return c > 0 && c < SHIM_MAX_COMMS && g_comm_live[c]; }

int MPI_Init(int *argc, char ***argv) {
  (void)argc;
  (void)argv;
  g_initialized = 1;
  return MPI_SUCCESS;
}
int MPI_Finalize(void) {
  g_initialized = 0;
  return MPI_SUCCESS;
}
int MPI_Abort(MPI_Comm comm, int errorcode) {
  (void)comm;
  fflush(stdout);
  fflush(stderr);
  exit(errorcode ? errorcode : 1);
}
int MPI_Comm_size(MPI_Comm comm, int *size) {
  if (!comm_ok(comm) || !size) return MPI_ERR_COMM;
  *size = 1;
  return MPI_SUCCESS;
}
int MPI_Comm_rank(MPI_Comm comm, int *rank) {
  if (!comm_ok(comm) || !rank) return MPI_ERR_COMM;
  *rank = 0;
  return MPI_SUCCESS;
}
int MPI_Comm_free(MPI_Comm *comm) {
  if (!comm || !comm_ok(*comm) || *comm == MPI_COMM_WORLD) return MPI_ERR_COMM;
  g_comm_live[*comm] = 0;
  *comm = MPI_COMM_NULL;
  return MPI_SUCCESS;
}
int MPI_Barrier(MPI_Comm comm) { return comm_ok(comm) ? MPI_SUCCESS : MPI_ERR_COMM; }

/* Balanced factorisation of nnodes over the dimensions that are 0 on entry. */
int MPI_Dims_create(int nnodes, int ndims, int dims[]) {
  int fixed = 1, is_free[16] = {0};
  if (ndims < 1 || ndims > 16 || nnodes < 1) return MPI_ERR_ARG;
  for (int i = 0; i < ndims; ++i) {
    if (dims[i] < 0) return MPI_ERR_ARG;
    if (dims[i] > 0) fixed *= dims[i];
    else is_free[i] = 1;
  }
  if (nnodes % fixed) return MPI_ERR_ARG;
  int rest = nnodes / fixed, nfree = 0;
  for (int i = 0; i < ndims; ++i)
    if (is_free[i]) {
      dims[i] = 1;
      ++nfree;
    }
  if (!nfree) return rest == 1 ? MPI_SUCCESS : MPI_ERR_ARG;
  /* prime factors, largest first, each onto the currently smallest free dim */
  int factors[64], nf = 0;
  for (int p = rest, f = 2; p > 1;) {
    if (p % f == 0) {
      factors[nf++] = f;
      p /= f;
    } else {
      ++f;
    }
  }
  for (int j = nf - 1; j >= 0; --j) {
    int best = -1;
    for (int i = 0; i < ndims; ++i)
      if (is_free[i] && (best < 0 || dims[i] < dims[best])) best = i;
    dims[best] *= factors[j];
  }
  /* non-increasing order over the free dims, as MPI specifies */
  for (int i = 0; i < ndims; ++i)
    for (int j = i + 1; j < ndims; ++j)
      if (is_free[i] && is_free[j] && dims[j] > dims[i]) {
        int t = dims[i];
        dims[i] = dims[j];
        dims[j] = t;
      }
  return MPI_SUCCESS;
}

static int new_comm(int ndims, MPI_Comm *out) {
  if (g_next_comm >= SHIM_MAX_COMMS) {
    for (int c = 2; c < SHIM_MAX_COMMS; ++c)
      if (!g_comm_live[c]) {
        g_comm_live[c] = 1;
        g_comm_ndims[c] = ndims;
        *out = c;
        return MPI_SUCCESS;
      }
    return MPI_ERR_COMM;
  }
  g_comm_live[g_next_comm] = 1;
  g_comm_ndims[g_next_comm] = ndims;
  *out = g_next_comm++;
  return MPI_SUCCESS;
}

int MPI_Cart_create(MPI_Comm old, int ndims, const int dims[], const int periods[], int reorder, MPI_Comm *cart) {
  (void)periods;
  (void)reorder;
  if (!comm_ok(old) || ndims < 1 || !cart) return MPI_ERR_ARG;
  int n = 1;
  for (int i = 0; i < ndims; ++i) n *= dims[i];
  if (n != 1) return MPI_ERR_ARG; /* one process: every dimension must be 1 */
  return new_comm(ndims, cart);
}
int MPI_Cart_coords(MPI_Comm comm, int rank, int maxdims, int coords[]) {
  if (!comm_ok(comm) || rank != 0) return MPI_ERR_RANK;
  for (int i = 0; i < maxdims; ++i) coords[i] = 0;
  return MPI_SUCCESS;
}
int MPI_Cart_get(MPI_Comm comm, int maxdims, int dims[], int periods[], int coords[]) {
  if (!comm_ok(comm)) return MPI_ERR_COMM;
  for (int i = 0; i < maxdims; ++i) {
    dims[i] = 1;
    periods[i] = 1;
    coords[i] = 0;
  }
  return MPI_SUCCESS;
}
int MPI_Cart_sub(MPI_Comm comm, const int remain_dims[], MPI_Comm *sub) {
  if (!comm_ok(comm) || !sub) return MPI_ERR_COMM;
  int nd = 0;
  for (int i = 0; i < g_comm_ndims[comm]; ++i) nd += remain_dims[i] != 0;
  return new_comm(nd > 0 ? nd : 1, sub);
}

int MPI_Type_vector(int count, int blocklength, int stride, MPI_Datatype old, MPI_Datatype *newtype) {
  const int bs = base_size(old);
  if (count < 0 || blocklength < 0 || bs <= 0 || !newtype) return MPI_ERR_ARG;
  for (int i = 0; i < SHIM_MAX_TYPES; ++i)
    if (!g_types[i].live) {
      g_types[i].live = 1;
      g_types[i].count = count;
      g_types[i].blocklength = blocklength;
      g_types[i].stride = stride;
      g_types[i].base_size = bs;
      *newtype = 16 + i;
      return MPI_SUCCESS;
    }
  return MPI_ERR_ARG;
}
int MPI_Type_commit(MPI_Datatype *type) { return type && base_size(*type) != 0 ? MPI_SUCCESS : MPI_ERR_ARG; }
int MPI_Type_free(MPI_Datatype *type) {
  if (!type || *type < 16 || *type >= 16 + SHIM_MAX_TYPES || !g_types[*type - 16].live) return MPI_ERR_ARG;
  g_types[*type - 16].live = 0;
  *type = MPI_DATATYPE_NULL;
  return MPI_SUCCESS;
}

/* With one rank the root is the only member: its buffer already holds the data. */
int MPI_Bcast(void *buf, int count, MPI_Datatype type, int root, MPI_Comm comm) {
  (void)buf;
  if (!comm_ok(comm)) return MPI_ERR_COMM;
  if (root != 0 || count < 0 || base_size(type) == 0) return MPI_ERR_ARG;
  return MPI_SUCCESS;
}
/* Non-blocking form: complete on return (there is nothing to wait for). */
int MPI_Ibcast(void *buf, int count, MPI_Datatype type, int root, MPI_Comm comm, MPI_Request *request) {
  if (!request) return MPI_ERR_ARG;
  *request = MPI_REQUEST_NULL;
  return MPI_Bcast(buf, count, type, root, comm);
}
int MPI_Wait(MPI_Request *request, MPI_Status *status) {
  (void)status;
  if (!request) return MPI_ERR_ARG;
  *request = MPI_REQUEST_NULL;
  return MPI_SUCCESS;
}
int MPI_Waitall(int count, MPI_Request requests[], MPI_Status statuses[]) {
  (void)statuses;
  if (count < 0 || (count > 0 && !requests)) return MPI_ERR_ARG;
  for (int i = 0; i < count; ++i) requests[i] = MPI_REQUEST_NULL;
  return MPI_SUCCESS;
}
int MPI_Reduce(const void *sendbuf, void *recvbuf, int count, MPI_Datatype type, MPI_Op op, int root, MPI_Comm comm) {
  if (!comm_ok(comm)) return MPI_ERR_COMM;
  const int bs = base_size(type);
  if (root != 0 || (op != MPI_SUM && op != MPI_MAX) || count < 0 || bs <= 0) return MPI_ERR_ARG;
  if (sendbuf != MPI_IN_PLACE && sendbuf != recvbuf) memcpy(recvbuf, sendbuf, (size_t)count * bs);
  return MPI_SUCCESS;
}
int MPI_Send(const void *buf, int count, MPI_Datatype type, int dest, int tag, MPI_Comm comm) {
  (void)buf;
  (void)count;
  (void)type;
  (void)dest;
  (void)tag;
  (void)comm;
  return MPI_ERR_RANK; /* no peer in a one-process job */
}
int MPI_Recv(void *buf, int count, MPI_Datatype type, int source, int tag, MPI_Comm comm, MPI_Status *status) {
  (void)buf;
  (void)count;
  (void)type;
  (void)source;
  (void)tag;
  (void)comm;
  (void)status;
  return MPI_ERR_RANK;
}
