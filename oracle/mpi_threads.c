/*
 * mpi_threads.c - thread-per-rank MPI for the CPU tests (TEST INFRASTRUCTURE
 * ONLY; see oracle/mpi_threads/mpi.h for the contract).
 *
 * A communicator is a shared `group` (its members' world ranks, Cartesian
 * shape and a rendezvous: mutex, condition, arrival count, generation); each
 * thread maps its own MPI_Comm handles to groups. Collectives are two
 * rendezvous: the root (or every member) publishes a pointer and layout, all
 * meet, the others copy, all meet again. Point-to-point messages go through
 * a mailbox per world rank and are copied at send time.
 */
#include "mpi.h"

#include <errno.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#define MT_MAX_RANKS 64
#define MT_MAX_HANDLES 64
#define MT_MAX_DIMS 8

/* A buffer as `count` repetitions of `nblocks` runs of `blocklen` elements,
 * `stride` elements apart; repetitions are `extent` bytes apart. */
typedef struct {
  char *base;
  int count, nblocks, blocklen, stride, elsize;
  long extent;
} layout;

static long layout_elems(const layout *l) { return (long)l->count * l->nblocks * l->blocklen; }

static void layout_pack(const layout *l, char *dst) {
  const size_t run = (size_t)l->blocklen * l->elsize;
  for (int r = 0; r < l->count; ++r)
    for (int b = 0; b < l->nblocks; ++b) {
      memcpy(dst, l->base + r * l->extent + (long)b * l->stride * l->elsize, run);
      dst += run;
    }
}

static void layout_unpack(const layout *l, const char *src) {
  const size_t run = (size_t)l->blocklen * l->elsize;
  for (int r = 0; r < l->count; ++r)
    for (int b = 0; b < l->nblocks; ++b) {
      memcpy(l->base + r * l->extent + (long)b * l->stride * l->elsize, src, run);
      src += run;
    }
}

typedef struct group {
  int size, ctx, refs;
  int world[MT_MAX_RANKS];
  int ndims, dims[MT_MAX_DIMS], periods[MT_MAX_DIMS];
  pthread_mutex_t mu;
  pthread_cond_t cv;
  int arrived;
  unsigned gen;
  layout desc[MT_MAX_RANKS];
  const void *ptr[MT_MAX_RANKS];
  struct group *made[MT_MAX_RANKS];
} group;

typedef struct msg {
  struct msg *next;
  int ctx, src, tag, elsize;
  long nelems;
  char data[];
} msg;

static struct {
  pthread_mutex_t mu;
  pthread_cond_t cv;
  msg *head;
} g_box[MT_MAX_RANKS];

static pthread_mutex_t g_mu = PTHREAD_MUTEX_INITIALIZER;
static int g_next_ctx = 1;

static __thread int t_world_rank = -1;
static __thread int *t_result;
static __thread group *t_comm[MT_MAX_HANDLES];
static __thread int t_rank_in[MT_MAX_HANDLES];
static __thread struct {
  int live, nblocks, blocklen, stride, elsize;
} t_type[MT_MAX_HANDLES];
static __thread struct {
  int live;
  unsigned long seq;
  void *buf;
  int count, root;
  MPI_Datatype type;
  MPI_Comm comm;
} t_req[MT_MAX_HANDLES];
static __thread unsigned long t_req_seq;

static void deadline(struct timespec *ts) {
  clock_gettime(CLOCK_REALTIME, ts);
  ts->tv_sec += MPI_THREADS_WAIT_SECONDS;
}

static group *group_new(int size) {
  group *g = (group *)calloc(1, sizeof(group));
  if (!g) return NULL;
  g->size = size;
  g->refs = size;
  pthread_mutex_init(&g->mu, NULL);
  pthread_cond_init(&g->cv, NULL);
  pthread_mutex_lock(&g_mu);
  g->ctx = g_next_ctx++;
  pthread_mutex_unlock(&g_mu);
  return g;
}

static void group_release(group *g) {
  pthread_mutex_lock(&g_mu);
  const int last = --g->refs == 0;
  pthread_mutex_unlock(&g_mu);
  if (last) {
    pthread_mutex_destroy(&g->mu);
    pthread_cond_destroy(&g->cv);
    free(g);
  }
}

/* All members meet; MPI_ERR_OTHER when some member does not arrive in time. */
static int group_sync(group *g) {
  struct timespec until;
  deadline(&until);
  pthread_mutex_lock(&g->mu);
  const unsigned gen = g->gen;
  if (++g->arrived == g->size) {
    g->arrived = 0;
    g->gen++;
    pthread_cond_broadcast(&g->cv);
    pthread_mutex_unlock(&g->mu);
    return MPI_SUCCESS;
  }
  while (g->gen == gen)
    if (pthread_cond_timedwait(&g->cv, &g->mu, &until) == ETIMEDOUT && g->gen == gen) {
      pthread_mutex_unlock(&g->mu);
      fprintf(stderr, "mpi_threads: rank %d timed out in a collective\n", t_world_rank);
      return MPI_ERR_OTHER;
    }
  pthread_mutex_unlock(&g->mu);
  return MPI_SUCCESS;
}

static group *comm_group(MPI_Comm c) {
  if (c <= 0 || c >= MT_MAX_HANDLES) return NULL;
  return t_comm[c];
}

static int new_handle(group *g, int rank_in, MPI_Comm *out) {
  for (int h = 2; h < MT_MAX_HANDLES; ++h)
    if (!t_comm[h]) {
      t_comm[h] = g;
      t_rank_in[h] = rank_in;
      *out = h;
      return MPI_SUCCESS;
    }
  return MPI_ERR_COMM;
}

static int elsize_of(MPI_Datatype t) {
  switch (t) {
    case MPI_FLOAT: return 4;
    case MPI_DOUBLE: return 8;
    case MPI_INT: return 4;
    default: return 0;
  }
}

static int make_layout(void *buf, int count, MPI_Datatype t, layout *l) {
  if (count < 0) return MPI_ERR_ARG;
  l->base = (char *)buf;
  l->count = count;
  const int es = elsize_of(t);
  if (es) {
    l->nblocks = 1;
    l->blocklen = 1;
    l->stride = 1;
    l->elsize = es;
    l->extent = es;
    return MPI_SUCCESS;
  }
  const int h = t - 16;
  if (h < 0 || h >= MT_MAX_HANDLES || !t_type[h].live) return MPI_ERR_ARG;
  l->nblocks = t_type[h].nblocks;
  l->blocklen = t_type[h].blocklen;
  l->stride = t_type[h].stride;
  l->elsize = t_type[h].elsize;
  l->extent = ((long)(l->nblocks - 1) * l->stride + l->blocklen) * l->elsize;
  return MPI_SUCCESS;
}

static int flush_requests(void);

/* ---- environment ------------------------------------------------------- */

int MPI_Init(int *argc, char ***argv) {
  (void)argc;
  (void)argv;
  return t_world_rank >= 0 ? MPI_SUCCESS : MPI_ERR_OTHER;
}
int MPI_Finalize(void) { return flush_requests(); }
int MPI_Abort(MPI_Comm comm, int errorcode) {
  (void)comm;
  fflush(stdout);
  fflush(stderr);
  if (t_result) *t_result = errorcode ? errorcode : 1;
  pthread_exit(NULL);
}
int MPI_Comm_size(MPI_Comm comm, int *size) {
  group *g = comm_group(comm);
  if (!g || !size) return MPI_ERR_COMM;
  *size = g->size;
  return MPI_SUCCESS;
}
int MPI_Comm_rank(MPI_Comm comm, int *rank) {
  group *g = comm_group(comm);
  if (!g || !rank) return MPI_ERR_COMM;
  *rank = t_rank_in[comm];
  return MPI_SUCCESS;
}
int MPI_Comm_free(MPI_Comm *comm) {
  if (!comm || *comm == MPI_COMM_WORLD) return MPI_ERR_COMM;
  group *g = comm_group(*comm);
  if (!g) return MPI_ERR_COMM;
  t_comm[*comm] = NULL;
  *comm = MPI_COMM_NULL;
  group_release(g);
  return MPI_SUCCESS;
}
int MPI_Barrier(MPI_Comm comm) {
  group *g = comm_group(comm);
  if (!g) return MPI_ERR_COMM;
  const int rc = flush_requests();
  return rc ? rc : group_sync(g);
}

/* Balanced factorisation of nnodes over the dimensions that are 0 on entry,
 * non-increasing over those dimensions. */
int MPI_Dims_create(int nnodes, int ndims, int dims[]) {
  if (nnodes < 1 || ndims < 1 || ndims > MT_MAX_DIMS) return MPI_ERR_ARG;
  int fixed = 1, nfree = 0, fr[MT_MAX_DIMS];
  for (int i = 0; i < ndims; ++i) {
    if (dims[i] < 0) return MPI_ERR_ARG;
    if (dims[i] > 0)
      fixed *= dims[i];
    else
      fr[nfree++] = i;
  }
  if (nnodes % fixed) return MPI_ERR_ARG;
  int rest = nnodes / fixed;
  if (!nfree) return rest == 1 ? MPI_SUCCESS : MPI_ERR_ARG;
  int val[MT_MAX_DIMS];
  for (int i = 0; i < nfree; ++i) val[i] = 1;
  int primes[32], np = 0;
  for (int f = 2; rest > 1;)
    if (rest % f == 0) {
      primes[np++] = f;
      rest /= f;
    } else {
      ++f;
    }
  for (int j = np - 1; j >= 0; --j) { /* largest prime onto the smallest value */
    int lo = 0;
    for (int i = 1; i < nfree; ++i)
      if (val[i] < val[lo]) lo = i;
    val[lo] *= primes[j];
  }
  for (int i = 0; i < nfree; ++i)
    for (int j = i + 1; j < nfree; ++j)
      if (val[j] > val[i]) {
        const int t = val[i];
        val[i] = val[j];
        val[j] = t;
      }
  for (int i = 0; i < nfree; ++i) dims[fr[i]] = val[i];
  return MPI_SUCCESS;
}

/* ---- Cartesian communicators ------------------------------------------- */

static void coords_of(const group *g, int rank, int *coords) {
  for (int d = g->ndims - 1; d >= 0; --d) {
    coords[d] = rank % g->dims[d];
    rank /= g->dims[d];
  }
}

int MPI_Cart_create(MPI_Comm old, int ndims, const int dims[], const int periods[], int reorder, MPI_Comm *cart) {
  (void)reorder;
  group *g = comm_group(old);
  if (!g || !cart || ndims < 1 || ndims > MT_MAX_DIMS) return MPI_ERR_ARG;
  int n = 1;
  for (int d = 0; d < ndims; ++d) n *= dims[d];
  if (n != g->size) return MPI_ERR_ARG; /* every rank of `old` takes part */
  int rc = flush_requests();
  if (!rc) rc = group_sync(g);
  if (rc) return rc;
  const int me = t_rank_in[old];
  if (me == 0) {
    group *c = group_new(g->size);
    if (c) {
      memcpy(c->world, g->world, sizeof(int) * g->size);
      c->ndims = ndims;
      for (int d = 0; d < ndims; ++d) {
        c->dims[d] = dims[d];
        c->periods[d] = periods ? periods[d] : 0;
      }
    }
    g->made[0] = c;
  }
  rc = group_sync(g);
  group *c = g->made[0];
  const int rc2 = group_sync(g);
  if (me == 0) g->made[0] = NULL;
  if (rc || rc2) return rc ? rc : rc2;
  if (!c) return MPI_ERR_OTHER;
  return new_handle(c, me, cart);
}

int MPI_Cart_coords(MPI_Comm comm, int rank, int maxdims, int coords[]) {
  group *g = comm_group(comm);
  if (!g || g->ndims == 0) return MPI_ERR_COMM;
  if (rank < 0 || rank >= g->size || maxdims < g->ndims) return MPI_ERR_RANK;
  coords_of(g, rank, coords);
  return MPI_SUCCESS;
}

int MPI_Cart_get(MPI_Comm comm, int maxdims, int dims[], int periods[], int coords[]) {
  group *g = comm_group(comm);
  if (!g || g->ndims == 0) return MPI_ERR_COMM;
  if (maxdims < g->ndims) return MPI_ERR_ARG;
  int c[MT_MAX_DIMS];
  coords_of(g, t_rank_in[comm], c);
  for (int d = 0; d < g->ndims; ++d) {
    dims[d] = g->dims[d];
    periods[d] = g->periods[d];
    coords[d] = c[d];
  }
  return MPI_SUCCESS;
}

/* Members with equal coordinates in the dropped dimensions form one
 * sub-communicator, ranked row-major over the kept dimensions. */
int MPI_Cart_sub(MPI_Comm comm, const int remain_dims[], MPI_Comm *sub) {
  group *g = comm_group(comm);
  if (!g || g->ndims == 0 || !sub) return MPI_ERR_COMM;
  const int me = t_rank_in[comm];
  int c[MT_MAX_DIMS];
  coords_of(g, me, c);
  int color = 0, key = 0, size = 1, kept = 0, kdims[MT_MAX_DIMS], kper[MT_MAX_DIMS];
  for (int d = 0; d < g->ndims; ++d) {
    if (remain_dims[d]) {
      key = key * g->dims[d] + c[d];
      size *= g->dims[d];
      kdims[kept] = g->dims[d];
      kper[kept++] = g->periods[d];
    } else {
      color = color * g->dims[d] + c[d];
    }
  }
  int rc = flush_requests();
  if (!rc) rc = group_sync(g);
  if (rc) return rc;
  pthread_mutex_lock(&g->mu);
  if (!g->made[color]) {
    group *s = group_new(size);
    if (s) {
      s->ndims = kept ? kept : 1;
      for (int d = 0; d < kept; ++d) {
        s->dims[d] = kdims[d];
        s->periods[d] = kper[d];
      }
      if (!kept) s->dims[0] = 1;
      /* member r of the new group: my coordinates with the kept ones replaced
       * by r's row-major coordinates over the kept dimensions */
      for (int r = 0; r < size; ++r) {
        int full[MT_MAX_DIMS], rest = r;
        for (int d = g->ndims - 1; d >= 0; --d) {
          if (remain_dims[d]) {
            full[d] = rest % g->dims[d];
            rest /= g->dims[d];
          } else {
            full[d] = c[d];
          }
        }
        int old_rank = 0;
        for (int d = 0; d < g->ndims; ++d) old_rank = old_rank * g->dims[d] + full[d];
        s->world[r] = g->world[old_rank];
      }
    }
    g->made[color] = s;
  }
  group *s = g->made[color];
  pthread_mutex_unlock(&g->mu);
  rc = group_sync(g);
  if (me == 0) memset(g->made, 0, sizeof(g->made));
  if (rc) return rc;
  if (!s) return MPI_ERR_OTHER;
  return new_handle(s, key, sub);
}

/* ---- datatypes --------------------------------------------------------- */

int MPI_Type_vector(int count, int blocklength, int stride, MPI_Datatype old, MPI_Datatype *newtype) {
  const int es = elsize_of(old);
  if (count < 0 || blocklength < 0 || !es || !newtype) return MPI_ERR_ARG;
  for (int h = 0; h < MT_MAX_HANDLES; ++h)
    if (!t_type[h].live) {
      t_type[h].live = 1;
      t_type[h].nblocks = count;
      t_type[h].blocklen = blocklength;
      t_type[h].stride = stride;
      t_type[h].elsize = es;
      *newtype = 16 + h;
      return MPI_SUCCESS;
    }
  return MPI_ERR_ARG;
}
int MPI_Type_commit(MPI_Datatype *type) {
  layout l;
  return type && make_layout(NULL, 1, *type, &l) == MPI_SUCCESS ? MPI_SUCCESS : MPI_ERR_ARG;
}
int MPI_Type_free(MPI_Datatype *type) {
  if (!type) return MPI_ERR_ARG;
  const int h = *type - 16;
  if (h < 0 || h >= MT_MAX_HANDLES || !t_type[h].live) return MPI_ERR_ARG;
  t_type[h].live = 0;
  *type = MPI_DATATYPE_NULL;
  return MPI_SUCCESS;
}

/* ---- broadcast --------------------------------------------------------- */

static int bcast_now(void *buf, int count, MPI_Datatype type, int root, MPI_Comm comm) {
  group *g = comm_group(comm);
  if (!g) return MPI_ERR_COMM;
  if (root < 0 || root >= g->size) return MPI_ERR_ARG;
  layout mine;
  int rc = make_layout(buf, count, type, &mine);
  if (rc) return rc;
  const int me = t_rank_in[comm];
  if (me == root) g->desc[root] = mine;
  rc = group_sync(g);
  if (rc) return rc;
  int err = MPI_SUCCESS;
  if (me != root) {
    const layout *src = &g->desc[root];
    if (src->elsize != mine.elsize || layout_elems(src) != layout_elems(&mine)) {
      err = MPI_ERR_TRUNCATE;
    } else {
      char *tmp = (char *)malloc((size_t)layout_elems(src) * src->elsize + 1);
      if (!tmp) {
        err = MPI_ERR_OTHER;
      } else {
        layout_pack(src, tmp);
        layout_unpack(&mine, tmp);
        free(tmp);
      }
    }
  }
  rc = group_sync(g);
  return err ? err : rc;
}

/* Completes this rank's pending non-blocking broadcasts, oldest first. */
static int complete_until(unsigned long seq) {
  int rc = MPI_SUCCESS;
  for (;;) {
    int best = -1;
    for (int h = 1; h < MT_MAX_HANDLES; ++h)
      if (t_req[h].live && t_req[h].seq <= seq && (best < 0 || t_req[h].seq < t_req[best].seq)) best = h;
    if (best < 0) return rc;
    t_req[best].live = 0;
    const int r = bcast_now(t_req[best].buf, t_req[best].count, t_req[best].type, t_req[best].root,
                            t_req[best].comm);
    if (r && !rc) rc = r;
  }
}

static int flush_requests(void) { return complete_until(~0UL); }

int mpi_threads_pending(void) {
  int n = 0;
  for (int h = 1; h < MT_MAX_HANDLES; ++h) n += t_req[h].live;
  return n;
}

int MPI_Bcast(void *buf, int count, MPI_Datatype type, int root, MPI_Comm comm) {
  const int rc = flush_requests();
  return rc ? rc : bcast_now(buf, count, type, root, comm);
}

int MPI_Ibcast(void *buf, int count, MPI_Datatype type, int root, MPI_Comm comm, MPI_Request *request) {
  group *g = comm_group(comm);
  layout l;
  if (!request) return MPI_ERR_ARG;
  if (!g) return MPI_ERR_COMM;
  if (root < 0 || root >= g->size || make_layout(buf, count, type, &l)) return MPI_ERR_ARG;
  for (int h = 1; h < MT_MAX_HANDLES; ++h)
    if (!t_req[h].live) {
      t_req[h].live = 1;
      t_req[h].seq = ++t_req_seq;
      t_req[h].buf = buf;
      t_req[h].count = count;
      t_req[h].type = type;
      t_req[h].root = root;
      t_req[h].comm = comm;
      *request = h;
      return MPI_SUCCESS;
    }
  return MPI_ERR_OTHER;
}

int MPI_Wait(MPI_Request *request, MPI_Status *status) {
  (void)status;
  if (!request) return MPI_ERR_ARG;
  const int h = *request;
  if (h == MPI_REQUEST_NULL) return MPI_SUCCESS;
  if (h < 1 || h >= MT_MAX_HANDLES || !t_req[h].live) return MPI_ERR_ARG;
  *request = MPI_REQUEST_NULL;
  return complete_until(t_req[h].seq);
}

int MPI_Waitall(int count, MPI_Request requests[], MPI_Status statuses[]) {
  (void)statuses;
  int rc = MPI_SUCCESS;
  for (int i = 0; i < count; ++i) {
    const int r = MPI_Wait(&requests[i], MPI_STATUS_IGNORE);
    if (r && !rc) rc = r;
  }
  return rc;
}

/* ---- reduction --------------------------------------------------------- */

int MPI_Reduce(const void *sendbuf, void *recvbuf, int count, MPI_Datatype type, MPI_Op op, int root, MPI_Comm comm) {
  group *g = comm_group(comm);
  if (!g) return MPI_ERR_COMM;
  const int es = elsize_of(type);
  if (!es || count < 0 || root < 0 || root >= g->size || (op != MPI_SUM && op != MPI_MAX)) return MPI_ERR_ARG;
  int rc = flush_requests();
  if (rc) return rc;
  const int me = t_rank_in[comm];
  g->ptr[me] = (me == root && sendbuf == MPI_IN_PLACE) ? recvbuf : sendbuf;
  rc = group_sync(g);
  if (rc) return rc;
  if (me == root) {
    for (int i = 0; i < count; ++i) { /* rank order: ((x0 op x1) op x2) ... */
      double acc = 0;
      for (int r = 0; r < g->size; ++r) {
        const char *p = (const char *)g->ptr[r] + (size_t)i * es;
        const double v = type == MPI_FLOAT ? *(const float *)p : type == MPI_DOUBLE ? *(const double *)p
                                                                                   : *(const int *)p;
        if (type == MPI_FLOAT) {
          const float a = (float)acc, b = (float)v;
          acc = r == 0 ? b : (op == MPI_SUM ? (double)(a + b) : (a > b ? a : b));
        } else {
          acc = r == 0 ? v : (op == MPI_SUM ? acc + v : (acc > v ? acc : v));
        }
      }
      char *q = (char *)recvbuf + (size_t)i * es;
      if (type == MPI_FLOAT)
        *(float *)q = (float)acc;
      else if (type == MPI_DOUBLE)
        *(double *)q = acc;
      else
        *(int *)q = (int)acc;
    }
  }
  return group_sync(g);
}

/* ---- point to point ---------------------------------------------------- */

int MPI_Send(const void *buf, int count, MPI_Datatype type, int dest, int tag, MPI_Comm comm) {
  group *g = comm_group(comm);
  if (!g) return MPI_ERR_COMM;
  if (dest < 0 || dest >= g->size) return MPI_ERR_RANK;
  layout l;
  if (make_layout((void *)buf, count, type, &l)) return MPI_ERR_ARG;
  const long ne = layout_elems(&l);
  msg *m = (msg *)malloc(sizeof(msg) + (size_t)ne * l.elsize);
  if (!m) return MPI_ERR_OTHER;
  m->next = NULL;
  m->ctx = g->ctx;
  m->src = t_rank_in[comm];
  m->tag = tag;
  m->elsize = l.elsize;
  m->nelems = ne;
  layout_pack(&l, m->data);
  const int w = g->world[dest];
  pthread_mutex_lock(&g_box[w].mu);
  msg **tail = &g_box[w].head;
  while (*tail) tail = &(*tail)->next;
  *tail = m;
  pthread_cond_broadcast(&g_box[w].cv);
  pthread_mutex_unlock(&g_box[w].mu);
  return MPI_SUCCESS;
}

int MPI_Recv(void *buf, int count, MPI_Datatype type, int source, int tag, MPI_Comm comm, MPI_Status *status) {
  group *g = comm_group(comm);
  if (!g) return MPI_ERR_COMM;
  if (source < 0 || source >= g->size) return MPI_ERR_RANK;
  layout l;
  if (make_layout(buf, count, type, &l)) return MPI_ERR_ARG;
  const int w = t_world_rank;
  struct timespec until;
  deadline(&until);
  msg *m = NULL;
  pthread_mutex_lock(&g_box[w].mu);
  for (;;) {
    for (msg **p = &g_box[w].head; *p; p = &(*p)->next)
      if ((*p)->ctx == g->ctx && (*p)->src == source && (*p)->tag == tag) {
        m = *p;
        *p = m->next;
        break;
      }
    if (m) break;
    if (pthread_cond_timedwait(&g_box[w].cv, &g_box[w].mu, &until) == ETIMEDOUT) break;
  }
  pthread_mutex_unlock(&g_box[w].mu);
  if (!m) {
    fprintf(stderr, "mpi_threads: rank %d timed out in MPI_Recv\n", t_world_rank);
    return MPI_ERR_OTHER;
  }
  int rc = MPI_SUCCESS;
  if (m->elsize != l.elsize || m->nelems != layout_elems(&l))
    rc = MPI_ERR_TRUNCATE;
  else
    layout_unpack(&l, m->data);
  if (status) {
    status->MPI_SOURCE = source;
    status->MPI_TAG = tag;
    status->MPI_ERROR = rc;
  }
  free(m);
  return rc;
}

/* ---- launcher ---------------------------------------------------------- */

typedef struct {
  int (*body)(void *, int);
  void *arg;
  group *world;
  int rank, result;
} rank_start;

static void *rank_main(void *p) {
  rank_start *s = (rank_start *)p;
  t_world_rank = s->rank;
  t_result = &s->result;
  memset(t_comm, 0, sizeof(t_comm));
  memset(t_type, 0, sizeof(t_type));
  memset(t_req, 0, sizeof(t_req));
  t_req_seq = 0;
  t_comm[MPI_COMM_WORLD] = s->world;
  t_rank_in[MPI_COMM_WORLD] = s->rank;
  s->result = s->body(s->arg, s->rank);
  if (s->result == 0 && mpi_threads_pending()) s->result = MPI_ERR_OTHER;
  return NULL;
}

int mpi_threads_run(int nprocs, int (*body)(void *arg, int rank), void *arg) {
  if (nprocs < 1 || nprocs > MT_MAX_RANKS || !body) return -1;
  group *world = group_new(nprocs);
  rank_start *st = (rank_start *)calloc((size_t)nprocs, sizeof(rank_start));
  pthread_t *tid = (pthread_t *)calloc((size_t)nprocs, sizeof(pthread_t));
  if (!world || !st || !tid) {
    free(world);
    free(st);
    free(tid);
    return -1;
  }
  for (int r = 0; r < nprocs; ++r) {
    world->world[r] = r;
    pthread_mutex_init(&g_box[r].mu, NULL);
    pthread_cond_init(&g_box[r].cv, NULL);
    g_box[r].head = NULL;
  }
  int started = 0, rc = 0;
  for (int r = 0; r < nprocs; ++r) {
    st[r] = (rank_start){body, arg, world, r, -1};
    if (pthread_create(&tid[r], NULL, rank_main, &st[r]) != 0) break;
    ++started;
  }
  for (int r = 0; r < started; ++r) pthread_join(tid[r], NULL);
  if (started < nprocs) rc = -1;
  for (int r = 0; r < nprocs && !rc; ++r)
    if (st[r].result) rc = st[r].result;
  for (int r = 0; r < nprocs; ++r) {
    while (g_box[r].head) { /* messages nobody received */
      msg *m = g_box[r].head;
      g_box[r].head = m->next;
      free(m);
      if (!rc) rc = MPI_ERR_OTHER;
    }
  }
  free(tid);
  free(st);
  for (int r = 0; r < nprocs; ++r) group_release(world); /* one reference per rank */
  return rc;
}
