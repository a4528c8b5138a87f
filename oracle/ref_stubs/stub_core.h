/* ORACLE BUILD SUPPORT (test infrastructure only).
 *
 * Minimal stand-ins for the parts of p4est, libsc, PETSc and MPI that the reference's headers name, so that
 * reference translation units whose arithmetic does not depend on those libraries compile unchanged from the
 * reference tree. Only the declarations the reference code mentions are given; the functions that a reference
 * build here actually calls are defined in ref_stubs.cpp (single process, no ghost layer), the rest are
 * declared and never called.
 */
#ifndef REF_STUB_CORE_H
#define REF_STUB_CORE_H

#include <limits.h>
#include <math.h>
#include <stddef.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/types.h>
#include <stdarg.h>
#include <unistd.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- MPI (one process) */
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;
#define MPI_COMM_WORLD 0
#define MPI_COMM_SELF 1
#define MPI_SUCCESS 0
#define MPI_DOUBLE 1
#define MPI_INT 2
#define MPI_UNSIGNED_CHAR 3
#define MPI_UNSIGNED_SHORT 4
#define MPI_UNSIGNED 5
#define MPI_UNSIGNED_LONG 6
#define MPI_UNSIGNED_LONG_LONG 7
#define MPI_CHAR 8
#define MPI_LONG 9
#define MPI_LONG_LONG 10
#define MPI_LONG_LONG_INT 10
#define MPI_SHORT 11
#define MPI_FLOAT 12
#define MPI_BYTE 13
#define MPI_C_BOOL 14
#define MPI_CXX_BOOL 14
#define MPI_INT8_T 15
#define MPI_INT64_T 16
#define MPI_MAX 1
#define MPI_MIN 2
#define MPI_SUM 3
#define MPI_LOR 4
#define MPI_LAND 5
#define MPI_MAXLOC 6
#define MPI_IN_PLACE ((void*)1)
#define MPI_STATUS_IGNORE ((MPI_Status*)0)
#define MPI_STATUSES_IGNORE ((MPI_Status*)0)
#define MPI_ANY_SOURCE (-1)
#define MPI_ANY_TAG (-1)
#define MPI_REQUEST_NULL 0
#define MPI_DATATYPE_NULL 0
double MPI_Wtime(void);
int MPI_Comm_size(MPI_Comm, int*);
int MPI_Comm_rank(MPI_Comm, int*);
int MPI_Init(int*, char***);
int MPI_Finalize(void);
int MPI_Barrier(MPI_Comm);
int MPI_Bcast(void*, int, MPI_Datatype, int, MPI_Comm);
int MPI_Gather(const void*, int, MPI_Datatype, void*, int, MPI_Datatype, int, MPI_Comm);
int MPI_Allgatherv(const void*, int, MPI_Datatype, void*, const int*, const int*, MPI_Datatype, MPI_Comm);
int MPI_Reduce_scatter(const void*, void*, const int*, MPI_Datatype, MPI_Op, MPI_Comm);
int MPI_Allgather(const void*, int, MPI_Datatype, void*, int, MPI_Datatype, MPI_Comm);
int MPI_Allreduce(const void*, void*, int, MPI_Datatype, MPI_Op, MPI_Comm);
int MPI_Reduce(const void*, void*, int, MPI_Datatype, MPI_Op, int, MPI_Comm);
int MPI_Isend(const void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request*);
int MPI_Irecv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request*);
int MPI_Send(const void*, int, MPI_Datatype, int, int, MPI_Comm);
int MPI_Recv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status*);
int MPI_Waitall(int, MPI_Request*, MPI_Status*);
int MPI_Wait(MPI_Request*, MPI_Status*);
int MPI_Probe(int, int, MPI_Comm, MPI_Status*);
int MPI_Iprobe(int, int, MPI_Comm, int*, MPI_Status*);
int MPI_Get_count(const MPI_Status*, MPI_Datatype, int*);
int MPI_Abort(MPI_Comm, int);
int MPI_Scan(const void*, void*, int, MPI_Datatype, MPI_Op, MPI_Comm);
int MPI_Alltoall(const void*, int, MPI_Datatype, void*, int, MPI_Datatype, MPI_Comm);

/* ---------------------------------------------------------------- libsc */
typedef struct sc_array {
  size_t elem_size;
  size_t elem_count;
  ssize_t byte_alloc;
  char *array;
} sc_array_t;
static inline void *sc_array_index(sc_array_t *a, size_t i) { return (void *)(a->array + a->elem_size * i); }
static inline void *sc_array_index_int(sc_array_t *a, int i) { return (void *)(a->array + a->elem_size * (size_t)i); }
sc_array_t *sc_array_new(size_t elem_size);
sc_array_t *sc_array_new_size(size_t elem_size, size_t n);
void sc_array_init(sc_array_t *a, size_t elem_size);
void sc_array_reset(sc_array_t *a);
void sc_array_destroy(sc_array_t *a);
void sc_array_resize(sc_array_t *a, size_t n);
void *sc_array_push(sc_array_t *a);
void *sc_array_push_count(sc_array_t *a, size_t n);
void sc_array_sort(sc_array_t *a, int (*compar)(const void *, const void *));
ssize_t sc_array_bsearch(sc_array_t *a, const void *key, int (*compar)(const void *, const void *));
void sc_array_truncate(sc_array_t *a);
void sc_init(MPI_Comm, int, int, void *, int);
void sc_finalize(void);
typedef void (*sc_log_handler_t)(FILE *, const char *, int, int, int, int, const char *);
#define SC_LP_DEFAULT (-1)
#define SC_LP_SILENT 9
#define SC_LP_ESSENTIAL 6
#define SC_LP_ERROR 8
#define SC_LP_PRODUCTION 5
#define SC_LP_INFO 4
#ifdef __cplusplus
#define SC_EXTERN_C_BEGIN extern "C" {
#define SC_EXTERN_C_END }
#else
#define SC_EXTERN_C_BEGIN
#define SC_EXTERN_C_END
#endif
#define SC_CHECK_MPI(r) ((void)(r))
#define SC_CHECK_ABORT(c, s) ((void)(c))
#define SC_ASSERT(c) ((void)0)
#define SC_ABORT(s) abort()
#define SC_ALLOC(t, n) ((t *)malloc((n) * sizeof(t)))
#define SC_FREE(p) free(p)
#define SC_MIN(a, b) ((a) < (b) ? (a) : (b))
#define SC_MAX(a, b) ((a) > (b) ? (a) : (b))

/* ---------------------------------------------------------------- p4est */
typedef int32_t p4est_qcoord_t;
typedef int32_t p4est_topidx_t;
typedef int32_t p4est_locidx_t;
typedef int64_t p4est_gloidx_t;
typedef int p4est_bool_t;
#define P4EST_FALSE 0
#define P4EST_TRUE 1
#define P4EST_MPI_LOCIDX MPI_INT
#define P4EST_MPI_GLOIDX MPI_LONG_LONG_INT
#define P4EST_MPI_TOPIDX MPI_INT
#define P4EST_LOCIDX_MAX INT32_MAX
#define P4EST_GLOIDX_MAX INT64_MAX
#define P4EST_TOPIDX_MAX INT32_MAX

#ifdef P4_TO_P8
#define P4EST_DIM 3
#define P4EST_FACES 6
#define P4EST_CHILDREN 8
#define P4EST_HALF 4
#define P4EST_EDGES 12
#define P4EST_MAXLEVEL 19
#define P4EST_QMAXLEVEL 18
#define P4EST_STRING "p8est"
#else
#define P4EST_DIM 2
#define P4EST_FACES 4
#define P4EST_CHILDREN 4
#define P4EST_HALF 2
#define P4EST_MAXLEVEL 30
#define P4EST_QMAXLEVEL 29
#define P4EST_STRING "p4est"
#endif
#define P8EST_DIM 3
#define P8EST_FACES 6
#define P8EST_CHILDREN 8
#define P8EST_MAXLEVEL 19
#define P4EST_ROOT_LEN ((p4est_qcoord_t)1 << P4EST_MAXLEVEL)
#define P4EST_QUADRANT_LEN(l) ((p4est_qcoord_t)1 << (P4EST_MAXLEVEL - (l)))
#define P4EST_LAST_OFFSET(l) (P4EST_ROOT_LEN - P4EST_QUADRANT_LEN(l))
#define P8EST_ROOT_LEN ((p4est_qcoord_t)1 << P8EST_MAXLEVEL)
#define P8EST_QUADRANT_LEN(l) ((p4est_qcoord_t)1 << (P8EST_MAXLEVEL - (l)))
#define P4EST_ASSERT(c) ((void)0)
#define P4EST_QUADRANT_INIT(q) ((void)memset((q), 0, sizeof(p4est_quadrant_t)))
#define P4EST_GLOBAL_PRODUCTIONF(...) ((void)0)
#define P4EST_GLOBAL_PRODUCTION(...) ((void)0)
#define P4EST_LDEBUGF(...) ((void)0)
#define P4EST_ALLOC(t, n) ((t *)malloc((n) * sizeof(t)))
#define P4EST_ALLOC_ZERO(t, n) ((t *)calloc((n), sizeof(t)))
#define P4EST_REALLOC(p, t, n) ((t *)realloc((p), (n) * sizeof(t)))
#define P4EST_FREE(p) free(p)

typedef struct p4est_quadrant {
  p4est_qcoord_t x, y;
#ifdef P4_TO_P8
  p4est_qcoord_t z;
#endif
  int8_t level, pad8;
  int16_t pad16;
  union {
    void *user_data;
    long user_long;
    int user_int;
    p4est_topidx_t which_tree;
    struct { p4est_topidx_t which_tree; int owner_rank; } piggy1;
    struct { p4est_topidx_t which_tree; p4est_topidx_t from_tree; } piggy2;
    struct { p4est_topidx_t which_tree; p4est_locidx_t local_num; } piggy3;
  } p;
} p4est_quadrant_t;
typedef p4est_quadrant_t p4est_indep_t;

typedef struct p4est_tree {
  sc_array_t quadrants;
  p4est_quadrant_t first_desc, last_desc;
  p4est_locidx_t quadrants_offset;
  p4est_locidx_t quadrants_per_level[P4EST_MAXLEVEL + 1];
  int8_t maxlevel;
} p4est_tree_t;

typedef enum { P4EST_CONNECT_SELF = 20, P4EST_CONNECT_FACE = 21, P4EST_CONNECT_EDGE = 22, P4EST_CONNECT_CORNER = 23,
               P4EST_CONNECT_FULL = 23 } p4est_connect_type_t;
#define P8EST_CONNECT_FULL P4EST_CONNECT_FULL
#define P8EST_CONNECT_FACE P4EST_CONNECT_FACE

typedef struct p4est_connectivity {
  p4est_topidx_t num_vertices;
  p4est_topidx_t num_trees;
#ifdef P4_TO_P8
  p4est_topidx_t num_edges;
#endif
  p4est_topidx_t num_corners;
  double *vertices;
  p4est_topidx_t *tree_to_vertex;
  size_t tree_attr_bytes;
  char *tree_to_attr;
  p4est_topidx_t *tree_to_tree;
  int8_t *tree_to_face;
#ifdef P4_TO_P8
  p4est_topidx_t *tree_to_edge;
#endif
  p4est_topidx_t *tree_to_corner;
  p4est_topidx_t *ctt_offset;
  p4est_topidx_t *corner_to_tree;
  int8_t *corner_to_corner;
} p4est_connectivity_t;

typedef struct p4est_inspect p4est_inspect_t;
typedef struct p4est {
  MPI_Comm mpicomm;
  int mpisize, mpirank;
  int mpicomm_owned;
  size_t data_size;
  void *user_pointer;
  long revision;
  p4est_topidx_t first_local_tree;
  p4est_topidx_t last_local_tree;
  p4est_locidx_t local_num_quadrants;
  p4est_gloidx_t global_num_quadrants;
  p4est_gloidx_t *global_first_quadrant;
  p4est_quadrant_t *global_first_position;
  p4est_connectivity_t *connectivity;
  sc_array_t *trees;
  void *user_data_pool;
  void *quadrant_pool;
  p4est_inspect_t *inspect;
} p4est_t;

typedef struct p4est_ghost {
  int mpisize;
  p4est_topidx_t num_trees;
  p4est_connect_type_t btype;
  sc_array_t ghosts;
  p4est_locidx_t *tree_offsets;
  p4est_locidx_t *proc_offsets;
  sc_array_t mirrors;
  p4est_locidx_t *mirror_tree_offsets;
  p4est_locidx_t *mirror_proc_mirrors;
  p4est_locidx_t *mirror_proc_offsets;
  p4est_locidx_t *mirror_proc_fronts;
  p4est_locidx_t *mirror_proc_front_offsets;
} p4est_ghost_t;

typedef struct p4est_nodes {
  p4est_locidx_t num_local_quadrants;
  p4est_locidx_t num_owned_indeps, num_owned_shared;
  p4est_locidx_t offset_owned_indeps;
  sc_array_t indep_nodes;
  sc_array_t face_hangings;
#ifdef P4_TO_P8
  sc_array_t edge_hangings;
#endif
  p4est_locidx_t *local_nodes;
  sc_array_t shared_indeps;
  p4est_locidx_t *shared_offsets;
  int *nonlocal_ranks;
  p4est_locidx_t *global_owned_indeps;
} p4est_nodes_t;

typedef void (*p4est_init_t)(p4est_t *, p4est_topidx_t, p4est_quadrant_t *);
typedef int (*p4est_refine_t)(p4est_t *, p4est_topidx_t, p4est_quadrant_t *);
typedef int (*p4est_coarsen_t)(p4est_t *, p4est_topidx_t, p4est_quadrant_t *[]);
typedef int (*p4est_weight_t)(p4est_t *, p4est_topidx_t, p4est_quadrant_t *);
typedef void (*p4est_replace_t)(p4est_t *, p4est_topidx_t, int, p4est_quadrant_t *[], int, p4est_quadrant_t *[]);

static inline p4est_tree_t *p4est_tree_array_index(sc_array_t *a, p4est_topidx_t i) { return (p4est_tree_t *)(a->array + sizeof(p4est_tree_t) * (size_t)i); }
static inline p4est_quadrant_t *p4est_quadrant_array_index(sc_array_t *a, size_t i) { return (p4est_quadrant_t *)(a->array + sizeof(p4est_quadrant_t) * i); }
static inline p4est_quadrant_t *p4est_quadrant_array_push(sc_array_t *a) { return (p4est_quadrant_t *)sc_array_push(a); }

void p4est_node_clamp_inside(const p4est_quadrant_t *, p4est_quadrant_t *);
void p4est_node_unclamp(p4est_quadrant_t *);
void p4est_nodes_destroy(p4est_nodes_t *);
int p4est_nodes_is_valid(p4est_t *, p4est_nodes_t *);
p4est_nodes_t *p4est_nodes_new(p4est_t *, p4est_ghost_t *);
p4est_ghost_t *p4est_ghost_new(p4est_t *, p4est_connect_type_t);
void p4est_ghost_destroy(p4est_ghost_t *);
void p4est_ghost_expand(p4est_t *, p4est_ghost_t *);
ssize_t p4est_ghost_contains(p4est_ghost_t *, int, p4est_topidx_t, const p4est_quadrant_t *);
ssize_t p4est_ghost_bsearch(p4est_ghost_t *, int, p4est_topidx_t, const p4est_quadrant_t *);
void p4est_ghost_exchange_data(p4est_t *, p4est_ghost_t *, void *);
p4est_t *p4est_new(MPI_Comm, p4est_connectivity_t *, size_t, p4est_init_t, void *);
p4est_t *p4est_new_ext(MPI_Comm, p4est_connectivity_t *, p4est_locidx_t, int, int, size_t, p4est_init_t, void *);
p4est_t *p4est_copy(p4est_t *, int);
void p4est_destroy(p4est_t *);
void p4est_refine(p4est_t *, int, p4est_refine_t, p4est_init_t);
void p4est_refine_ext(p4est_t *, int, int, p4est_refine_t, p4est_init_t, p4est_replace_t);
void p4est_coarsen(p4est_t *, int, p4est_coarsen_t, p4est_init_t);
void p4est_coarsen_ext(p4est_t *, int, int, p4est_coarsen_t, p4est_init_t, p4est_replace_t);
void p4est_balance(p4est_t *, p4est_connect_type_t, p4est_init_t);
void p4est_balance_ext(p4est_t *, p4est_connect_type_t, p4est_init_t, p4est_replace_t);
void p4est_partition(p4est_t *, int, p4est_weight_t);
p4est_gloidx_t p4est_partition_ext(p4est_t *, int, p4est_weight_t);
unsigned p4est_checksum(p4est_t *);
int p4est_is_valid(p4est_t *);
p4est_connectivity_t *p4est_connectivity_new_brick(int, int,
#ifdef P4_TO_P8
                                                   int,
#endif
                                                   int, int
#ifdef P4_TO_P8
                                                   , int
#endif
                                                   );
void p4est_connectivity_destroy(p4est_connectivity_t *);
int p4est_quadrant_is_equal(const p4est_quadrant_t *, const p4est_quadrant_t *);
int p4est_quadrant_compare(const void *, const void *);
int p4est_quadrant_compare_piggy(const void *, const void *);
int p4est_quadrant_is_ancestor(const p4est_quadrant_t *, const p4est_quadrant_t *);
int p4est_quadrant_overlaps(const p4est_quadrant_t *, const p4est_quadrant_t *);
int p4est_quadrant_is_valid(const p4est_quadrant_t *);
int p4est_quadrant_is_inside_root(const p4est_quadrant_t *);
int p4est_quadrant_child_id(const p4est_quadrant_t *);
void p4est_quadrant_parent(const p4est_quadrant_t *, p4est_quadrant_t *);
void p4est_quadrant_child(const p4est_quadrant_t *, p4est_quadrant_t *, int);
void p4est_quadrant_childrenv(const p4est_quadrant_t *, p4est_quadrant_t[]);
void p4est_quadrant_sibling(const p4est_quadrant_t *, p4est_quadrant_t *, int);
void p4est_quadrant_face_neighbor(const p4est_quadrant_t *, int, p4est_quadrant_t *);
p4est_topidx_t p4est_quadrant_face_neighbor_extra(const p4est_quadrant_t *, p4est_topidx_t, int, p4est_quadrant_t *, int *, p4est_connectivity_t *);
void p4est_quadrant_corner_neighbor(const p4est_quadrant_t *, int, p4est_quadrant_t *);
void p4est_quadrant_first_descendant(const p4est_quadrant_t *, p4est_quadrant_t *, int);
void p4est_quadrant_last_descendant(const p4est_quadrant_t *, p4est_quadrant_t *, int);
void p4est_quadrant_ancestor(const p4est_quadrant_t *, int, p4est_quadrant_t *);
void p4est_nearest_common_ancestor(const p4est_quadrant_t *, const p4est_quadrant_t *, p4est_quadrant_t *);
uint64_t p4est_quadrant_linear_id(const p4est_quadrant_t *, int);
void p4est_quadrant_set_morton(p4est_quadrant_t *, int, uint64_t);
int p4est_comm_is_owner(p4est_t *, p4est_locidx_t, const p4est_quadrant_t *, int);
int p4est_comm_find_owner(p4est_t *, p4est_locidx_t, const p4est_quadrant_t *, int);
void p4est_qcoord_to_vertex(p4est_connectivity_t *, p4est_topidx_t, p4est_qcoord_t, p4est_qcoord_t,
#ifdef P4_TO_P8
                            p4est_qcoord_t,
#endif
                            double[3]);
ssize_t p4est_find_lower_bound(sc_array_t *, const p4est_quadrant_t *, size_t);
ssize_t p4est_find_higher_bound(sc_array_t *, const p4est_quadrant_t *, size_t);
typedef struct p4est_lnodes p4est_lnodes_t;
void p4est_init(sc_log_handler_t, int);

#ifdef __cplusplus
}
#endif

#endif
