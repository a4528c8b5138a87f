// ORACLE BUILD SUPPORT (test infrastructure only).
//
// Single-process run-time for reference translation units compiled from the reference tree against the
// stand-in headers of this folder: the libsc arrays, the MPI calls (one rank), PETSc vectors (a plain array
// plus an optional ghost tail, which is always empty here) and the few p4est helpers the reference calls
// while it builds a node hierarchy, neighbours, level-set iterations and node interpolation on one process.
// Everything here follows the documented behaviour of those libraries for a communicator of size one; it
// holds no arithmetic of the level-set path.
#include <time.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

#include "stub_petsc.h"

struct ref_vec_s {
  PetscInt n_owned;   // owned entries
  PetscInt n_ghost;   // ghost tail (0 on one process)
  PetscInt bs;        // block size
  double *a;          // n_owned + n_ghost entries
  bool owns;          // false for a local form, which views its parent's array
  ref_vec_s *local;   // cached local form
};

namespace {

[[noreturn]] void fail(const char *what) {
  fprintf(stderr, "reference run-time: unsupported call %s\n", what);
  abort();
}

ref_vec_s *vec_new(PetscInt n_owned, PetscInt n_ghost, PetscInt bs) {
  ref_vec_s *v = new ref_vec_s();
  v->n_owned = n_owned;
  v->n_ghost = n_ghost;
  v->bs = bs;
  v->a = (double *)calloc((size_t)std::max<PetscInt>(1, n_owned + n_ghost), sizeof(double));
  v->owns = true;
  v->local = nullptr;
  return v;
}

}  // namespace

extern "C" {

// ------------------------------------------------------------------------------------------------ MPI
double MPI_Wtime(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec + 1e-9 * ts.tv_nsec;
}
int MPI_Comm_size(MPI_Comm, int *s) { *s = 1; return MPI_SUCCESS; }
int MPI_Comm_rank(MPI_Comm, int *r) { *r = 0; return MPI_SUCCESS; }
int MPI_Barrier(MPI_Comm) { return MPI_SUCCESS; }
int MPI_Bcast(void *, int, MPI_Datatype, int, MPI_Comm) { return MPI_SUCCESS; }

static size_t mpi_size_of(MPI_Datatype t) {
  switch (t) {
    case MPI_DOUBLE: return sizeof(double);
    case MPI_INT: return sizeof(int);
    case MPI_UNSIGNED_CHAR: case MPI_CHAR: case MPI_BYTE: case MPI_INT8_T: return 1;
    case MPI_UNSIGNED_SHORT: case MPI_SHORT: return sizeof(short);
    case MPI_UNSIGNED: return sizeof(unsigned);
    case MPI_UNSIGNED_LONG: case MPI_LONG: return sizeof(long);
    case MPI_UNSIGNED_LONG_LONG: case MPI_LONG_LONG: case MPI_INT64_T: return sizeof(long long);
    case MPI_FLOAT: return sizeof(float);
    case MPI_C_BOOL: return sizeof(bool);
    default: fail("MPI datatype");
  }
}

int MPI_Allreduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op, MPI_Comm) {
  if (s != MPI_IN_PLACE) memcpy(r, s, (size_t)n * mpi_size_of(t));
  return MPI_SUCCESS;
}
int MPI_Reduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op, int, MPI_Comm) {
  if (s != MPI_IN_PLACE) memcpy(r, s, (size_t)n * mpi_size_of(t));
  return MPI_SUCCESS;
}
int MPI_Scan(const void *s, void *r, int n, MPI_Datatype t, MPI_Op, MPI_Comm) {
  if (s != MPI_IN_PLACE) memcpy(r, s, (size_t)n * mpi_size_of(t));
  return MPI_SUCCESS;
}
int MPI_Allgather(const void *s, int n, MPI_Datatype t, void *r, int, MPI_Datatype, MPI_Comm) {
  if (s != MPI_IN_PLACE) memcpy(r, s, (size_t)n * mpi_size_of(t));
  return MPI_SUCCESS;
}
int MPI_Gather(const void *s, int n, MPI_Datatype t, void *r, int, MPI_Datatype, int, MPI_Comm) {
  if (s != MPI_IN_PLACE) memcpy(r, s, (size_t)n * mpi_size_of(t));
  return MPI_SUCCESS;
}
int MPI_Alltoall(const void *s, int n, MPI_Datatype t, void *r, int, MPI_Datatype, MPI_Comm) {
  if (s != MPI_IN_PLACE) memcpy(r, s, (size_t)n * mpi_size_of(t));
  return MPI_SUCCESS;
}
int MPI_Allgatherv(const void *s, int n, MPI_Datatype t, void *r, const int *, const int *displs, MPI_Datatype, MPI_Comm) {
  if (s != MPI_IN_PLACE) memcpy((char *)r + (size_t)displs[0] * mpi_size_of(t), s, (size_t)n * mpi_size_of(t));
  return MPI_SUCCESS;
}
int MPI_Reduce_scatter(const void *s, void *r, const int *counts, MPI_Datatype t, MPI_Op, MPI_Comm) {
  if (s != MPI_IN_PLACE) memcpy(r, s, (size_t)counts[0] * mpi_size_of(t));
  return MPI_SUCCESS;
}
int MPI_Waitall(int, MPI_Request *, MPI_Status *) { return MPI_SUCCESS; }
int MPI_Wait(MPI_Request *, MPI_Status *) { return MPI_SUCCESS; }
int MPI_Iprobe(int, int, MPI_Comm, int *flag, MPI_Status *) { *flag = 0; return MPI_SUCCESS; }

// ------------------------------------------------------------------------------------------------ libsc arrays
void sc_array_init(sc_array_t *a, size_t elem_size) {
  a->elem_size = elem_size;
  a->elem_count = 0;
  a->byte_alloc = 0;
  a->array = nullptr;
}
sc_array_t *sc_array_new(size_t elem_size) {
  sc_array_t *a = (sc_array_t *)malloc(sizeof(sc_array_t));
  sc_array_init(a, elem_size);
  return a;
}
void sc_array_resize(sc_array_t *a, size_t n) {
  const size_t need = n * a->elem_size;
  if ((ssize_t)need > a->byte_alloc) {
    size_t cap = std::max<size_t>(need, 2 * (size_t)a->byte_alloc);
    a->array = (char *)realloc(a->array, std::max<size_t>(cap, 1));
    a->byte_alloc = (ssize_t)cap;
  }
  a->elem_count = n;
}
sc_array_t *sc_array_new_size(size_t elem_size, size_t n) {
  sc_array_t *a = sc_array_new(elem_size);
  sc_array_resize(a, n);
  return a;
}
void sc_array_reset(sc_array_t *a) {
  free(a->array);
  a->array = nullptr;
  a->elem_count = 0;
  a->byte_alloc = 0;
}
void sc_array_truncate(sc_array_t *a) { a->elem_count = 0; }
void sc_array_destroy(sc_array_t *a) {
  if (!a) return;
  sc_array_reset(a);
  free(a);
}
void *sc_array_push_count(sc_array_t *a, size_t n) {
  const size_t old = a->elem_count;
  sc_array_resize(a, old + n);
  return a->array + old * a->elem_size;
}
void *sc_array_push(sc_array_t *a) { return sc_array_push_count(a, 1); }
void sc_array_sort(sc_array_t *a, int (*compar)(const void *, const void *)) {
  if (a->elem_count > 1) qsort(a->array, a->elem_count, a->elem_size, compar);
}
ssize_t sc_array_bsearch(sc_array_t *a, const void *key, int (*compar)(const void *, const void *)) {
  void *r = bsearch(key, a->array, a->elem_count, a->elem_size, compar);
  return r ? (ssize_t)(((char *)r - a->array) / (ssize_t)a->elem_size) : -1;
}

// ------------------------------------------------------------------------------------------------ p4est helpers
int p4est_quadrant_is_equal(const p4est_quadrant_t *a, const p4est_quadrant_t *b) {
  return a->level == b->level && a->x == b->x && a->y == b->y
#ifdef P4_TO_P8
         && a->z == b->z
#endif
      ;
}
int p4est_comm_find_owner(p4est_t *, p4est_locidx_t, const p4est_quadrant_t *, int guess) { return guess < 0 ? 0 : 0; }
// node coordinates are stored clamped inside the tree (ROOT_LEN -> ROOT_LEN - 1); this undoes it
void p4est_node_unclamp(p4est_quadrant_t *n) {
  if (n->x == P4EST_ROOT_LEN - 1) n->x = P4EST_ROOT_LEN;
  if (n->y == P4EST_ROOT_LEN - 1) n->y = P4EST_ROOT_LEN;
#ifdef P4_TO_P8
  if (n->z == P4EST_ROOT_LEN - 1) n->z = P4EST_ROOT_LEN;
#endif
}
void p4est_connectivity_destroy(p4est_connectivity_t *c) {
  if (!c) return;
  free(c->vertices);
  free(c->tree_to_vertex);
  free(c->tree_to_tree);
  free(c->tree_to_face);
  free(c->tree_to_corner);
  free(c->ctt_offset);
  free(c->corner_to_tree);
  free(c->corner_to_corner);
  free(c);
}

// A brick of nx x ny (x nz) trees, numbered along the Morton curve of their integer position (the order
// p4est gives a brick); each tree has its own 2^D vertices at integer coordinates (the reference rescales
// them per tree corner afterwards); face neighbours point to the adjacent tree or, on the domain boundary,
// to the tree itself. Every vertex point strictly inside the brick is a corner shared by 2^D trees, listed in
// z-order of their position around the point (entry e holds the tree on the + side of the point along the axes
// whose bit is set in e, which touches the point with its local corner 2^D-1-e); corners on the domain
// boundary connect no other tree (tree_to_corner = -1). Periodic bricks are not supported.
p4est_connectivity_t *p4est_connectivity_new_brick(int nx, int ny,
#ifdef P4_TO_P8
                                                   int nz,
#endif
                                                   int px, int py
#ifdef P4_TO_P8
                                                   , int pz
#endif
) {
#ifndef P4_TO_P8
  const int nz = 1, pz = 0;
#endif
  if (px || py || pz) fail("periodic brick");
  const int n[3] = {nx, ny, nz};
  std::vector<std::pair<uint64_t, int>> order;
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        uint64_t key = 0;
        const int c[3] = {i, j, k};
        for (int b = 0; b < 21; ++b)
          for (int a = 0; a < P4EST_DIM; ++a) key |= (uint64_t)((c[a] >> b) & 1) << (P4EST_DIM * b + a);
        order.push_back({key, (k * ny + j) * nx + i});
      }
  std::sort(order.begin(), order.end());
  p4est_connectivity_t *conn = (p4est_connectivity_t *)calloc(1, sizeof(p4est_connectivity_t));
  const int T = nx * ny * nz;
  conn->num_trees = T;
  conn->num_vertices = T * P4EST_CHILDREN;
  conn->vertices = (double *)calloc((size_t)3 * T * P4EST_CHILDREN, sizeof(double));
  conn->tree_to_vertex = (p4est_topidx_t *)malloc(sizeof(p4est_topidx_t) * T * P4EST_CHILDREN);
  conn->tree_to_tree = (p4est_topidx_t *)malloc(sizeof(p4est_topidx_t) * T * P4EST_FACES);
  conn->tree_to_face = (int8_t *)malloc((size_t)T * P4EST_FACES);
  std::vector<int> tree_of(T);
  for (int t = 0; t < T; ++t) tree_of[order[t].second] = t;
  for (int t = 0; t < T; ++t) {
    const int lin = order[t].second;
    const int ijk[3] = {lin % nx, (lin / nx) % ny, lin / (nx * ny)};
    for (int c = 0; c < P4EST_CHILDREN; ++c) {
      const int v = t * P4EST_CHILDREN + c;
      conn->tree_to_vertex[v] = v;
      for (int a = 0; a < P4EST_DIM; ++a) conn->vertices[3 * v + a] = ijk[a] + ((c >> a) & 1);
    }
    for (int f = 0; f < P4EST_FACES; ++f) {
      const int a = f / 2, s = (f & 1) ? 1 : -1;
      int nb[3] = {ijk[0], ijk[1], ijk[2]};
      nb[a] += s;
      if (nb[a] < 0 || nb[a] >= n[a]) {
        conn->tree_to_tree[t * P4EST_FACES + f] = t;
        conn->tree_to_face[t * P4EST_FACES + f] = (int8_t)f;
      } else {
        conn->tree_to_tree[t * P4EST_FACES + f] = tree_of[(nb[2] * ny + nb[1]) * nx + nb[0]];
        conn->tree_to_face[t * P4EST_FACES + f] = (int8_t)(f ^ 1);
      }
    }
  }
  // corners
  conn->tree_to_corner = (p4est_topidx_t *)malloc(sizeof(p4est_topidx_t) * T * P4EST_CHILDREN);
  for (int v = 0; v < T * P4EST_CHILDREN; ++v) conn->tree_to_corner[v] = -1;
  std::vector<p4est_topidx_t> ctt_offset(1, 0), corner_to_tree;
  std::vector<int8_t> corner_to_corner;
  for (int k = (P4EST_DIM == 3 ? 1 : 0); k < (P4EST_DIM == 3 ? nz : 1); ++k)
    for (int j = 1; j < ny; ++j)
      for (int i = 1; i < nx; ++i) {
        const p4est_topidx_t corner = (p4est_topidx_t)ctt_offset.size() - 1;
        for (int e = 0; e < P4EST_CHILDREN; ++e) {
          const int ti = i - 1 + (e & 1), tj = j - 1 + ((e >> 1) & 1), tk = (P4EST_DIM == 3) ? k - 1 + ((e >> 2) & 1) : 0;
          const int t = tree_of[(tk * ny + tj) * nx + ti];
          corner_to_tree.push_back(t);
          corner_to_corner.push_back((int8_t)(P4EST_CHILDREN - 1 - e));
          conn->tree_to_corner[t * P4EST_CHILDREN + (P4EST_CHILDREN - 1 - e)] = corner;
        }
        ctt_offset.push_back((p4est_topidx_t)corner_to_tree.size());
      }
  conn->num_corners = (p4est_topidx_t)ctt_offset.size() - 1;
  conn->ctt_offset = (p4est_topidx_t *)malloc(sizeof(p4est_topidx_t) * ctt_offset.size());
  std::copy(ctt_offset.begin(), ctt_offset.end(), conn->ctt_offset);
  conn->corner_to_tree = (p4est_topidx_t *)malloc(sizeof(p4est_topidx_t) * std::max<size_t>(1, corner_to_tree.size()));
  std::copy(corner_to_tree.begin(), corner_to_tree.end(), conn->corner_to_tree);
  conn->corner_to_corner = (int8_t *)malloc(std::max<size_t>(1, corner_to_corner.size()));
  std::copy(corner_to_corner.begin(), corner_to_corner.end(), conn->corner_to_corner);
  return conn;
}

void p4est_nodes_destroy(p4est_nodes_t *) {}
void p4est_ghost_destroy(p4est_ghost_t *) {}

// ------------------------------------------------------------------------------------------------ PETSc
PetscErrorCode PetscPrintf(MPI_Comm, const char *, ...) { return 0; }
PetscErrorCode PetscFPrintf(MPI_Comm, FILE *, const char *, ...) { return 0; }
PetscErrorCode PetscSynchronizedPrintf(MPI_Comm, const char *, ...) { return 0; }
PetscErrorCode PetscSynchronizedFPrintf(MPI_Comm, FILE *, const char *, ...) { return 0; }
PetscErrorCode PetscSynchronizedFlush(MPI_Comm, FILE *) { return 0; }

PetscErrorCode VecCreateGhost(MPI_Comm, PetscInt n, PetscInt, PetscInt nghost, const PetscInt[], Vec *v) {
  *v = vec_new(n, nghost, 1);
  return 0;
}
PetscErrorCode VecCreateGhostBlock(MPI_Comm, PetscInt bs, PetscInt n, PetscInt, PetscInt nghost, const PetscInt[], Vec *v) {
  *v = vec_new(n, nghost * bs, bs);
  return 0;
}
PetscErrorCode VecCreateMPI(MPI_Comm, PetscInt n, PetscInt, Vec *v) {
  *v = vec_new(n, 0, 1);
  return 0;
}
PetscErrorCode VecCreateSeq(MPI_Comm, PetscInt n, Vec *v) {
  *v = vec_new(n, 0, 1);
  return 0;
}
PetscErrorCode VecSetFromOptions(Vec) { return 0; }
PetscErrorCode VecSetBlockSize(Vec v, PetscInt bs) { v->bs = bs; return 0; }
PetscErrorCode VecGetBlockSize(Vec v, PetscInt *bs) { *bs = v->bs; return 0; }
PetscErrorCode VecDuplicate(Vec x, Vec *y) {
  *y = vec_new(x->n_owned, x->n_ghost, x->bs);
  return 0;
}
PetscErrorCode VecDestroy(Vec *v) {
  if (!v || !*v) return 0;
  if ((*v)->local) {
    delete (*v)->local;
  }
  if ((*v)->owns) free((*v)->a);
  delete *v;
  *v = nullptr;
  return 0;
}
PetscErrorCode VecGetSize(Vec v, PetscInt *n) { *n = v->n_owned; return 0; }
PetscErrorCode VecGetLocalSize(Vec v, PetscInt *n) { *n = v->n_owned; return 0; }
PetscErrorCode VecGetArray(Vec v, PetscScalar **a) { *a = v->a; return 0; }
PetscErrorCode VecRestoreArray(Vec, PetscScalar **a) { if (a) *a = nullptr; return 0; }
PetscErrorCode VecGetArrayRead(Vec v, const PetscScalar **a) { *a = v->a; return 0; }
PetscErrorCode VecRestoreArrayRead(Vec, const PetscScalar **a) { if (a) *a = nullptr; return 0; }
PetscErrorCode VecGhostGetLocalForm(Vec v, Vec *l) {
  if (!v->local) {
    ref_vec_s *w = new ref_vec_s(*v);
    w->n_owned = v->n_owned + v->n_ghost;
    w->n_ghost = 0;
    w->owns = false;
    w->local = nullptr;
    v->local = w;
  }
  *l = v->local;
  return 0;
}
PetscErrorCode VecGhostRestoreLocalForm(Vec, Vec *l) { *l = nullptr; return 0; }
// one process: the ghost tail is empty, so there is nothing to exchange
PetscErrorCode VecGhostUpdateBegin(Vec, InsertMode, ScatterMode) { return 0; }
PetscErrorCode VecGhostUpdateEnd(Vec, InsertMode, ScatterMode) { return 0; }
PetscErrorCode VecCopy(Vec x, Vec y) {
  memcpy(y->a, x->a, sizeof(double) * (size_t)x->n_owned);
  return 0;
}
PetscErrorCode VecSet(Vec v, PetscScalar s) {
  for (PetscInt i = 0; i < v->n_owned; ++i) v->a[i] = s;
  return 0;
}
PetscErrorCode VecScale(Vec v, PetscScalar s) {
  for (PetscInt i = 0; i < v->n_owned; ++i) v->a[i] *= s;
  return 0;
}
PetscErrorCode VecShift(Vec v, PetscScalar s) {
  for (PetscInt i = 0; i < v->n_owned; ++i) v->a[i] += s;
  return 0;
}
PetscErrorCode VecAXPY(Vec y, PetscScalar a, Vec x) {
  for (PetscInt i = 0; i < y->n_owned; ++i) y->a[i] += a * x->a[i];
  return 0;
}
PetscErrorCode VecAXPBY(Vec y, PetscScalar a, PetscScalar b, Vec x) {
  for (PetscInt i = 0; i < y->n_owned; ++i) y->a[i] = a * x->a[i] + b * y->a[i];
  return 0;
}
PetscErrorCode VecPointwiseMult(Vec w, Vec x, Vec y) {
  for (PetscInt i = 0; i < w->n_owned; ++i) w->a[i] = x->a[i] * y->a[i];
  return 0;
}
PetscErrorCode VecPointwiseMax(Vec w, Vec x, Vec y) {
  for (PetscInt i = 0; i < w->n_owned; ++i) w->a[i] = x->a[i] > y->a[i] ? x->a[i] : y->a[i];
  return 0;
}
PetscErrorCode VecPointwiseMin(Vec w, Vec x, Vec y) {
  for (PetscInt i = 0; i < w->n_owned; ++i) w->a[i] = x->a[i] < y->a[i] ? x->a[i] : y->a[i];
  return 0;
}
PetscErrorCode VecReciprocal(Vec v) {
  for (PetscInt i = 0; i < v->n_owned; ++i)
    if (v->a[i] != 0.0) v->a[i] = 1.0 / v->a[i];
  return 0;
}

}  // extern "C"
