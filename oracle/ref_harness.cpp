// ORACLE (test infrastructure only): the reference's own code, run on this machine's CPU.
//
// This file is compiled together with reference translation units taken unchanged from the reference tree
// (src/casl_math.cpp, src/my_p4est_{utils,hierarchy,cell_neighbors,node_neighbors,quad_neighbor_nodes_of_node,
// level_set,interpolation,interpolation_nodes,semi_lagrangian}.cpp, src/my_p4est_tools.c) and the stand-in
// headers of ref_stubs/ (recipe: oracle/Makefile, target `ref`; output oracle/_ref/, never committed).
// Built once for quadtrees (2D) and once with P4_TO_P8 for octrees (3D).
//
// p4est itself is not in the reference tree and is not installed, so this file plays p4est's part for one
// process: from a complete list of leaves (tree, level, integer corner, in tree-major Morton order) it
// builds the p4est_t forest, an empty ghost layer and the p4est_nodes_t node numbering (every leaf corner is
// a node owned by the lowest tree containing it, stored clamped inside that tree, nodes sorted by
// (owner tree, Morton index), as p4est_nodes_new does; src/my_p4est_nodes.h:55-63). Everything after that
// is the reference: my_p4est_brick_new, my_p4est_hierarchy_t, my_p4est_node_neighbors_t::init_neighbors
// (construct_neighbors), my_p4est_level_set_t, my_p4est_interpolation_nodes_t and
// my_p4est_semi_lagrangian_t::advect_from_n_to_np1.
#ifdef P4_TO_P8
#include <src/my_p8est_hierarchy.h>
#include <src/my_p8est_interpolation_nodes.h>
#include <src/my_p8est_level_set.h>
#include <src/my_p8est_node_neighbors.h>
#include <src/my_p8est_semi_lagrangian.h>
#include <src/my_p8est_tools.h>
#define REFH(name) refh3_##name
#else
#include <src/my_p4est_hierarchy.h>
#include <src/my_p4est_interpolation_nodes.h>
#include <src/my_p4est_level_set.h>
#include <src/my_p4est_node_neighbors.h>
#include <src/my_p4est_semi_lagrangian.h>
#include <src/my_p4est_tools.h>
#define REFH(name) refh2_##name
#endif
#include <src/casl_math.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

namespace {

constexpr int D = P4EST_DIM;
constexpr int CH = P4EST_CHILDREN;
std::string g_err;

uint64_t interleave(const int64_t *x) {
  uint64_t key = 0;
  for (int b = 0; b < 31; ++b)
    for (int a = 0; a < D; ++a) key |= (uint64_t)((x[a] >> b) & 1) << (D * b + a);
  return key;
}

// Record layout of the neighbour export (the same as the product's and the restatement's).
struct Record {
  int32_t node_000;
  int32_t nb[2 * D][1 << (D - 1)];
  double d[2 * D];
  double dt[2 * D][2 * (D - 1)];
  double inverse_d_max;
};

struct Grid {
  my_p4est_brick_t brick;
  p4est_connectivity_t *conn = nullptr;
  p4est_t p4est;
  sc_array_t trees;
  p4est_ghost_t ghost;
  p4est_nodes_t nodes;
  std::vector<p4est_gloidx_t> first_quadrant;
  std::vector<p4est_locidx_t> ghost_tree_offsets, ghost_proc_offsets, global_owned;
  std::vector<p4est_locidx_t> local_nodes;
  my_p4est_hierarchy_t *hierarchy = nullptr;
  my_p4est_node_neighbors_t *ngbd = nullptr;
  p4est_locidx_t N = 0;

  ~Grid() {
    delete ngbd;
    delete hierarchy;
    for (p4est_topidx_t t = 0; t < (p4est_topidx_t)trees.elem_count; ++t) sc_array_reset(&p4est_tree_array_index(&trees, t)->quadrants);
    sc_array_reset(&trees);
    sc_array_reset(&nodes.indep_nodes);
    if (conn) my_p4est_brick_destroy(conn, &brick);
  }
};

Grid *build(const int *n_xyz, const double *lo, const double *hi, int64_t nleaves, const int32_t *tree, const int32_t *level,
            const int32_t *xyz) {
  Grid *g = new Grid();
  int per[3] = {0, 0, 0};
  g->conn = my_p4est_brick_new(n_xyz, lo, hi, &g->brick, per);
  const p4est_topidx_t T = g->conn->num_trees;
  // forest
  memset(&g->p4est, 0, sizeof(p4est_t));
  sc_array_init(&g->trees, sizeof(p4est_tree_t));
  sc_array_resize(&g->trees, (size_t)T);
  for (p4est_topidx_t t = 0; t < T; ++t) {
    p4est_tree_t *tr = p4est_tree_array_index(&g->trees, t);
    memset(tr, 0, sizeof(p4est_tree_t));
    sc_array_init(&tr->quadrants, sizeof(p4est_quadrant_t));
  }
  for (int64_t q = 0; q < nleaves; ++q) {
    if (tree[q] < 0 || tree[q] >= T) throw std::invalid_argument("leaf tree out of range");
    p4est_tree_t *tr = p4est_tree_array_index(&g->trees, tree[q]);
    p4est_quadrant_t *Q = (p4est_quadrant_t *)sc_array_push(&tr->quadrants);
    memset(Q, 0, sizeof(p4est_quadrant_t));
    Q->x = xyz[3 * q + 0];
    Q->y = xyz[3 * q + 1];
#ifdef P4_TO_P8
    Q->z = xyz[3 * q + 2];
#endif
    Q->level = (int8_t)level[q];
    tr->quadrants_per_level[level[q]]++;
    tr->maxlevel = std::max<int8_t>(tr->maxlevel, (int8_t)level[q]);
  }
  p4est_locidx_t off = 0;
  for (p4est_topidx_t t = 0; t < T; ++t) {
    p4est_tree_t *tr = p4est_tree_array_index(&g->trees, t);
    tr->quadrants_offset = off;
    off += (p4est_locidx_t)tr->quadrants.elem_count;
  }
  g->first_quadrant = {0, (p4est_gloidx_t)nleaves};
  g->p4est.mpicomm = MPI_COMM_WORLD;
  g->p4est.mpisize = 1;
  g->p4est.mpirank = 0;
  g->p4est.first_local_tree = 0;
  g->p4est.last_local_tree = T - 1;
  g->p4est.local_num_quadrants = (p4est_locidx_t)nleaves;
  g->p4est.global_num_quadrants = nleaves;
  g->p4est.global_first_quadrant = g->first_quadrant.data();
  g->p4est.connectivity = g->conn;
  g->p4est.trees = &g->trees;
  // empty ghost layer
  memset(&g->ghost, 0, sizeof(p4est_ghost_t));
  g->ghost.mpisize = 1;
  g->ghost.num_trees = T;
  g->ghost.btype = P4EST_CONNECT_FULL;
  sc_array_init(&g->ghost.ghosts, sizeof(p4est_quadrant_t));
  sc_array_init(&g->ghost.mirrors, sizeof(p4est_quadrant_t));
  g->ghost_tree_offsets.assign((size_t)T + 1, 0);
  g->ghost_proc_offsets.assign(2, 0);
  g->ghost.tree_offsets = g->ghost_tree_offsets.data();
  g->ghost.proc_offsets = g->ghost_proc_offsets.data();
  // nodes
  std::vector<int> tijk_of((size_t)3 * T, 0);
  std::map<std::vector<int>, int> tree_at;
  {
    const double *vv = g->conn->vertices;
    for (p4est_topidx_t t = 0; t < T; ++t) {
      const p4est_topidx_t v0 = g->conn->tree_to_vertex[CH * t];
      std::vector<int> ijk(3, 0);
      for (int a = 0; a < D; ++a)
        ijk[a] = (int)std::lround((vv[3 * v0 + a] - lo[a]) / ((hi[a] - lo[a]) / n_xyz[a]));
      tree_at[ijk] = t;
      for (int a = 0; a < 3; ++a) tijk_of[(size_t)3 * t + a] = ijk[a];
    }
  }
  typedef std::pair<int32_t, uint64_t> Key;
  std::map<Key, std::vector<int64_t>> uniq;
  std::vector<Key> corner_key((size_t)nleaves * CH);
  const int64_t R = P4EST_ROOT_LEN;
  for (int64_t q = 0; q < nleaves; ++q) {
    const int64_t h = R >> level[q];
    for (int c = 0; c < CH; ++c) {
      int64_t G[3] = {0, 0, 0};
      for (int a = 0; a < D; ++a) G[a] = (int64_t)tijk_of[3 * tree[q] + a] * R + xyz[3 * q + a] + (((c >> a) & 1) ? h : 0);
      int lo_t[3] = {0, 0, 0}, hi_t[3] = {0, 0, 0};
      for (int a = 0; a < D; ++a) {
        const int64_t t = G[a] / R;
        if (G[a] == (int64_t)n_xyz[a] * R) lo_t[a] = hi_t[a] = (int)t - 1;
        else if (G[a] % R == 0 && G[a] > 0) { lo_t[a] = (int)t - 1; hi_t[a] = (int)t; }
        else lo_t[a] = hi_t[a] = (int)t;
      }
      int32_t owner = -1;
      int oijk[3] = {0, 0, 0};
      for (int k = lo_t[2]; k <= hi_t[2]; ++k)
        for (int j = lo_t[1]; j <= hi_t[1]; ++j)
          for (int i = lo_t[0]; i <= hi_t[0]; ++i) {
            const int32_t t = tree_at.at(std::vector<int>{i, j, k});
            if (owner < 0 || t < owner) { owner = t; oijk[0] = i; oijk[1] = j; oijk[2] = k; }
          }
      std::vector<int64_t> xl(3, 0);
      for (int a = 0; a < D; ++a) {
        int64_t v = G[a] - (int64_t)oijk[a] * R;
        if (v == R) v = R - 1;  // clamped inside the owner tree
        xl[a] = v;
      }
      const Key key(owner, interleave(xl.data()));
      corner_key[(size_t)q * CH + c] = key;
      uniq.emplace(key, xl);
    }
  }
  memset(&g->nodes, 0, sizeof(p4est_nodes_t));
  sc_array_init(&g->nodes.indep_nodes, sizeof(p4est_indep_t));
  sc_array_init(&g->nodes.face_hangings, sizeof(p4est_indep_t));
#ifdef P4_TO_P8
  sc_array_init(&g->nodes.edge_hangings, sizeof(p4est_indep_t));
#endif
  sc_array_init(&g->nodes.shared_indeps, sizeof(sc_array_t));
  sc_array_resize(&g->nodes.indep_nodes, uniq.size());
  std::map<Key, int32_t> index;
  int32_t k = 0;
  for (auto &kv : uniq) {
    p4est_indep_t *ni = (p4est_indep_t *)sc_array_index(&g->nodes.indep_nodes, (size_t)k);
    memset(ni, 0, sizeof(p4est_indep_t));
    ni->x = (p4est_qcoord_t)kv.second[0];
    ni->y = (p4est_qcoord_t)kv.second[1];
#ifdef P4_TO_P8
    ni->z = (p4est_qcoord_t)kv.second[2];
#endif
    ni->level = P4EST_MAXLEVEL;
    ni->p.piggy3.which_tree = kv.first.first;
    ni->p.piggy3.local_num = k;
    index[kv.first] = k++;
  }
  g->N = k;
  g->local_nodes.resize((size_t)nleaves * CH);
  for (size_t i = 0; i < g->local_nodes.size(); ++i) g->local_nodes[i] = index.at(corner_key[i]);
  g->global_owned = {g->N};
  g->nodes.num_local_quadrants = (p4est_locidx_t)nleaves;
  g->nodes.num_owned_indeps = g->N;
  g->nodes.num_owned_shared = 0;
  g->nodes.offset_owned_indeps = 0;
  g->nodes.local_nodes = g->local_nodes.data();
  g->nodes.shared_offsets = nullptr;
  g->nodes.nonlocal_ranks = nullptr;
  g->nodes.global_owned_indeps = g->global_owned.data();
  // the reference's own objects from here on
  g->hierarchy = new my_p4est_hierarchy_t(&g->p4est, &g->ghost, &g->brick);
  g->ngbd = new my_p4est_node_neighbors_t(g->hierarchy, &g->nodes);
  g->ngbd->init_neighbors();
  return g;
}

template <class F>
int guard(F &&f) {
  try {
    f();
    return 0;
  } catch (const std::exception &e) {
    g_err = e.what();
  } catch (...) {
    g_err = "unknown error";
  }
  return 1;
}

Vec node_vec(Grid *g, const double *src) {
  Vec v;
  if (VecCreateGhostNodes(&g->p4est, &g->nodes, &v)) throw std::runtime_error("VecCreateGhostNodes");
  double *p;
  VecGetArray(v, &p);
  if (src) memcpy(p, src, sizeof(double) * (size_t)g->N);
  else memset(p, 0, sizeof(double) * (size_t)g->N);
  VecRestoreArray(v, &p);
  return v;
}

void read_vec(Grid *g, Vec v, double *dst) {
  const double *p;
  VecGetArrayRead(v, &p);
  memcpy(dst, p, sizeof(double) * (size_t)g->N);
  VecRestoreArrayRead(v, &p);
}

// exposes the protected departure-point steps of the semi-Lagrangian class
class SemiLagrangian : public my_p4est_semi_lagrangian_t {
 public:
  using my_p4est_semi_lagrangian_t::my_p4est_semi_lagrangian_t;
  using my_p4est_semi_lagrangian_t::advect_from_n_to_np1;
};

}  // namespace

extern "C" {

const char *REFH(last_error)(void) { return g_err.c_str(); }
int REFH(dim)(void) { return D; }
size_t REFH(record_bytes)(void) { return sizeof(Record); }

int REFH(create)(const int *n_xyz, const double *lo, const double *hi, int64_t nleaves, const int32_t *tree, const int32_t *level,
                 const int32_t *xyz, void **out) {
  return guard([&] { *out = build(n_xyz, lo, hi, nleaves, tree, level, xyz); });
}

void REFH(destroy)(void *h) { delete static_cast<Grid *>(h); }
int64_t REFH(num_nodes)(void *h) { return static_cast<Grid *>(h)->N; }

int REFH(nodes)(void *h, int32_t *tree, int32_t *xyz) {
  return guard([&] {
    Grid *g = static_cast<Grid *>(h);
    for (p4est_locidx_t n = 0; n < g->N; ++n) {
      const p4est_indep_t *ni = (const p4est_indep_t *)sc_array_index(&g->nodes.indep_nodes, (size_t)n);
      tree[n] = ni->p.piggy3.which_tree;
      xyz[3 * n + 0] = ni->x;
      xyz[3 * n + 1] = ni->y;
#ifdef P4_TO_P8
      xyz[3 * n + 2] = ni->z;
#else
      xyz[3 * n + 2] = 0;
#endif
    }
  });
}

int REFH(local_nodes)(void *h, int32_t *out) {
  return guard([&] {
    Grid *g = static_cast<Grid *>(h);
    std::copy(g->local_nodes.begin(), g->local_nodes.end(), out);
  });
}

// node_xyz_fr_n (src/my_p4est_utils.h:1398)
int REFH(node_xyz)(void *h, double *xyz) {
  return guard([&] {
    Grid *g = static_cast<Grid *>(h);
    for (p4est_locidx_t n = 0; n < g->N; ++n) node_xyz_fr_n(n, &g->p4est, &g->nodes, xyz + (size_t)D * n);
  });
}

// is_node_{x,y,z}{m,p}Wall (src/my_p4est_utils.cpp:1815-1905): bit 2*axis+side
int REFH(wall_mask)(void *h, uint8_t *out) {
  return guard([&] {
    Grid *g = static_cast<Grid *>(h);
    for (p4est_locidx_t n = 0; n < g->N; ++n) {
      const p4est_indep_t *ni = (const p4est_indep_t *)sc_array_index(&g->nodes.indep_nodes, (size_t)n);
      uint8_t m = 0;
      m |= is_node_xmWall(&g->p4est, ni) ? 1 : 0;
      m |= is_node_xpWall(&g->p4est, ni) ? 2 : 0;
      m |= is_node_ymWall(&g->p4est, ni) ? 4 : 0;
      m |= is_node_ypWall(&g->p4est, ni) ? 8 : 0;
#ifdef P4_TO_P8
      m |= is_node_zmWall(&g->p4est, ni) ? 16 : 0;
      m |= is_node_zpWall(&g->p4est, ni) ? 32 : 0;
#endif
      out[n] = m;
    }
  });
}

// quad_neighbor_nodes_of_node_t of every node, as construct_neighbors built them
int REFH(export_qnnn)(void *h, void *out) {
  return guard([&] {
    Grid *g = static_cast<Grid *>(h);
    Record *r = static_cast<Record *>(out);
    for (p4est_locidx_t n = 0; n < g->N; ++n) {
      const quad_neighbor_nodes_of_node_t *q;
      g->ngbd->get_neighbors(n, q);
      Record &R = r[n];
      memset(&R, 0, sizeof(Record));
      R.node_000 = q->node_000;
      R.nb[0][0] = q->node_m00_mm; R.nb[0][1] = q->node_m00_pm;
      R.nb[1][0] = q->node_p00_mm; R.nb[1][1] = q->node_p00_pm;
      R.nb[2][0] = q->node_0m0_mm; R.nb[2][1] = q->node_0m0_pm;
      R.nb[3][0] = q->node_0p0_mm; R.nb[3][1] = q->node_0p0_pm;
      R.d[0] = q->d_m00; R.d[1] = q->d_p00; R.d[2] = q->d_0m0; R.d[3] = q->d_0p0;
      R.dt[0][0] = q->d_m00_m0; R.dt[0][1] = q->d_m00_p0;
      R.dt[1][0] = q->d_p00_m0; R.dt[1][1] = q->d_p00_p0;
      R.dt[2][0] = q->d_0m0_m0; R.dt[2][1] = q->d_0m0_p0;
      R.dt[3][0] = q->d_0p0_m0; R.dt[3][1] = q->d_0p0_p0;
#ifdef P4_TO_P8
      R.nb[0][2] = q->node_m00_mp; R.nb[0][3] = q->node_m00_pp;
      R.nb[1][2] = q->node_p00_mp; R.nb[1][3] = q->node_p00_pp;
      R.nb[2][2] = q->node_0m0_mp; R.nb[2][3] = q->node_0m0_pp;
      R.nb[3][2] = q->node_0p0_mp; R.nb[3][3] = q->node_0p0_pp;
      R.nb[4][0] = q->node_00m_mm; R.nb[4][1] = q->node_00m_pm; R.nb[4][2] = q->node_00m_mp; R.nb[4][3] = q->node_00m_pp;
      R.nb[5][0] = q->node_00p_mm; R.nb[5][1] = q->node_00p_pm; R.nb[5][2] = q->node_00p_mp; R.nb[5][3] = q->node_00p_pp;
      R.d[4] = q->d_00m; R.d[5] = q->d_00p;
      R.dt[0][2] = q->d_m00_0m; R.dt[0][3] = q->d_m00_0p;
      R.dt[1][2] = q->d_p00_0m; R.dt[1][3] = q->d_p00_0p;
      R.dt[2][2] = q->d_0m0_0m; R.dt[2][3] = q->d_0m0_0p;
      R.dt[3][2] = q->d_0p0_0m; R.dt[3][3] = q->d_0p0_0p;
      R.dt[4][0] = q->d_00m_m0; R.dt[4][1] = q->d_00m_p0; R.dt[4][2] = q->d_00m_0m; R.dt[4][3] = q->d_00m_0p;
      R.dt[5][0] = q->d_00p_m0; R.dt[5][1] = q->d_00p_p0; R.dt[5][2] = q->d_00p_0m; R.dt[5][3] = q->d_00p_0p;
#endif
      R.inverse_d_max = q->inverse_d_max;
    }
  });
}

// my_p4est_node_neighbors_t::second_derivatives_central (src/my_p4est_node_neighbors.cpp:1422-1640): D x N out
int REFH(second_derivatives)(void *h, const double *f, double *fdd) {
  return guard([&] {
    Grid *g = static_cast<Grid *>(h);
    Vec F = node_vec(g, f);
    Vec dd[P4EST_DIM];
    for (int a = 0; a < D; ++a) dd[a] = node_vec(g, nullptr);
    g->ngbd->second_derivatives_central(F, dd);
    for (int a = 0; a < D; ++a) {
      read_vec(g, dd[a], fdd + (size_t)a * g->N);
      VecDestroy(dd[a]);
    }
    VecDestroy(F);
  });
}

// my_p4est_node_neighbors_t::first_derivatives_central (src/my_p4est_node_neighbors.cpp:1643-1948): D x N out
int REFH(first_derivatives)(void *h, const double *f, double *fd) {
  return guard([&] {
    Grid *g = static_cast<Grid *>(h);
    Vec F = node_vec(g, f);
    Vec dd[P4EST_DIM];
    for (int a = 0; a < D; ++a) dd[a] = node_vec(g, nullptr);
    g->ngbd->first_derivatives_central(F, dd);
    for (int a = 0; a < D; ++a) {
      read_vec(g, dd[a], fd + (size_t)a * g->N);
      VecDestroy(dd[a]);
    }
    VecDestroy(F);
  });
}

// my_p4est_level_set_t::reinitialize_* (src/my_p4est_level_set.h:434-613): the public method for each
// (space, pseudo-time) order pair, with the phi_0 range [limit_low, limit_high]
int REFH(reinitialize)(void *h, double *phi, int order_space, int order_time, double limit_high, double limit_low, int iterations) {
  return guard([&] {
    Grid *g = static_cast<Grid *>(h);
    my_p4est_level_set_t ls(g->ngbd);
    Vec P = node_vec(g, phi);
    if (order_space == 2 && order_time == 2) ls.reinitialize_2nd_order_above_threshold(P, limit_low, iterations, limit_high);
    else if (order_space == 1 && order_time == 1) ls.reinitialize_1st_order_above_threshold(P, limit_low, iterations, limit_high);
    else if (order_space == 1 && order_time == 2) ls.reinitialize_2nd_order_time_1st_order_space_above_threshold(P, limit_low, iterations, limit_high);
    else if (order_space == 2 && order_time == 1) ls.reinitialize_1st_order_time_2nd_order_space_above_threshold(P, limit_low, iterations, limit_high);
    else throw std::invalid_argument("orders must be 1 or 2");
    read_vec(g, P, phi);
    VecDestroy(P);
  });
}

// reinitialize_2nd_order (src/my_p4est_level_set.h:468-472), with its default limit DBL_MAX
int REFH(reinitialize_2nd_order)(void *h, double *phi, int iterations) {
  return guard([&] {
    Grid *g = static_cast<Grid *>(h);
    my_p4est_level_set_t ls(g->ngbd);
    Vec P = node_vec(g, phi);
    ls.reinitialize_2nd_order(P, iterations);
    read_vec(g, P, phi);
    VecDestroy(P);
  });
}

// reinitialize_2nd_order_with_mask (src/my_p4est_level_set.h:487-531)
int REFH(reinitialize_with_mask)(void *h, double *phi, const double *mask, int iterations, double limit) {
  return guard([&] {
    Grid *g = static_cast<Grid *>(h);
    my_p4est_level_set_t ls(g->ngbd);
    Vec P = node_vec(g, phi), M = node_vec(g, mask);
    int masked = 0;
    for (p4est_locidx_t n = 0; n < g->N; ++n) masked += mask[n] == 0 ? 1 : 0;
    ls.reinitialize_2nd_order_with_mask(P, M, masked, iterations, limit);
    read_vec(g, P, phi);
    VecDestroy(P);
    VecDestroy(M);
  });
}

// advect_in_normal_direction(vn, phi, dt[, phi_xx...]) and (vn, vn_np1, phi, dt[, ...])
// (src/my_p4est_level_set.cpp:656-815); returns the dt the method returns
// phi_dd (D x N, optional) is in/out like the caller's Vecs: the reference overwrites them with the second
// derivatives of the first stage's result
int REFH(advect_in_normal_direction)(void *h, const double *vn, const double *vn_np1, double *phi, double dt, double *phi_dd,
                                     double *dt_out) {
  return guard([&] {
    Grid *g = static_cast<Grid *>(h);
    my_p4est_level_set_t ls(g->ngbd);
    Vec V = node_vec(g, vn), P = node_vec(g, phi);
    Vec V1 = vn_np1 ? node_vec(g, vn_np1) : nullptr;
    Vec dd[3] = {nullptr, nullptr, nullptr};
    if (phi_dd)
      for (int a = 0; a < D; ++a) dd[a] = node_vec(g, phi_dd + (size_t)a * g->N);
    double r;
    if (V1) r = ls.advect_in_normal_direction(V, V1, P, dt, DIM(dd[0], dd[1], dd[2]));
    else r = ls.advect_in_normal_direction(V, P, dt, DIM(dd[0], dd[1], dd[2]));
    if (dt_out) *dt_out = r;
    read_vec(g, P, phi);
    VecDestroy(V);
    VecDestroy(P);
    if (V1) VecDestroy(V1);
    for (int a = 0; a < D; ++a)
      if (dd[a]) {
        read_vec(g, dd[a], phi_dd + (size_t)a * g->N);
        VecDestroy(dd[a]);
      }
  });
}

// my_p4est_interpolation_nodes_t (src/my_p4est_interpolation_nodes.cpp:27-288, src/my_p4est_interpolation.cpp):
// nf fields (N each, field-major), optional second derivatives Fdd (nf x D x N), np points (D each);
// out: nf x np
int REFH(interpolate)(void *h, int method, int nf, const double *F, const double *Fdd, int64_t np, const double *xyz, double *out) {
  return guard([&] {
    Grid *g = static_cast<Grid *>(h);
    my_p4est_interpolation_nodes_t interp(g->ngbd);
    for (int64_t i = 0; i < np; ++i) interp.add_point((p4est_locidx_t)i, xyz + (size_t)D * i);
    std::vector<Vec> Fv(nf), Fx(nf), Fy(nf), Fz(nf);
    for (int k = 0; k < nf; ++k) Fv[k] = node_vec(g, F + (size_t)k * g->N);
    if (Fdd) {
      for (int k = 0; k < nf; ++k) {
        Fx[k] = node_vec(g, Fdd + ((size_t)k * D + 0) * g->N);
        Fy[k] = node_vec(g, Fdd + ((size_t)k * D + 1) * g->N);
#ifdef P4_TO_P8
        Fz[k] = node_vec(g, Fdd + ((size_t)k * D + 2) * g->N);
#endif
      }
      interp.set_input(Fv.data(), DIM(Fx.data(), Fy.data(), Fz.data()), (interpolation_method)method, (size_t)nf);
    } else {
      interp.set_input(Fv.data(), (interpolation_method)method, (size_t)nf);
    }
    std::vector<double *> outs(nf);
    for (int k = 0; k < nf; ++k) outs[k] = out + (size_t)k * np;
    interp.interpolate(outs.data());
    for (int k = 0; k < nf; ++k) {
      VecDestroy(Fv[k]);
      if (Fdd) {
        VecDestroy(Fx[k]);
        VecDestroy(Fy[k]);
#ifdef P4_TO_P8
        VecDestroy(Fz[k]);
#endif
      }
    }
  });
}

// my_p4est_semi_lagrangian_t::advect_from_n_to_np1(dt, Vec *v, Vec **vxx, phi_n, phi_xx_n, phi_np1)
// (src/my_p4est_semi_lagrangian.cpp:148-223) with the new grid equal to h: v (D x N), vxx (D x D x N: component,
// then derivative direction), phi_n, phi_xx_n (D x N); phi_np1 (N) out
int REFH(sl_advect)(void *h, double dt, const double *v, const double *vxx, const double *phi_n, const double *phi_xx, int velo_method,
                    int phi_method, double *phi_np1) {
  return guard([&] {
    Grid *g = static_cast<Grid *>(h);
    p4est_t *p = &g->p4est;
    p4est_nodes_t *nd = &g->nodes;
    p4est_ghost_t *gh = &g->ghost;
    SemiLagrangian sl(&p, &nd, &gh, g->ngbd);
    sl.set_velo_interpolation((interpolation_method)velo_method);
    sl.set_phi_interpolation((interpolation_method)phi_method);
    Vec V[P4EST_DIM], VXX_store[P4EST_DIM][P4EST_DIM], *VXX[P4EST_DIM], PXX[P4EST_DIM];
    for (int c = 0; c < D; ++c) {
      V[c] = node_vec(g, v + (size_t)c * g->N);
      for (int a = 0; a < D; ++a) VXX_store[c][a] = node_vec(g, vxx + ((size_t)c * D + a) * g->N);
      VXX[c] = VXX_store[c];
      PXX[c] = node_vec(g, phi_xx + (size_t)c * g->N);
    }
    Vec P = node_vec(g, phi_n);
    sl.advect_from_n_to_np1(dt, V, VXX, P, PXX, phi_np1);
    for (int c = 0; c < D; ++c) {
      VecDestroy(V[c]);
      VecDestroy(PXX[c]);
      for (int a = 0; a < D; ++a) VecDestroy(VXX_store[c][a]);
    }
    VecDestroy(P);
  });
}

// the two-velocity second-order step advect_from_n_to_np1(dt_nm1, dt_n, vnm1, vxx_nm1, vn, vxx_n, phi_n,
// phi_xx_n, phi_np1) (src/my_p4est_semi_lagrangian.cpp:225-319): the new grid is h_np1, velocity n and phi_n
// live on h_n, velocity n-1 on h_nm1
int REFH(sl_advect2)(void *h_np1, void *h_n, void *h_nm1, double dt_nm1, double dt_n, const double *vnm1, const double *vxx_nm1,
                     const double *vn, const double *vxx_n, const double *phi_n, const double *phi_xx, int velo_method, int phi_method,
                     double *phi_np1) {
  return guard([&] {
    Grid *g1 = static_cast<Grid *>(h_np1), *gn = static_cast<Grid *>(h_n), *gm = static_cast<Grid *>(h_nm1);
    p4est_t *p = &g1->p4est;
    p4est_nodes_t *nd = &g1->nodes;
    p4est_ghost_t *gh = &g1->ghost;
    SemiLagrangian sl(&p, &nd, &gh, gn->ngbd, gm->ngbd);
    sl.set_velo_interpolation((interpolation_method)velo_method);
    sl.set_phi_interpolation((interpolation_method)phi_method);
    Vec Vn[P4EST_DIM], Vm[P4EST_DIM], XXn[P4EST_DIM][P4EST_DIM], XXm[P4EST_DIM][P4EST_DIM], *pXXn[P4EST_DIM], *pXXm[P4EST_DIM],
        PXX[P4EST_DIM];
    for (int c = 0; c < D; ++c) {
      Vn[c] = node_vec(gn, vn + (size_t)c * gn->N);
      Vm[c] = node_vec(gm, vnm1 + (size_t)c * gm->N);
      for (int a = 0; a < D; ++a) {
        XXn[c][a] = node_vec(gn, vxx_n + ((size_t)c * D + a) * gn->N);
        XXm[c][a] = node_vec(gm, vxx_nm1 + ((size_t)c * D + a) * gm->N);
      }
      pXXn[c] = XXn[c];
      pXXm[c] = XXm[c];
      PXX[c] = node_vec(gn, phi_xx + (size_t)c * gn->N);
    }
    Vec P = node_vec(gn, phi_n);
    sl.advect_from_n_to_np1(dt_nm1, dt_n, Vm, pXXm, Vn, pXXn, P, PXX, phi_np1);
    for (int c = 0; c < D; ++c) {
      VecDestroy(Vn[c]);
      VecDestroy(Vm[c]);
      VecDestroy(PXX[c]);
      for (int a = 0; a < D; ++a) {
        VecDestroy(XXn[c][a]);
        VecDestroy(XXm[c][a]);
      }
    }
    VecDestroy(P);
  });
}

// src/casl_math.cpp:55-97 and src/casl_math.h:80-88
double REFH(interface_location)(double a, double b, double fa, double fb) { return interface_Location(a, b, fa, fb); }
double REFH(interface_location_2nd)(double a, double b, double fa, double fb, double fxxa, double fxxb) {
  return interface_Location_With_Second_Order_Derivative(a, b, fa, fb, fxxa, fxxb);
}
double REFH(minmod)(double a, double b) { return MINMOD(a, b); }

}  // extern "C"
