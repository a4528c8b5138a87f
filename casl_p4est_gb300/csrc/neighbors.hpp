// Node-neighbour stencils: the per-node record parCASL calls quad_neighbor_nodes_of_node_t
// (src/my_p4est_quad_neighbor_nodes_of_node.h:1191-1225) and the routine that fills it,
// my_p4est_node_neighbors_t::construct_neighbors (src/my_p4est_node_neighbors.cpp:114-1201).
//
// Field layout, with dir = 2*axis + side (m00, p00, 0m0, 0p0, 00m, 00p, p4est face order) and the two
// tangential axes of `axis` taken in increasing order (x: y,z; y: x,z; z: x,y):
//   nb[dir][k]  node_<dir>_{mm,pm,mp,pp}  with k = (t1 is p) + 2*(t2 is p)
//   d[dir]      d_<dir>                   (negative for the second-degree neighbour at a wall)
//   dt[dir][j]  d_<dir>_{m0,p0,0m,0p}     j = 0,1 along t1 and 2,3 along t2
// The rules restated here:
//   - the neighbouring cell on a side is the finest of the 2^(D-1) leaves touching the node on that
//     side, the first one in index order winning ties (node_neighbors.cpp:318-330 and siblings);
//   - its size gives d, its face corners give the neighbour nodes and its lower corner gives the
//     tangential offsets, zeroed below one logical unit (node_neighbors.cpp:341-362);
//   - at a wall the record instead points to the cell past the neighbour on the opposite side,
//     with d = -d_opposite - size (node_neighbors.cpp:610-700 and the five sibling blocks);
//   - inverse_d_max, including the reference's use of d_00p_0p in the 00m pair
//     (node_neighbors.cpp:1171-1187).
#pragma once
#include <math.h>

#include "forest.hpp"

namespace lsg {

template <int D>
struct Qnnn {
  int32_t node_000;
  int32_t nb[2 * D][Dim<D>::HALF];
  double d[2 * D];
  double dt[2 * D][2 * (D - 1)];
  double inverse_d_max;
};

// The construction below reads the grid through a view, so that one restatement serves the host
// builder (HostForestView over Forest) and the device builder (a view over device arrays):
//   node_tree(n), node_x(n, a) (clamped), node_unclamped(n, x), nt(a) (trees per axis), tree_ijk(t, a),
//   tree_at(ijk), tmin(t, a), tmax(t, a), find_leaf(tree, x) (-1 if none), leaf_level(q), leaf_tree(q),
//   leaf_x(q, a), local_node(q, c).
template <int D>
struct HostForestView {
  const Forest<D>& F;
  const NodeArrays& A = F.nd->host();
  int32_t node_tree(int32_t n) const { return A.node_tree[n]; }
  int32_t node_x(int32_t n, int a) const { return A.node_x[(size_t)D * n + a]; }
  void node_unclamped(int32_t n, int32_t* x) const { F.node_unclamped(n, x); }
  int nt(int a) const { return F.brick.n[a]; }
  int tree_ijk(int32_t t, int a) const { return F.brick.tree_ijk[3 * t + a]; }
  int32_t tree_at(const int* ijk) const { return F.brick.tree_at(ijk); }
  double tmin(int32_t t, int a) const { return F.brick.tmin[3 * t + a]; }
  double tmax(int32_t t, int a) const { return F.brick.tmax[3 * t + a]; }
  int32_t find_leaf(int32_t tree, const int32_t* x) const { return F.find_leaf(tree, x); }
  int leaf_level(int32_t q) const { return F.leaves[q].level; }
  int32_t leaf_tree(int32_t q) const { return F.leaves[q].tree; }
  int32_t leaf_x(int32_t q, int a) const { return F.leaves[q].x[a]; }
  int32_t local_node(int32_t q, int c) const { return A.local_nodes[(size_t)Dim<D>::CHILDREN * q + c]; }
};

// find_neighbor_cell_of_node (src/my_p4est_hierarchy.cpp:569-600): perturb the unclamped node by one
// logical unit along the diagonal direction c and return the leaf containing that point.
template <int D, class V>
LSG_HD bool find_neighbor_cell_of_node_v(const V& F, int32_t n, const int* c, int32_t& quad, int32_t& tree) {
  using DD = Dim<D>;
  int32_t xu[3] = {0, 0, 0};
  F.node_unclamped(n, xu);
  const int32_t t = F.node_tree(n);
  int ijk[3] = {0, 0, 0};
  int32_t xl[3] = {0, 0, 0};
  for (int a = 0; a < D; ++a) {
    const int64_t G = (int64_t)F.tree_ijk(t, a) * DD::ROOT_LEN + xu[a] + c[a];
    if (G < 0 || G >= (int64_t)F.nt(a) * DD::ROOT_LEN) {
      quad = -1;
      tree = -1;
      return false;
    }
    ijk[a] = (int)(G / DD::ROOT_LEN);
    xl[a] = (int32_t)(G - (int64_t)ijk[a] * DD::ROOT_LEN);
  }
  tree = F.tree_at(ijk);
  quad = F.find_leaf(tree, xl);
  return quad >= 0;
}

template <int D, class V>
LSG_HD void tangential_offsets_v(const V& F, int32_t quad, int axis, const double* cxyz, double* out) {
  using DD = Dim<D>;
  const int t1 = (axis == 0) ? 1 : 0;
  const int t2 = (axis == 2) ? 1 : 2;
  const int tan[2] = {t1, t2};
  const int32_t qt_ = F.leaf_tree(quad);
  const double qh = quadrant_len(DD::MAXLEVEL, F.leaf_level(quad)) / (double)DD::ROOT_LEN;
  for (int j = 0; j < D - 1; ++j) {
    const int t = tan[j];
    const double tmin = F.tmin(qt_, t);
    const double tmax = F.tmax(qt_, t);
    const double thr = (tmax - tmin) * ((double)1) / ((double)DD::ROOT_LEN);
    const double qt = (tmax - tmin) * (F.leaf_x(quad, t) / (double)DD::ROOT_LEN) + tmin;
    const double m0 = (fabs(cxyz[t] - qt) > thr) ? (cxyz[t] - qt) : 0.0;
    const double p0 = (fabs((tmax - tmin) * qh - m0) > thr) ? ((tmax - tmin) * qh - m0) : 0.0;
    out[2 * j + 0] = m0;
    out[2 * j + 1] = p0;
  }
}

// Corner index of a cell: bit `axis` = abit, tangential bits from k.
template <int D>
LSG_HD int face_corner(int axis, int abit, int k) {
  const int t1 = (axis == 0) ? 1 : 0;
  const int t2 = (axis == 2) ? 1 : 2;
  int c = (abit << axis) | ((k & 1) << t1);
  if (D == 3) c |= ((k >> 1) & 1) << t2;
  return c;
}

// Returns true if a stencil could not be completed (cannot happen for a complete single-process
// forest); fills q otherwise. Mirrors construct_neighbors (src/my_p4est_node_neighbors.cpp:114-1201).
template <int D, class V>
LSG_HD bool construct_neighbors_v(const V& F, int32_t n, Qnnn<D>& q) {
  using DD = Dim<D>;
  constexpr int NC = DD::CHILDREN;
  const int32_t t = F.node_tree(n);
  int32_t xu[3] = {0, 0, 0};
  F.node_unclamped(n, xu);
  double cxyz[3] = {0, 0, 0};
  for (int a = 0; a < D; ++a) {
    const double tmin = F.tmin(t, a), tmax = F.tmax(t, a);
    cxyz[a] = (tmax - tmin) * (xu[a] / (double)DD::ROOT_LEN) + tmin;
  }
  int32_t cq[NC], ct[NC];
  for (int v = 0; v < NC; ++v) {
    int c[3] = {0, 0, 0};
    for (int a = 0; a < D; ++a) c[a] = ((v >> a) & 1) ? 1 : -1;
    find_neighbor_cell_of_node_v<D>(F, n, c, cq[v], ct[v]);
  }
  auto lvl = [&](int32_t quad) -> int { return quad < 0 ? -1 : F.leaf_level(quad); };

  q.node_000 = n;
  for (int dir = 0; dir < 2 * D; ++dir) {
    q.d[dir] = 0.0;
    for (int k = 0; k < DD::HALF; ++k) q.nb[dir][k] = 0;
    for (int j = 0; j < 2 * (D - 1); ++j) q.dt[dir][j] = 0.0;
  }
  bool wall[2 * D];
  for (int dir = 0; dir < 2 * D; ++dir) {
    const int axis = dir / 2, side = dir % 2;
    int32_t best = -1;
    for (int v = 0; v < NC; ++v) {
      if (((v >> axis) & 1) != side) continue;
      if (lvl(best) < lvl(cq[v])) best = cq[v];
    }
    wall[dir] = (best < 0);
    if (wall[dir]) continue;
    const int32_t bt = F.leaf_tree(best);
    q.d[dir] = (F.tmax(bt, axis) - F.tmin(bt, axis)) * (quadrant_len(DD::MAXLEVEL, F.leaf_level(best)) / (double)DD::ROOT_LEN);
    for (int k = 0; k < DD::HALF; ++k) q.nb[dir][k] = F.local_node(best, face_corner<D>(axis, side, k));
    tangential_offsets_v<D>(F, best, axis, cxyz, q.dt[dir]);
  }
  for (int dir = 0; dir < 2 * D; ++dir) {
    if (!wall[dir]) continue;
    const int axis = dir / 2, side = dir % 2, opp = 1 - side;
    int32_t qmin = -1;
    int cvec[3] = {-1, -1, -1};
    for (int v = 0; v < NC; ++v) {
      if (((v >> axis) & 1) != opp) continue;
      if (lvl(qmin) < lvl(cq[v])) {
        qmin = cq[v];
        for (int a = 0; a < D; ++a) cvec[a] = ((v >> a) & 1) ? 1 : -1;
      }
    }
    if (qmin < 0) return true;
    int corner = 0;
    for (int a = 0; a < D; ++a) {
      const int bit = (a == axis) ? opp : (cvec[a] != 1 ? 1 : 0);
      corner |= bit << a;
    }
    const int32_t ntmp = F.local_node(qmin, corner);
    int32_t qtmp, ttmp;
    if (!find_neighbor_cell_of_node_v<D>(F, ntmp, cvec, qtmp, ttmp)) return true;
    const int32_t tt = F.leaf_tree(qtmp);
    q.d[dir] = -q.d[2 * axis + opp] - (F.tmax(tt, axis) - F.tmin(tt, axis)) *
                                          (quadrant_len(DD::MAXLEVEL, F.leaf_level(qtmp)) / (double)DD::ROOT_LEN);
    for (int k = 0; k < DD::HALF; ++k) q.nb[dir][k] = F.local_node(qtmp, face_corner<D>(axis, opp, k));
    tangential_offsets_v<D>(F, qtmp, axis, cxyz, q.dt[dir]);
  }
  // inverse_d_max (src/my_p4est_node_neighbors.cpp:1171-1187)
  double m = max2(q.d[0], q.d[1]);
  m = max3(m, q.d[2], q.d[3]);
  if (D == 3) m = max3(m, q.d[4], q.d[5]);
  m = max3(m, q.dt[0][0], q.dt[0][1]);
  m = max3(m, q.dt[1][0], q.dt[1][1]);
  m = max3(m, q.dt[2][0], q.dt[2][1]);
  m = max3(m, q.dt[3][0], q.dt[3][1]);
  if (D == 3) {
    m = max3(m, q.dt[0][2], q.dt[0][3]);
    m = max3(m, q.dt[1][2], q.dt[1][3]);
    m = max3(m, q.dt[2][2], q.dt[2][3]);
    m = max3(m, q.dt[3][2], q.dt[3][3]);
    m = max3(m, q.dt[4][0], q.dt[4][1]);
    m = max3(m, q.dt[4][2], q.dt[5][3]);
    m = max3(m, q.dt[5][0], q.dt[5][1]);
    m = max3(m, q.dt[5][2], q.dt[5][3]);
  }
  q.inverse_d_max = 1.0 / m;
  return false;
}

// host entry points over the Forest
template <int D>
inline bool find_neighbor_cell_of_node(const Forest<D>& F, int32_t n, const int* c, int32_t& quad, int32_t& tree) {
  return find_neighbor_cell_of_node_v<D>(HostForestView<D>{F}, n, c, quad, tree);
}
template <int D>
inline bool construct_neighbors(const Forest<D>& F, int32_t n, Qnnn<D>& q) {
  return construct_neighbors_v<D>(HostForestView<D>{F}, n, q);
}

// Wall flags of a node, bit dir set when the node lies on that domain face
// (is_node_xmWall ... is_node_zpWall, src/my_p4est_utils.cpp:1815-1905; non-periodic brick).
template <int D, class V>
LSG_HD unsigned wall_mask_v(const V& F, int32_t n) {
  using DD = Dim<D>;
  unsigned m = 0;
  const int32_t t = F.node_tree(n);
  for (int a = 0; a < D; ++a) {
    const int32_t v = F.node_x(n, a);
    const int ijk = F.tree_ijk(t, a);
    if (v == 0 && ijk == 0) m |= 1u << (2 * a);
    if ((v == DD::ROOT_LEN - 1 || v == DD::ROOT_LEN) && ijk == F.nt(a) - 1) m |= 1u << (2 * a + 1);
  }
  return m;
}
template <int D>
inline unsigned wall_mask(const Forest<D>& F, int32_t n) {
  return wall_mask_v<D>(HostForestView<D>{F}, n);
}

}  // namespace lsg
