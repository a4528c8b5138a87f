// ORACLE — test infrastructure only. CPU restatement of parCASL's level-set hot path, used by the
// tests, by smoke() and by the benchmark's CPU baseline as the checker of the CUDA path. Nothing in
// the product links, loads or calls this file.
//
// Plain IEEE double arithmetic compiled with -ffp-contract=off, following the reference line by line:
//   node numbering          src/my_p4est_nodes.h:55-63, src/my_p4est_nodes.c:606-627 (every leaf corner
//                           is a node, owned by the lowest tree, clamped, sorted by (tree, Morton))
//   cell tree / point location  src/my_p4est_hierarchy.h:142-152, src/my_p4est_hierarchy.cpp:264-600
//   construct_neighbors     src/my_p4est_node_neighbors.cpp:114-1201
//   walls                   src/my_p4est_utils.cpp:1815-1905
//   linear interpolation, laplace, second-derivative correction, quadratic neighbours
//                           src/my_p4est_quad_neighbor_nodes_of_node.h:214-245, 290-306, 513-524,
//                           615-635, 1514-1545; .cpp:44-298
//   interface location      src/casl_math.cpp:55-97, MINMOD src/casl_math.h:80-88
//   reinitialisation        src/my_p4est_level_set.cpp:59-557
//   normal advection        src/my_p4est_level_set.cpp:559-815
//   node interpolation      src/my_p4est_utils.cpp:367-576, src/my_p4est_interpolation_nodes.cpp:107-288,
//                           src/my_p4est_hierarchy.cpp:264-567, src/my_p4est_utils.h:2177-2187
//   semi-Lagrangian step    src/my_p4est_semi_lagrangian.cpp:148-223
// Pinned to the reference itself: oracle/_ref compiles the reference's own sources for these functions
// (ref_harness.cpp, `make ref`), and tests/test_ref_pin.py checks this restatement against them bit for bit;
// also pinned by analytic known answers and convergence orders.
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <parallel/algorithm>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

#define ORA_EPS 1e-13

namespace {

std::string g_err;

inline double MINMOD(double a, double b) {
  if (a * b <= 0) return 0;
  if ((fabs(a)) < (fabs(b))) return a;
  return b;
}
template <typename T>
inline const T& MIN(const T& a, const T& b) { return a < b ? a : b; }
template <typename T>
inline const T& MIN(const T& a, const T& b, const T& c) { return a < b ? MIN(a, c) : MIN(b, c); }
template <typename T>
inline const T& MAX(const T& a, const T& b) { return b < a ? a : b; }
template <typename T>
inline const T& MAX(const T& a, const T& b, const T& c) { return b < a ? MAX(a, c) : MAX(b, c); }

// ---------------------------------------------------------------------------------------------
// record layout identical to the product export (include/lsgpu.h, lsg_forest_export_qnnn)
template <int D>
struct Qnnn {
  int32_t node_000;
  int32_t nb[2 * D][1 << (D - 1)];
  double d[2 * D];
  double dt[2 * D][2 * (D - 1)];
  double inverse_d_max;
};

struct Leaf {
  int32_t tree, level, x[3];
};

struct Cell {  // HierarchyCell: child = -1 for a leaf
  int32_t child;
  int32_t quad;
  int32_t imin[3];
  int32_t level;
};

template <int D>
struct Grid {
  static constexpr int MAXLEVEL = (D == 2 ? 30 : 19);
  static constexpr int64_t ROOT_LEN = int64_t(1) << MAXLEVEL;
  static constexpr int CH = 1 << D;
  int n[3];
  double xyz_min[3], xyz_max[3];
  std::vector<int> tree_ijk;                 // 3 per tree
  std::vector<int> ijk_to_tree;
  std::vector<double> tv_min, tv_max;         // 3 per tree
  std::vector<Leaf> leaves;
  std::vector<std::vector<Cell>> cells;       // per tree
  // nodes
  std::vector<int32_t> node_tree;
  std::vector<int64_t> node_x;                // D per node, clamped
  std::vector<int32_t> local_nodes;
  std::vector<Qnnn<D>> qnnn;
  std::vector<uint8_t> wall;
  double tree_dim[3];

  int32_t tree_at(int i, int j, int k) const { return ijk_to_tree[(size_t)n[0] * n[1] * k + (size_t)n[0] * j + i]; }
};

uint64_t interleave(const int64_t* x, int D) {
  uint64_t key = 0;
  const int bits = (D == 2 ? 30 : 19);
  for (int b = 0; b < bits; ++b)
    for (int a = 0; a < D; ++a) key |= (uint64_t)((x[a] >> b) & 1) << (D * b + a);
  return key;
}

template <int D>
void setup_brick(Grid<D>& g, const int* n, const double* lo, const double* hi) {
  for (int a = 0; a < 3; ++a) {
    g.n[a] = a < D ? n[a] : 1;
    g.xyz_min[a] = a < D ? lo[a] : 0;
    g.xyz_max[a] = a < D ? hi[a] : 0;
  }
  const int nt = g.n[0] * g.n[1] * g.n[2];
  // trees along a Morton curve of their brick position
  std::vector<std::pair<uint64_t, int>> order;
  for (int k = 0; k < g.n[2]; ++k)
    for (int j = 0; j < g.n[1]; ++j)
      for (int i = 0; i < g.n[0]; ++i) {
        int64_t c[3] = {i, j, k};
        uint64_t key = 0;
        for (int b = 0; b < 20; ++b)
          for (int a = 0; a < 3; ++a) key |= (uint64_t)((c[a] >> b) & 1) << (3 * b + a);
        order.push_back({key, g.n[0] * g.n[1] * k + g.n[0] * j + i});
      }
  std::sort(order.begin(), order.end());
  g.tree_ijk.assign(3 * nt, 0);
  g.ijk_to_tree.assign(nt, 0);
  g.tv_min.assign(3 * nt, 0);
  g.tv_max.assign(3 * nt, 0);
  double dxyz[3];
  for (int a = 0; a < 3; ++a) dxyz[a] = (g.xyz_max[a] - g.xyz_min[a]) / (double)g.n[a];
  for (int t = 0; t < nt; ++t) {
    const int lin = order[t].second;
    const int ijk[3] = {lin % g.n[0], (lin / g.n[0]) % g.n[1], lin / (g.n[0] * g.n[1])};
    g.ijk_to_tree[lin] = t;
    for (int a = 0; a < 3; ++a) {
      g.tree_ijk[3 * t + a] = ijk[a];
      if (a < D) {
        g.tv_min[3 * t + a] = g.xyz_min[a] + (ijk[a] + 0) * dxyz[a];
        g.tv_max[3 * t + a] = g.xyz_min[a] + (ijk[a] + 1) * dxyz[a];
      }
    }
  }
  for (int a = 0; a < D; ++a) g.tree_dim[a] = (g.xyz_max[a] - g.xyz_min[a]) / g.n[a];
}

// ---- hierarchy: explicit cell tree per tree (HierarchyCell) ----------------------------------
template <int D>
void build_hierarchy(Grid<D>& g) {
  const int nt = g.n[0] * g.n[1] * g.n[2];
  g.cells.assign(nt, std::vector<Cell>());
  for (int t = 0; t < nt; ++t) {
    Cell root;
    root.child = -1;
    root.quad = -1;
    root.imin[0] = root.imin[1] = root.imin[2] = 0;
    root.level = 0;
    g.cells[t].push_back(root);
  }
  for (size_t q = 0; q < g.leaves.size(); ++q) {
    const Leaf& L = g.leaves[q];
    std::vector<Cell>& C = g.cells[L.tree];
    int ind = 0;
    while (C[ind].level < L.level) {
      if (C[ind].child < 0) {
        const int first = (int)C.size();
        const int64_t h = Grid<D>::ROOT_LEN >> (C[ind].level + 1);
        for (int c = 0; c < Grid<D>::CH; ++c) {
          Cell ch;
          ch.child = -1;
          ch.quad = -1;
          ch.level = C[ind].level + 1;
          for (int a = 0; a < 3; ++a) ch.imin[a] = C[ind].imin[a] + (a < D && ((c >> a) & 1) ? (int32_t)h : 0);
          C.push_back(ch);
        }
        C[ind].child = first;
      }
      const int64_t half = Grid<D>::ROOT_LEN >> (C[ind].level + 1);
      int c = 0;
      for (int a = 0; a < D; ++a) c |= (L.x[a] >= C[ind].imin[a] + half ? 1 : 0) << a;
      ind = C[ind].child + c;
    }
    C[ind].quad = (int32_t)q;
  }
}

// descend with logical (possibly non-integer) coordinates; returns the leaf quad index
template <int D>
int32_t descend(const Grid<D>& g, int tree, const double* s) {
  const std::vector<Cell>& C = g.cells[tree];
  int ind = 0;
  while (C[ind].child >= 0) {
    const int64_t half = Grid<D>::ROOT_LEN >> (C[ind].level + 1);
    int c = 0;
    for (int a = 0; a < D; ++a) c |= (s[a] >= (double)(C[ind].imin[a] + half) ? 1 : 0) << a;
    ind = C[ind].child + c;
  }
  return C[ind].quad;
}

// ---- nodes -----------------------------------------------------------------------------------
// Every leaf corner is a node owned by the lowest tree containing it, stored clamped inside that tree
// (ROOT_LEN -> ROOT_LEN - 1); nodes are numbered in (owner tree, Morton index) order. The corner keys are
// made in parallel, sorted and made unique, and each corner finds its node by binary search.
template <int D>
void build_nodes(Grid<D>& g) {
  typedef std::pair<int32_t, uint64_t> Key;
  const size_t nc = g.leaves.size() * Grid<D>::CH;
  std::vector<Key> corner_keys(nc);
#pragma omp parallel for schedule(static)
  for (long long qq = 0; qq < (long long)g.leaves.size(); ++qq) {
    const size_t q = (size_t)qq;
    const Leaf& L = g.leaves[q];
    const int64_t h = Grid<D>::ROOT_LEN >> L.level;
    for (int c = 0; c < Grid<D>::CH; ++c) {
      int64_t G[3] = {0, 0, 0};
      for (int a = 0; a < D; ++a) G[a] = (int64_t)g.tree_ijk[3 * L.tree + a] * Grid<D>::ROOT_LEN + L.x[a] + (((c >> a) & 1) ? h : 0);
      // owner: lowest tree id among trees containing the point
      int32_t owner = -1;
      int oijk[3] = {0, 0, 0};
      int lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
      for (int a = 0; a < D; ++a) {
        const int64_t Lx = (int64_t)g.n[a] * Grid<D>::ROOT_LEN;
        int64_t t = G[a] / Grid<D>::ROOT_LEN;
        if (G[a] == Lx) lo[a] = hi[a] = (int)t - 1;
        else if (G[a] % Grid<D>::ROOT_LEN == 0 && G[a] > 0) {
          lo[a] = (int)t - 1;
          hi[a] = (int)t;
        } else lo[a] = hi[a] = (int)t;
      }
      for (int k = lo[2]; k <= hi[2]; ++k)
        for (int j = lo[1]; j <= hi[1]; ++j)
          for (int i = lo[0]; i <= hi[0]; ++i) {
            const int32_t t = g.tree_at(i, j, k);
            if (owner < 0 || t < owner) {
              owner = t;
              oijk[0] = i;
              oijk[1] = j;
              oijk[2] = k;
            }
          }
      int64_t xl[3] = {0, 0, 0};
      for (int a = 0; a < D; ++a) {
        int64_t v = G[a] - (int64_t)oijk[a] * Grid<D>::ROOT_LEN;
        if (v == Grid<D>::ROOT_LEN) v = Grid<D>::ROOT_LEN - 1;
        xl[a] = v;
      }
      corner_keys[q * Grid<D>::CH + c] = Key(owner, interleave(xl, D));
    }
  }
  // (tree, Morton) order
  std::vector<Key> nodes(corner_keys);
  __gnu_parallel::sort(nodes.begin(), nodes.end());
  nodes.erase(std::unique(nodes.begin(), nodes.end()), nodes.end());
  const size_t N = nodes.size();
  g.node_tree.assign(N, 0);
  g.node_x.assign(N * D, 0);
  const int bits = (D == 2 ? 30 : 19);
#pragma omp parallel for schedule(static)
  for (long long ii = 0; ii < (long long)N; ++ii) {
    const size_t i = (size_t)ii;
    g.node_tree[i] = nodes[i].first;
    const uint64_t key = nodes[i].second;
    for (int a = 0; a < D; ++a) {
      int64_t v = 0;
      for (int b = 0; b < bits; ++b) v |= (int64_t)((key >> (D * b + a)) & 1) << b;
      g.node_x[i * D + a] = v;
    }
  }
  g.local_nodes.assign(nc, 0);
#pragma omp parallel for schedule(static)
  for (long long ii = 0; ii < (long long)nc; ++ii)
    g.local_nodes[(size_t)ii] = (int32_t)(std::lower_bound(nodes.begin(), nodes.end(), corner_keys[(size_t)ii]) - nodes.begin());
}

// ---- construct_neighbors ----------------------------------------------------------------------
template <int D>
void unclamped(const Grid<D>& g, int32_t n, int64_t* x) {
  for (int a = 0; a < D; ++a) {
    int64_t v = g.node_x[(size_t)n * D + a];
    x[a] = (v == Grid<D>::ROOT_LEN - 1) ? Grid<D>::ROOT_LEN : v;
  }
}

// find_neighbor_cell_of_node: perturbed node, is_node_in_domain, descend the owning tree
template <int D>
int32_t find_neighbor_cell_of_node(const Grid<D>& g, int32_t n, const int* c) {
  int64_t x[3] = {0, 0, 0};
  unclamped(g, n, x);
  const int t = g.node_tree[n];
  int ijk[3] = {0, 0, 0};
  double s[3] = {0, 0, 0};
  for (int a = 0; a < D; ++a) {
    int64_t G = (int64_t)g.tree_ijk[3 * t + a] * Grid<D>::ROOT_LEN + x[a] + c[a];
    if (G < 0 || G >= (int64_t)g.n[a] * Grid<D>::ROOT_LEN) return -1;
    ijk[a] = (int)(G / Grid<D>::ROOT_LEN);
    s[a] = (double)(G - (int64_t)ijk[a] * Grid<D>::ROOT_LEN);
  }
  return descend(g, g.tree_at(ijk[0], ijk[1], D == 3 ? ijk[2] : 0), s);
}

template <int D>
void neighbor_offsets(const Grid<D>& g, const Leaf& Q, int axis, const double* c, double* out) {
  int tan[2];
  int j = 0;
  for (int a = 0; a < D; ++a)
    if (a != axis) tan[j++] = a;
  const double qh = (double)(Grid<D>::ROOT_LEN >> Q.level) / (double)Grid<D>::ROOT_LEN;
  for (int jj = 0; jj < D - 1; ++jj) {
    const int t = tan[jj];
    const double tmin = g.tv_min[3 * Q.tree + t], tmax = g.tv_max[3 * Q.tree + t];
    const double thr = (tmax - tmin) * ((double)1) / ((double)Grid<D>::ROOT_LEN);
    const double q = (tmax - tmin) * (Q.x[t] / (double)Grid<D>::ROOT_LEN) + tmin;
    double m0 = ((fabs(c[t] - q) > thr) ? (c[t] - q) : 0.0);
    double p0 = ((fabs((tmax - tmin) * qh - m0) > thr) ? ((tmax - tmin) * qh - m0) : 0.0);
    out[2 * jj] = m0;
    out[2 * jj + 1] = p0;
  }
}

template <int D>
int corner_of(int axis, int abit, int k) {
  int tan[2];
  int j = 0;
  for (int a = 0; a < D; ++a)
    if (a != axis) tan[j++] = a;
  int c = abit << axis;
  c |= (k & 1) << tan[0];
  if (D == 3) c |= ((k >> 1) & 1) << tan[1];
  return c;
}

template <int D>
bool construct_neighbors(const Grid<D>& g, int32_t n, Qnnn<D>& q) {
  const int CH = Grid<D>::CH;
  memset(&q, 0, sizeof(q));
  int64_t xu[3] = {0, 0, 0};
  unclamped(g, n, xu);
  const int t = g.node_tree[n];
  double c[3] = {0, 0, 0};
  for (int a = 0; a < D; ++a)
    c[a] = (g.tv_max[3 * t + a] - g.tv_min[3 * t + a]) * (xu[a] / (double)Grid<D>::ROOT_LEN) + g.tv_min[3 * t + a];
  int32_t cell[8];
  for (int v = 0; v < CH; ++v) {
    int dir[3];
    for (int a = 0; a < D; ++a) dir[a] = ((v >> a) & 1) ? 1 : -1;
    cell[v] = find_neighbor_cell_of_node(g, n, dir);
  }
  auto level = [&](int32_t quad) { return quad < 0 ? -1 : g.leaves[quad].level; };
  q.node_000 = n;
  bool is_wall[6] = {false, false, false, false, false, false};
  for (int dir = 0; dir < 2 * D; ++dir) {
    const int axis = dir / 2, side = dir % 2;
    int32_t best = -1;
    for (int v = 0; v < CH; ++v)
      if (((v >> axis) & 1) == side && level(best) < level(cell[v])) best = cell[v];
    if (best < 0) {
      is_wall[dir] = true;
      continue;
    }
    const Leaf& Q = g.leaves[best];
    q.d[dir] = (g.tv_max[3 * Q.tree + axis] - g.tv_min[3 * Q.tree + axis]) * ((double)(Grid<D>::ROOT_LEN >> Q.level) / (double)Grid<D>::ROOT_LEN);
    for (int k = 0; k < (1 << (D - 1)); ++k) q.nb[dir][k] = g.local_nodes[(size_t)CH * best + corner_of<D>(axis, side, k)];
    neighbor_offsets(g, Q, axis, c, q.dt[dir]);
  }
  for (int dir = 0; dir < 2 * D; ++dir) {
    if (!is_wall[dir]) continue;
    const int axis = dir / 2, side = dir % 2, other = 1 - side;
    int32_t qmin = -1;
    int cv[3] = {-1, -1, -1};
    for (int v = 0; v < CH; ++v)
      if (((v >> axis) & 1) == other && level(qmin) < level(cell[v])) {
        qmin = cell[v];
        for (int a = 0; a < D; ++a) cv[a] = ((v >> a) & 1) ? 1 : -1;
      }
    if (qmin < 0) return true;
    int corner = 0;
    for (int a = 0; a < D; ++a) corner |= (a == axis ? other : (cv[a] != 1)) << a;
    const int32_t ntmp = g.local_nodes[(size_t)CH * qmin + corner];
    const int32_t qtmp = find_neighbor_cell_of_node(g, ntmp, cv);
    if (qtmp < 0) return true;
    const Leaf& Q = g.leaves[qtmp];
    q.d[dir] = -q.d[2 * axis + other] -
               (g.tv_max[3 * Q.tree + axis] - g.tv_min[3 * Q.tree + axis]) * ((double)(Grid<D>::ROOT_LEN >> Q.level) / (double)Grid<D>::ROOT_LEN);
    for (int k = 0; k < (1 << (D - 1)); ++k) q.nb[dir][k] = g.local_nodes[(size_t)CH * qtmp + corner_of<D>(axis, other, k)];
    neighbor_offsets(g, Q, axis, c, q.dt[dir]);
  }
  double m = MAX(q.d[0], q.d[1]);
  m = MAX(m, q.d[2], q.d[3]);
  if (D == 3) m = MAX(m, q.d[4], q.d[5]);
  m = MAX(m, q.dt[0][0], q.dt[0][1]);
  m = MAX(m, q.dt[1][0], q.dt[1][1]);
  m = MAX(m, q.dt[2][0], q.dt[2][1]);
  m = MAX(m, q.dt[3][0], q.dt[3][1]);
  if (D == 3) {
    m = MAX(m, q.dt[0][2], q.dt[0][3]);
    m = MAX(m, q.dt[1][2], q.dt[1][3]);
    m = MAX(m, q.dt[2][2], q.dt[2][3]);
    m = MAX(m, q.dt[3][2], q.dt[3][3]);
    m = MAX(m, q.dt[4][0], q.dt[4][1]);
    m = MAX(m, q.dt[4][2], q.dt[5][3]);  // d_00m_0m with d_00p_0p, as the reference
    m = MAX(m, q.dt[5][0], q.dt[5][1]);
    m = MAX(m, q.dt[5][2], q.dt[5][3]);
  }
  q.inverse_d_max = 1.0 / m;
  return false;
}

template <int D>
uint8_t wall_of(const Grid<D>& g, int32_t n) {
  uint8_t w = 0;
  const int t = g.node_tree[n];
  for (int a = 0; a < D; ++a) {
    const int64_t v = g.node_x[(size_t)n * D + a];
    if (v == 0 && g.tree_ijk[3 * t + a] == 0) w |= 1 << (2 * a);
    if ((v == Grid<D>::ROOT_LEN - 1 || v == Grid<D>::ROOT_LEN) && g.tree_ijk[3 * t + a] == g.n[a] - 1) w |= 1 << (2 * a + 1);
  }
  return w;
}

// ---- quad_neighbor_nodes_of_node_t arithmetic ---------------------------------------------------
// interpolate_linearly over the face nodes of direction dir
template <int D>
double f_linear(const Qnnn<D>& q, int dir, const double* f) {
  const double d_m0 = q.dt[dir][0], d_p0 = q.dt[dir][1];
  if (D == 2) {
    const double w_mm = d_p0, w_pm = d_m0, normalization = d_m0 + d_p0;
    return (f[q.nb[dir][1]] * w_pm + f[q.nb[dir][0]] * w_mm) / normalization;
  }
  const double d_0m = q.dt[dir][2], d_0p = q.dt[dir][3];
  const double w_mm = d_p0 * d_0p, w_pm = d_m0 * d_0p, w_mp = d_p0 * d_0m, w_pp = d_m0 * d_0m;
  const double normalization = (d_m0 + d_p0) * (d_0m + d_0p);
  return (f[q.nb[dir][3]] * w_pp + f[q.nb[dir][1]] * w_pm + f[q.nb[dir][2]] * w_mp + f[q.nb[dir][0]] * w_mm) / normalization;
}

inline double central_second_derivative(double fp, double f0, double fm, double dp, double dm) {
  return ((fp - f0) / dp + (fm - f0) / dm) * 2. / (dp + dm);
}
inline bool check_if_zero(double v) { return fabs(v) < ORA_EPS; }

template <int D>
void correct_naive_second_derivatives(const Qnnn<D>& q, double* Dxx, double* Dyy, double* Dzz) {
  const double d_m00 = q.d[0], d_p00 = q.d[1], d_0m0 = q.d[2], d_0p0 = q.d[3];
  const double m12 = q.dt[0][0] * q.dt[0][1] / d_m00 / (d_p00 + d_m00) + q.dt[1][0] * q.dt[1][1] / d_p00 / (d_p00 + d_m00);
  const double m21 = q.dt[2][0] * q.dt[2][1] / d_0m0 / (d_0p0 + d_0m0) + q.dt[3][0] * q.dt[3][1] / d_0p0 / (d_0p0 + d_0m0);
  if (D == 2) {
    if (check_if_zero(m12)) {
      if (!check_if_zero(m21)) *Dyy -= m21 * *Dxx;
    } else if (check_if_zero(m21)) {
      *Dxx -= m12 * *Dyy;
    } else {
      const double idet = 1.0 / (1.0 - m12 * m21);
      const double nDxx = *Dxx, nDyy = *Dyy;
      *Dxx = nDxx * idet - nDyy * (m12 * idet);
      *Dyy = nDyy * idet - nDxx * (m21 * idet);
    }
    return;
  }
  const double d_00m = q.d[D == 3 ? 4 : 0], d_00p = q.d[D == 3 ? 5 : 0];
  const int i4 = D == 3 ? 4 : 0, i5 = D == 3 ? 5 : 0, j2 = D == 3 ? 2 : 0, j3 = D == 3 ? 3 : 0;
  const double m13 = q.dt[0][j2] * q.dt[0][j3] / d_m00 / (d_p00 + d_m00) + q.dt[1][j2] * q.dt[1][j3] / d_p00 / (d_p00 + d_m00);
  const double m23 = q.dt[2][j2] * q.dt[2][j3] / d_0m0 / (d_0p0 + d_0m0) + q.dt[3][j2] * q.dt[3][j3] / d_0p0 / (d_0p0 + d_0m0);
  const double m31 = q.dt[i4][0] * q.dt[i4][1] / d_00m / (d_00p + d_00m) + q.dt[i5][0] * q.dt[i5][1] / d_00p / (d_00p + d_00m);
  const double m32 = q.dt[i4][j2] * q.dt[i4][j3] / d_00m / (d_00p + d_00m) + q.dt[i5][j2] * q.dt[i5][j3] / d_00p / (d_00p + d_00m);
  double &xx = *Dxx, &yy = *Dyy, &zz = *Dzz;
  if (check_if_zero(m12) && check_if_zero(m13)) {
    if (check_if_zero(m23)) {
      const bool a = !check_if_zero(m21), b = !check_if_zero(m31), c = !check_if_zero(m32);
      if (a) yy -= m21 * xx;
      if (b) zz -= m31 * xx;
      if (c) zz -= m32 * yy;
    } else if (check_if_zero(m32)) {
      const bool a = !check_if_zero(m21), b = !check_if_zero(m31);
      if (b) zz -= m31 * xx;
      yy -= m23 * zz;
      if (a) yy -= m21 * xx;
    } else {
      const double idet = 1.0 / (1.0 - m23 * m32);
      const bool a = check_if_zero(m21), b = check_if_zero(m31);
      const double ny = yy, nz = zz;
      yy = ((a ? ny : (ny - m21 * xx)) - m23 * (b ? nz : (nz - m31 * xx))) * idet;
      zz = ((b ? nz : (nz - m31 * xx)) - m32 * (a ? ny : (ny - m21 * xx))) * idet;
    }
  } else if (check_if_zero(m21) && check_if_zero(m23)) {
    if (check_if_zero(m13)) {
      const bool a = !check_if_zero(m12), b = !check_if_zero(m31), c = !check_if_zero(m32);
      if (a) xx -= m12 * yy;
      if (b) zz -= m31 * xx;
      if (c) zz -= m32 * yy;
    } else if (check_if_zero(m31)) {
      const bool a = !check_if_zero(m12), c = !check_if_zero(m32);
      if (c) zz -= m32 * yy;
      xx -= m13 * zz;
      if (a) xx -= m12 * yy;
    } else {
      const double idet = 1.0 / (1.0 - m13 * m31);
      const bool a = check_if_zero(m12), c = check_if_zero(m32);
      const double nx = xx, nz = zz;
      xx = ((a ? nx : (nx - m12 * yy)) - m13 * (c ? nz : (nz - m32 * yy))) * idet;
      zz = ((c ? nz : (nz - m32 * yy)) - m31 * (a ? nx : (nx - m12 * yy))) * idet;
    }
  } else if (check_if_zero(m31) && check_if_zero(m32)) {
    if (check_if_zero(m12)) {
      const bool a = !check_if_zero(m13), b = !check_if_zero(m21), c = !check_if_zero(m23);
      if (a) xx -= m13 * zz;
      if (b) yy -= m21 * xx;
      if (c) yy -= m23 * zz;
    } else if (check_if_zero(m21)) {
      const bool a = !check_if_zero(m13), c = !check_if_zero(m23);
      if (c) yy -= m23 * zz;
      xx -= m12 * yy;
      if (a) xx -= m13 * zz;
    } else {
      const double idet = 1.0 / (1.0 - m12 * m21);
      const bool a = check_if_zero(m13), c = check_if_zero(m23);
      const double nx = xx, ny = yy;
      xx = ((a ? nx : (nx - m13 * zz)) - m12 * (c ? ny : (ny - m23 * zz))) * idet;
      yy = ((c ? ny : (ny - m23 * zz)) - m21 * (a ? nx : (nx - m13 * zz))) * idet;
    }
  } else {
    const double idet = 1.0 / (1.0 + m12 * m23 * m31 + m13 * m21 * m32 - m12 * m21 - m13 * m31 - m23 * m32);
    const double nx = xx, ny = yy, nz = zz;
    xx = (nx * (idet * (1.0 - m23 * m32)) + ny * (idet * (m32 * m13 - m12)) + nz * (idet * (m12 * m23 - m13)));
    yy = (nx * (idet * (m31 * m23 - m21)) + ny * (idet * (1.0 - m31 * m13)) + nz * (idet * (m21 * m13 - m23)));
    zz = (nx * (idet * (m21 * m32 - m31)) + ny * (idet * (m31 * m12 - m32)) + nz * (idet * (1.0 - m21 * m12)));
  }
}

// laplace: neighbour values f_nb[2D] and corrected second derivatives fdd[D]
template <int D>
void laplace(const Qnnn<D>& q, const double* f, double* f_000, double* f_nb, double* fdd) {
  *f_000 = f[q.node_000];
  f_nb[1] = f_linear(q, 1, f);
  f_nb[0] = f_linear(q, 0, f);
  f_nb[3] = f_linear(q, 3, f);
  f_nb[2] = f_linear(q, 2, f);
  if (D == 3) {
    f_nb[D == 3 ? 5 : 0] = f_linear(q, D == 3 ? 5 : 0, f);
    f_nb[D == 3 ? 4 : 0] = f_linear(q, D == 3 ? 4 : 0, f);
  }
  for (int a = 0; a < D; ++a) fdd[a] = central_second_derivative(f_nb[2 * a + 1], *f_000, f_nb[2 * a], q.d[2 * a + 1], q.d[2 * a]);
  double dummy = 0;
  correct_naive_second_derivatives(q, &fdd[0], &fdd[1], D == 3 ? &fdd[D == 3 ? 2 : 0] : &dummy);
}

// ngbd_with_quadratic_interpolation
template <int D>
void ngbd_quadratic(const Qnnn<D>& q, const double* f, double* f_000, double* f_nb) {
  double fdd[3] = {0, 0, 0};
  laplace(q, f, f_000, f_nb, fdd);
  const double fxx = fdd[0], fyy = fdd[1], fzz = fdd[2];
  if (D == 2) {
    f_nb[0] -= (0.5 * q.dt[0][0] * q.dt[0][1] * fyy);
    f_nb[1] -= (0.5 * q.dt[1][0] * q.dt[1][1] * fyy);
    f_nb[2] -= (0.5 * q.dt[2][0] * q.dt[2][1] * fxx);
    f_nb[3] -= (0.5 * q.dt[3][0] * q.dt[3][1] * fxx);
  } else {
    const int j2 = D == 3 ? 2 : 0, j3 = D == 3 ? 3 : 0, i4 = D == 3 ? 4 : 0, i5 = D == 3 ? 5 : 0;
    f_nb[0] -= (0.5 * q.dt[0][0] * q.dt[0][1] * fyy + 0.5 * q.dt[0][j2] * q.dt[0][j3] * fzz);
    f_nb[1] -= (0.5 * q.dt[1][0] * q.dt[1][1] * fyy + 0.5 * q.dt[1][j2] * q.dt[1][j3] * fzz);
    f_nb[2] -= (0.5 * q.dt[2][0] * q.dt[2][1] * fxx + 0.5 * q.dt[2][j2] * q.dt[2][j3] * fzz);
    f_nb[3] -= (0.5 * q.dt[3][0] * q.dt[3][1] * fxx + 0.5 * q.dt[3][j2] * q.dt[3][j3] * fzz);
    f_nb[i4] -= (0.5 * q.dt[i4][0] * q.dt[i4][1] * fxx + 0.5 * q.dt[i4][j2] * q.dt[i4][j3] * fyy);
    f_nb[i5] -= (0.5 * q.dt[i5][0] * q.dt[i5][1] * fxx + 0.5 * q.dt[i5][j2] * q.dt[i5][j3] * fyy);
  }
}

double interface_Location(double a, double b, double fa, double fb) { return 0.5 * (a + b + (a - b) * (fa + fb) / (fb - fa)); }

double interface_Location_With_Second_Order_Derivative(double a, double b, double fa, double fb, double fxxa, double fxxb) {
  if (fabs(fa) < ORA_EPS) return a + ORA_EPS;
  if (fabs(fb) < ORA_EPS) return b - ORA_EPS;
  double fxx = MINMOD(fxxa, fxxb);
  double h = b - a;
  double c2 = 0.5 * fxx;
  double c1 = (fb - fa) / h;
  double c0 = 0.5 * (fb + fa) - h * h / 8 * fxx;
  double x;
  if (fabs(c2) < ORA_EPS)
    x = -c0 / c1;
  else {
    if (fb < 0)
      x = (-2 * c0) / (c1 - sqrt(c1 * c1 - 4 * c2 * c0));
    else
      x = (-2 * c0) / (c1 + sqrt(c1 * c1 - 4 * c2 * c0));
  }
  return x + 0.5 * (a + b);
}

struct Ctx {
  int dim;
  int64_t N;
  void* qnnn;        // Qnnn<D>* (owned or borrowed)
  const uint8_t* wall;
  double zero_distance_threshold;
  void* grid;        // Grid<D>* when built from leaves
  std::vector<uint8_t> wall_store;
  std::vector<char> qnnn_store;
};

// reinitialize_one_iteration (src/my_p4est_level_set.cpp:59-288)
template <int D>
void reinitialize_one_iteration(const Ctx& cx, double* phi_np1, const double* phi_0, const double* phi_n, double limit_high_,
                                double limit_low_, const double* phi_0_dd, const double* phi_n_dd, int nthreads, int64_t first = 0,
                                int64_t count = -1) {
  const Qnnn<D>* Q = static_cast<const Qnnn<D>*>(cx.qnnn);
  const bool second_order = phi_0_dd != nullptr && phi_n_dd != nullptr;
  const double zdt = cx.zero_distance_threshold;
  double big = 1.0;
  while (DBL_MAX - big == DBL_MAX) big *= 2.0;
  big = DBL_MAX - big;
  const double low = (limit_low_ < -big ? -DBL_MAX : limit_low_ - MAX(zdt, ORA_EPS * fabs(limit_low_)));
  const double high = (limit_high_ > big ? DBL_MAX : limit_high_ + MAX(zdt, ORA_EPS * fabs(limit_high_)));
  const int64_t N = cx.N;
  const int64_t end = count < 0 ? N : first + count;
#pragma omp parallel for schedule(dynamic, 1024) num_threads(nthreads)
  for (long long k = first; k < (long long)end; ++k) {
    const int64_t n = k;
    if (fabs(phi_0[n]) < zdt) {
      phi_np1[n] = 0.0;
      continue;
    }
    if (!(low < phi_0[n] && phi_0[n] < high)) {
      phi_np1[n] = phi_0[n];
      continue;
    }
    const Qnnn<D>& q = Q[n];
    double p0_000, p0_nb[6], pn_000, pn_nb[6];
    ngbd_quadratic(q, phi_0, &p0_000, p0_nb);
    ngbd_quadratic(q, phi_n, &pn_000, pn_nb);
    double s[6];
    for (int dir = 0; dir < 2 * D; ++dir) s[dir] = q.d[dir];
    double xx_000[3] = {NAN, NAN, NAN}, xx_nb[6] = {NAN, NAN, NAN, NAN, NAN, NAN};
    if (second_order) {
      for (int a = 0; a < D; ++a) {
        xx_000[a] = phi_n_dd[(size_t)a * N + n];
        xx_nb[2 * a] = f_linear(q, 2 * a, phi_n_dd + (size_t)a * N);
        xx_nb[2 * a + 1] = f_linear(q, 2 * a + 1, phi_n_dd + (size_t)a * N);
      }
    }
    bool near = false;
    for (int dir = 0; dir < 2 * D; ++dir) near = near || (p0_000 * p0_nb[dir] < 0.0);
    if (near) {
      double x0_000[3] = {NAN, NAN, NAN}, x0_nb[6] = {NAN, NAN, NAN, NAN, NAN, NAN};
      if (second_order)
        for (int a = 0; a < D; ++a) {
          x0_000[a] = phi_0_dd[(size_t)a * N + n];
          x0_nb[2 * a] = f_linear(q, 2 * a, phi_0_dd + (size_t)a * N);
          x0_nb[2 * a + 1] = f_linear(q, 2 * a + 1, phi_0_dd + (size_t)a * N);
        }
      for (int dir = 0; dir < 2 * D; ++dir) {
        if (!(p0_000 * p0_nb[dir] < 0.0)) continue;
        const int a = dir / 2;
        if (dir % 2 == 0) {
          if (second_order)
            s[dir] = -interface_Location_With_Second_Order_Derivative(-s[dir], 0.0, p0_nb[dir], p0_000, x0_nb[dir], x0_000[a]);
          else
            s[dir] = -interface_Location(-s[dir], 0.0, p0_nb[dir], p0_000);
        } else {
          if (second_order)
            s[dir] = interface_Location_With_Second_Order_Derivative(0.0, s[dir], p0_000, p0_nb[dir], x0_000[a], x0_nb[dir]);
          else
            s[dir] = interface_Location(0.0, s[dir], p0_000, p0_nb[dir]);
        }
        pn_nb[dir] = 0.0;
      }
      for (int dir = 0; dir < 2 * D; ++dir) s[dir] = MAX(s[dir], zdt);
    }
    const uint8_t w = cx.wall[n];
    for (int a = 0; a < D; ++a) {
      if (w & (1 << (2 * a))) {
        s[2 * a] = s[2 * a + 1];
        pn_nb[2 * a] = pn_nb[2 * a + 1];
        if (second_order) xx_000[a] = xx_nb[2 * a] = xx_nb[2 * a + 1] = 0.0;
      }
      if (w & (1 << (2 * a + 1))) {
        s[2 * a + 1] = s[2 * a];
        pn_nb[2 * a + 1] = pn_nb[2 * a];
        if (second_order) xx_000[a] = xx_nb[2 * a] = xx_nb[2 * a + 1] = 0.0;
      }
    }
    double gp[3], gm[3];
    for (int a = 0; a < D; ++a) {
      gp[a] = (pn_nb[2 * a + 1] - pn_000) / s[2 * a + 1];
      gm[a] = (pn_000 - pn_nb[2 * a]) / s[2 * a];
    }
    if (second_order)
      for (int a = 0; a < D; ++a) {
        xx_nb[2 * a] = MINMOD(xx_nb[2 * a], xx_000[a]);
        gm[a] += 0.5 * s[2 * a] * xx_nb[2 * a];
        xx_nb[2 * a + 1] = MINMOD(xx_nb[2 * a + 1], xx_000[a]);
        gp[a] -= 0.5 * s[2 * a + 1] * xx_nb[2 * a + 1];
      }
    const double sgn = (p0_000 > 0.0 ? 1.0 : -1.0);
    double dt = MIN(s[0], s[1]);
    dt = MIN(dt, s[2], s[3]);
    if (D == 3) dt = MIN(dt, s[4], s[5]);
    dt /= (double)D;
    for (int a = 0; a < D; ++a) {
      if (sgn * gp[a] > 0.0) gp[a] = 0.0;
      if (sgn * gm[a] < 0.0) gm[a] = 0.0;
    }
    double sum = MAX(gp[0] * gp[0], gm[0] * gm[0]) + MAX(gp[1] * gp[1], gm[1] * gm[1]);
    if (D == 3) sum = sum + MAX(gp[2] * gp[2], gm[2] * gm[2]);
    phi_np1[n] = pn_000 - dt * sgn * (sqrt(sum) - 1.);
    if (phi_0[n] * phi_np1[n] < 0.0) phi_np1[n] *= -1.0;
  }
}

template <int D>
void compute_derivatives(const Ctx& cx, const double* f, double* fdd, int nthreads, int64_t first = 0, int64_t count = -1) {
  const Qnnn<D>* Q = static_cast<const Qnnn<D>*>(cx.qnnn);
  const int64_t N = cx.N;
  const int64_t end = count < 0 ? N : first + count;
#pragma omp parallel for schedule(dynamic, 1024) num_threads(nthreads)
  for (long long n = first; n < (long long)end; ++n) {
    double f0, fnb[6], dd[3] = {0, 0, 0};
    laplace(Q[n], f, &f0, fnb, dd);
    for (int a = 0; a < D; ++a) fdd[(size_t)a * N + n] = dd[a];
  }
}

// reinitialize_within_range_of_phi_0 (src/my_p4est_level_set.cpp:290-557); with a mask
// (reinitialize_2nd_order_with_mask, src/my_p4est_level_set.h:487-525) the nodes where mask == 0 are
// left out of the update lists and copy their value into phi_np1 and phi_np2 (:377-400, :439-461).
template <int D>
void reinitialize(const Ctx& cx, double* phi, int order_space, int order_pseudotime, double hi, double lo, int iters, int nthreads,
                  const double* mask = nullptr) {
  const int64_t N = cx.N;
  std::vector<double> phi_np1(N), phi_np2(order_pseudotime > 1 ? N : 0), phi_0(phi, phi + N);
  std::vector<double> dd0, ddc;
  if (order_space > 1) {
    dd0.resize((size_t)D * N);
    ddc.resize((size_t)D * N);
    compute_derivatives<D>(cx, phi, dd0.data(), nthreads);
  }
  for (int i = 0; i < iters; ++i) {
    if (order_space > 1) compute_derivatives<D>(cx, phi, ddc.data(), nthreads);
    reinitialize_one_iteration<D>(cx, phi_np1.data(), phi_0.data(), phi, hi, lo, order_space > 1 ? dd0.data() : nullptr,
                                  order_space > 1 ? ddc.data() : nullptr, nthreads);
    if (mask)
      for (int64_t n = 0; n < N; ++n)
        if (mask[n] == 0) phi_np1[n] = phi[n];
    if (order_pseudotime > 1) {
      if (order_space > 1) compute_derivatives<D>(cx, phi_np1.data(), ddc.data(), nthreads);
      reinitialize_one_iteration<D>(cx, phi_np2.data(), phi_0.data(), phi_np1.data(), hi, lo, order_space > 1 ? dd0.data() : nullptr,
                                    order_space > 1 ? ddc.data() : nullptr, nthreads);
      if (mask)
        for (int64_t n = 0; n < N; ++n)
          if (mask[n] == 0) phi_np2[n] = phi_np1[n];
      for (int64_t n = 0; n < N; ++n) phi[n] = .5 * (phi[n] + phi_np2[n]);
    } else {
      memcpy(phi, phi_np1.data(), N * sizeof(double));
    }
  }
}

// advect_in_normal_direction_one_iteration (src/my_p4est_level_set.cpp:559-654)
template <int D>
void advect_one_iteration(const Ctx& cx, const double* vn, double dt, const double* dd, const double* phi_n, double* phi_np1,
                          int nthreads, int64_t first = 0, int64_t count = -1) {
  const Qnnn<D>* Q = static_cast<const Qnnn<D>*>(cx.qnnn);
  const int64_t N = cx.N;
  const int64_t end = count < 0 ? N : first + count;
#pragma omp parallel for schedule(dynamic, 1024) num_threads(nthreads)
  for (long long k = first; k < (long long)end; ++k) {
    const int64_t n = k;
    const Qnnn<D>& q = Q[n];
    double pn_000, pn_nb[6];
    ngbd_quadratic(q, phi_n, &pn_000, pn_nb);
    double s[6];
    for (int dir = 0; dir < 2 * D; ++dir) s[dir] = q.d[dir];
    double xx_000[3], xx_nb[6];
    for (int a = 0; a < D; ++a) {
      xx_000[a] = dd[(size_t)a * N + n];
      xx_nb[2 * a] = f_linear(q, 2 * a, dd + (size_t)a * N);
      xx_nb[2 * a + 1] = f_linear(q, 2 * a + 1, dd + (size_t)a * N);
    }
    const uint8_t w = cx.wall[n];
    for (int a = 0; a < D; ++a) {
      if (w & (1 << (2 * a))) {
        s[2 * a] = s[2 * a + 1];
        pn_nb[2 * a] = pn_nb[2 * a + 1];
        xx_000[a] = xx_nb[2 * a] = xx_nb[2 * a + 1] = 0.0;
      }
      if (w & (1 << (2 * a + 1))) {
        s[2 * a + 1] = s[2 * a];
        pn_nb[2 * a + 1] = pn_nb[2 * a];
        xx_000[a] = xx_nb[2 * a] = xx_nb[2 * a + 1] = 0.0;
      }
    }
    double gp[3], gm[3];
    for (int a = 0; a < D; ++a) {
      gp[a] = (pn_nb[2 * a + 1] - pn_000) / s[2 * a + 1];
      gm[a] = (pn_000 - pn_nb[2 * a]) / s[2 * a];
    }
    for (int a = 0; a < D; ++a) {
      xx_nb[2 * a] = MINMOD(xx_nb[2 * a], xx_000[a]);
      gm[a] += 0.5 * s[2 * a] * xx_nb[2 * a];
      xx_nb[2 * a + 1] = MINMOD(xx_nb[2 * a + 1], xx_000[a]);
      gp[a] -= 0.5 * s[2 * a + 1] * xx_nb[2 * a + 1];
    }
    const double sgn = (vn[n] > 0.0 ? +1.0 : -1.0);
    for (int a = 0; a < D; ++a) {
      if (sgn * gp[a] > 0.0) gp[a] = 0.0;
      if (sgn * gm[a] < 0.0) gm[a] = 0.0;
    }
    double sum = (gp[0] * gp[0] + gm[0] * gm[0]) + (gp[1] * gp[1] + gm[1] * gm[1]);
    if (D == 3) sum = sum + (gp[2] * gp[2] + gm[2] * gm[2]);
    phi_np1[n] = pn_000 - dt * vn[n] * (sqrt(sum));
  }
}

// advect_in_normal_direction(phi, dt, phi_xx.., vn, vn_np1) (src/my_p4est_level_set.cpp:656-725)
template <int D>
void advect_normal(const Ctx& cx, const double* vn, const double* vn_np1, double* phi, double dt, double* phi_dd, int nthreads) {
  const int64_t N = cx.N;
  std::vector<double> local_dd;
  double* dd = phi_dd;
  if (!dd) {
    local_dd.resize((size_t)D * N);
    dd = local_dd.data();
    compute_derivatives<D>(cx, phi, dd, nthreads);
  }
  std::vector<double> phi_n(phi, phi + N), phi_np2(N);
  advect_one_iteration<D>(cx, vn, dt, dd, phi_n.data(), phi, nthreads);
  compute_derivatives<D>(cx, phi, dd, nthreads);
  advect_one_iteration<D>(cx, vn_np1 ? vn_np1 : vn, dt, dd, phi, phi_np2.data(), nthreads);
  for (int64_t n = 0; n < N; ++n) phi[n] = 0.5 * (phi_n[n] + phi_np2[n]);
}

// ---- first derivatives, normals, curvature -------------------------------------------------------
// central_derivative and dd_correction_weight_to_naive_first_derivative
// (src/my_p4est_quad_neighbor_nodes_of_node.h:186-199)
inline double central_derivative(double fp, double f0, double fm, double dp, double dm) {
  return ((fp - f0) * dm / dp + (f0 - fm) * dp / dm) / (dp + dm);
}
inline double dd_correction_weight(double d_m, double d_p, double d_m_m, double d_m_p, double d_p_m, double d_p_p) {
  return 0.5 * (d_p_m * d_p_p * d_m / d_p - d_m_m * d_m_p * d_p / d_m) / (d_m + d_p);
}

// gradient / d{x,y,z}_central of f at the node: naive central differences of the linearly
// interpolated neighbours, corrected by the second derivatives along the tangential axes where
// the neighbours are offset (correct_naive_first_derivatives, .cpp:575-640); only the components
// in `which` (bit a) are computed
template <int D>
void gradient(const Qnnn<D>& q, const double* f, double* g, int which = 7) {
  double f0 = f[q.node_000], fnb[6];
  for (int dir = 0; dir < 2 * D; ++dir) fnb[dir] = f_linear(q, dir, f);
  double w[3][2] = {{0, 0}, {0, 0}, {0, 0}};
  bool need[3][2] = {{false, false}, {false, false}, {false, false}};
  bool any = false;
  for (int a = 0; a < D; ++a) {
    if (!((which >> a) & 1)) continue;
    g[a] = central_derivative(fnb[2 * a + 1], f0, fnb[2 * a], q.d[2 * a + 1], q.d[2 * a]);
    for (int j = 0; j < D - 1; ++j) {
      w[a][j] = dd_correction_weight(q.d[2 * a], q.d[2 * a + 1], q.dt[2 * a][2 * j], q.dt[2 * a][2 * j + 1], q.dt[2 * a + 1][2 * j],
                                     q.dt[2 * a + 1][2 * j + 1]);
      need[a][j] = !check_if_zero(w[a][j] * q.inverse_d_max);
      any = any || need[a][j];
    }
  }
  if (!any) return;
  double fdd[3] = {0, 0, 0}, fz, fn[6];
  laplace(q, f, &fz, fn, fdd);
  for (int a = 0; a < D; ++a) {
    if (!((which >> a) & 1)) continue;
    for (int j = 0; j < D - 1; ++j) {
      const int b = (j == 0) ? (a == 0 ? 1 : 0) : (a == 2 ? 1 : 2);  // j-th axis other than a
      if (need[a][j]) g[a] -= fdd[b] * w[a][j];
    }
  }
}

// first_derivatives_central (src/my_p4est_node_neighbors.cpp:1643-1948): D x N
template <int D>
void first_derivatives(const Ctx& cx, const double* f, double* out, int nthreads) {
  const Qnnn<D>* Q = static_cast<const Qnnn<D>*>(cx.qnnn);
  const int64_t N = cx.N;
#pragma omp parallel for schedule(dynamic, 1024) num_threads(nthreads)
  for (long long n = 0; n < (long long)N; ++n) {
    double g[3] = {0, 0, 0};
    gradient<D>(Q[n], f, g);
    for (int a = 0; a < D; ++a) out[(size_t)a * N + n] = g[a];
  }
}

// normalisation of compute_normals (src/my_p4est_utils.cpp:1717-1739), in place on D x N
template <int D>
void normalize(int64_t N, double* g) {
  for (int64_t n = 0; n < N; ++n) {
    double s = g[n] * g[n] + g[N + n] * g[N + n];
    if (D == 3) s = s + g[2 * N + n] * g[2 * N + n];
    const double abs = sqrt(s);
    for (int a = 0; a < D; ++a) g[(size_t)a * N + n] = abs < ORA_EPS ? 0 : g[(size_t)a * N + n] / abs;
  }
}

// compute_mean_curvature(neighbors, normals, kappa) (src/my_p4est_utils.cpp:1658-1696):
// dx_central(nx) + dy_central(ny) [+ dz_central(nz)]
template <int D>
void curvature_from_normals(const Ctx& cx, const double* nrm, double* kappa, int nthreads) {
  const Qnnn<D>* Q = static_cast<const Qnnn<D>*>(cx.qnnn);
  const int64_t N = cx.N;
#pragma omp parallel for schedule(dynamic, 1024) num_threads(nthreads)
  for (long long n = 0; n < (long long)N; ++n) {
    double gx[3], gy[3], gz[3];
    gradient<D>(Q[n], nrm, gx, 1);
    gradient<D>(Q[n], nrm + N, gy, 2);
    double k = gx[0] + gy[1];
    if (D == 3) {
      gradient<D>(Q[n], nrm + 2 * N, gz, 4);
      k = k + gz[2];
    }
    kappa[n] = k;
  }
}

// compute_normals_and_mean_curvature (src/my_p4est_utils.cpp:2776-2802) with get_curvature from the
// gradient and phi (src/my_p4est_quad_neighbor_nodes_of_node.h:2051-2087)
template <int D>
void normals_and_curvature(const Ctx& cx, const double* phi, double* nrm, double* kappa, int nthreads) {
  const Qnnn<D>* Q = static_cast<const Qnnn<D>*>(cx.qnnn);
  const int64_t N = cx.N;
  first_derivatives<D>(cx, phi, nrm, nthreads);
#pragma omp parallel for schedule(dynamic, 1024) num_threads(nthreads)
  for (long long n = 0; n < (long long)N; ++n) {
    const double dx = nrm[n], dy = nrm[N + n], dz = D == 3 ? nrm[2 * N + n] : 0.0;
    double mag = 0.0;
    mag += dx * dx;
    mag += dy * dy;
    if (D == 3) mag += dz * dz;
    mag = sqrt(mag);
    if (!(mag > ORA_EPS)) {
      kappa[n] = 0.0;
      continue;
    }
    double dd[3] = {0, 0, 0}, f0, fn[6];
    laplace(Q[n], phi, &f0, fn, dd);
    double gx[3], gy[3];
    gradient<D>(Q[n], nrm, gx, D == 3 ? 6 : 2);  // d/dy (and d/dz) of phi_x
    const double dxy = gx[1];
    if (D == 3) {
      gradient<D>(Q[n], nrm + N, gy, 4);  // d/dz of phi_y
      const double dxz = gx[2], dyz = gy[2];
      kappa[n] = ((dd[1] + dd[2]) * (dx * dx) + (dd[0] + dd[2]) * (dy * dy) + (dd[0] + dd[1]) * (dz * dz) -
                  2.0 * (dx * dy * dxy + dx * dz * dxz + dy * dz * dyz)) /
                 (mag * mag * mag);
    } else {
      kappa[n] = ((dd[1]) * (dx * dx) + (dd[0]) * (dy * dy) - 2.0 * (dx * dy * dxy)) / (mag * mag * mag);
    }
  }
  normalize<D>(N, nrm);
}

// ---- extension over the interface -------------------------------------------------------------
// edge-diagonal neighbours of get_all_neighbors (src/my_p4est_node_neighbors.cpp:2001-2153), in the
// order 3D: m0m p0m m0p p0p 0mm 0pm 0mp 0pp mm0 pm0 mp0 pp0; 2D: mm0 pm0 mp0 pp0; -1 if absent
template <int D>
void corner_neighbors(const Grid<D>& g, int32_t n, int32_t* out) {
  auto cell = [&](int i, int j, int k) {
    const int c[3] = {i, j, k};
    return find_neighbor_cell_of_node(g, n, c);
  };
  auto node = [&](int32_t quad, int v) { return g.local_nodes[(size_t)quad * Grid<D>::CH + v]; };
  if (D == 2) {
    const int32_t mm = cell(-1, -1, 0), pm = cell(1, -1, 0), mp = cell(-1, 1, 0), pp = cell(1, 1, 0);
    out[0] = mm >= 0 ? node(mm, 0) : -1;
    out[1] = pm >= 0 ? node(pm, 1) : -1;
    out[2] = mp >= 0 ? node(mp, 2) : -1;
    out[3] = pp >= 0 ? node(pp, 3) : -1;
    return;
  }
  const int32_t mmm = cell(-1, -1, -1), mpm = cell(-1, 1, -1), pmm = cell(1, -1, -1), ppm = cell(1, 1, -1);
  const int32_t mmp = cell(-1, -1, 1), mpp = cell(-1, 1, 1), pmp = cell(1, -1, 1), ppp = cell(1, 1, 1);
  auto pick = [&](int32_t q1, int v1, int32_t q2, int v2) { return q1 >= 0 ? node(q1, v1) : (q2 >= 0 ? node(q2, v2) : -1); };
  out[0] = pick(mmm, 2, mpm, 0);   // m0m
  out[1] = pick(pmm, 3, ppm, 1);   // p0m
  out[2] = pick(mmp, 6, mpp, 4);   // m0p
  out[3] = pick(pmp, 7, ppp, 5);   // p0p
  out[4] = pick(mmm, 1, pmm, 0);   // 0mm
  out[5] = pick(mpm, 3, ppm, 2);   // 0pm
  out[6] = pick(mmp, 5, pmp, 4);   // 0mp
  out[7] = pick(mpp, 7, ppp, 6);   // 0pp
  out[8] = pick(mmm, 4, mmp, 0);   // mm0
  out[9] = pick(pmm, 5, pmp, 1);   // pm0
  out[10] = pick(mpm, 6, mpp, 2);  // mp0
  out[11] = pick(ppm, 7, ppp, 3);  // pp0
}

// is_stencil_in_negative_domain (src/my_p4est_quad_neighbor_nodes_of_node.h:2492-2530): the node and
// every face node with a nonzero interpolation weight below -EPS
template <int D>
bool stencil_negative(const Qnnn<D>& q, const double* f) {
  if (!(f[q.node_000] < -ORA_EPS)) return false;
  for (int dir = 0; dir < 2 * D; ++dir) {
    const double m0 = q.dt[dir][0], p0 = q.dt[dir][1];
    const double m1 = D == 3 ? q.dt[dir][2] : 0.0, p1 = D == 3 ? q.dt[dir][3] : 0.0;
    for (int k = 0; k < Grid<D>::CH / 2; ++k) {
      // face node k: bit 0 along the first tangential axis (m/p), bit 1 along the second
      bool zero;
      if (D == 2)
        zero = (k == 0) ? fabs(p0) < ORA_EPS : fabs(m0) < ORA_EPS;
      else {
        const bool a = (k & 1) ? fabs(m0) < ORA_EPS : fabs(p0) < ORA_EPS;
        const bool b = (k & 2) ? fabs(m1) < ORA_EPS : fabs(p1) < ORA_EPS;
        zero = a || b;
      }
      if (!(f[q.nb[dir][k]] < -ORA_EPS || zero)) return false;
    }
  }
  return true;
}

// d_a of f at the node (dx_central, dy_central, dz_central)
template <int D>
double dcentral(const Qnnn<D>& q, const double* f, int a) {
  double g[3] = {0, 0, 0};
  gradient<D>(q, f, g, 1 << a);
  return g[a];
}

// one marching iteration of a field v along the normals, upwind first-order one-sided differences:
// tmp = v - dt (n . grad v - src) on the nodes selected by `on`
template <int D>
double march(const Qnnn<D>& q, const double* v, const double* const* nrm, int64_t n, double src, bool with_src) {
  const double dt = (D == 3 ? MIN(MIN(fabs(q.d[0]), fabs(q.d[2]), fabs(q.d[4])), MIN(fabs(q.d[1]), fabs(q.d[3]), fabs(q.d[5])))
                            : MIN(MIN(fabs(q.d[0]), fabs(q.d[2])), MIN(fabs(q.d[1]), fabs(q.d[3])))) /
                    double(D);
  double g[3];
  for (int a = 0; a < D; ++a)
    g[a] = nrm[a][n] > 0 ? (v[n] - f_linear(q, 2 * a, v)) / q.d[2 * a] : (f_linear(q, 2 * a + 1, v) - v[n]) / q.d[2 * a + 1];
  double s = nrm[0][n] * g[0] + nrm[1][n] * g[1];
  if (D == 3) s = s + nrm[2][n] * g[2];
  return with_src ? v[n] - dt * (s - src) : v[n] - dt * s;
}

// extend_Over_Interface_TVD(phi, q, iterations, order, band_use, band_extend, normal, mask) with no
// boundary conditions, no initial guesses and one-step extrapolation (src/my_p4est_level_set.cpp:969-1764)
template <int D>
void extend_over_interface(const Ctx& cx, const double* phi, const double* mask_in, double* q, int iterations, int order,
                           double band_use, double band_extend, const double* normal_in, int nthreads, bool nonzero_guess = false,
                           double* q_n_io = nullptr, double* q_nn_io = nullptr) {
  const Grid<D>& g = *static_cast<const Grid<D>*>(cx.grid);
  const Qnnn<D>* Q = static_cast<const Qnnn<D>*>(cx.qnnn);
  const int64_t N = cx.N;
  const double* mask = mask_in ? mask_in : phi;
  if (band_use > 0) band_use = -band_use;
  std::vector<double> nstore;
  const double* nrm_flat = normal_in;
  if (!nrm_flat) {
    nstore.resize((size_t)D * N);
    first_derivatives<D>(cx, phi, nstore.data(), nthreads);
    normalize<D>(N, nstore.data());
    nrm_flat = nstore.data();
  }
  const double* nrm[3] = {nrm_flat, nrm_flat + N, D == 3 ? nrm_flat + 2 * N : nrm_flat};
  // q_n / q_nn given by the caller: their values start the marching where no value is computed (the
  // reference then works in the caller's vectors); otherwise fresh zero vectors
  std::vector<double> qn((size_t)N, 0.0), qnn((size_t)N, 0.0), bqn((size_t)N, 0.0), bqnn((size_t)N, 0.0);
  if (q_n_io) qn.assign(q_n_io, q_n_io + N);
  if (q_nn_io) qnn.assign(q_nn_io, q_nn_io + N);
  std::vector<double> qx((size_t)D * N, 0.0);
  if (order >= 1) {
#pragma omp parallel for schedule(dynamic, 1024) num_threads(nthreads)
    for (long long n = 0; n < (long long)N; ++n) {
      if (phi[n] > band_use) {
        if (stencil_negative<D>(Q[n], mask)) {
          bqn[n] = -1;
          double gq[3] = {0, 0, 0};
          gradient<D>(Q[n], q, gq);
          for (int a = 0; a < D; ++a) qx[(size_t)a * N + n] = gq[a];
          double s = nrm[0][n] * qx[n] + nrm[1][n] * qx[N + n];
          if (D == 3) s = s + nrm[2][n] * qx[2 * N + n];
          qn[n] = s;
        } else {
          bqn[n] = 1;
          if (nonzero_guess) {
            double s = nrm[0][n] * dcentral<D>(Q[n], q, 0) + nrm[1][n] * dcentral<D>(Q[n], q, 1);
            if (D == 3) s = s + nrm[2][n] * dcentral<D>(Q[n], q, 2);
            qn[n] = s;
          } else if (!q_n_io) {
            qn[n] = 0;
          }
          for (int a = 0; a < D; ++a) qx[(size_t)a * N + n] = 0;
        }
      } else {
        bqn[n] = -1;
        qn[n] = 0;
        for (int a = 0; a < D; ++a) qx[(size_t)a * N + n] = 0;
      }
    }
  }
  if (order == 2) {
#pragma omp parallel for schedule(dynamic, 1024) num_threads(nthreads)
    for (long long n = 0; n < (long long)N; ++n) {
      const Qnnn<D>& qq = Q[n];
      if (!(phi[n] > band_use)) {
        bqnn[n] = -1;
        qnn[n] = 0;
        continue;
      }
      bqnn[n] = 1;
      if (!stencil_negative<D>(qq, mask)) {
        if (nonzero_guess) {
          double s = nrm[0][n] * dcentral<D>(qq, qn.data(), 0) + nrm[1][n] * dcentral<D>(qq, qn.data(), 1);
          if (D == 3) s = s + nrm[2][n] * dcentral<D>(qq, qn.data(), 2);
          qnn[n] = s;
        } else if (!q_nn_io) {
          qnn[n] = 0;
        }
        continue;
      }
      double Qxy = 0, Qyz = 0, Qzx = 0;
      const double* qxa = qx.data();
      const double* qya = qx.data() + N;
      const double* qza = D == 3 ? qx.data() + 2 * N : qx.data();
      if (stencil_negative<D>(qq, bqn.data())) {
        bqnn[n] = -1;
        Qxy = .5 * (dcentral<D>(qq, qya, 0) + dcentral<D>(qq, qxa, 1));
        if (D == 3) {
          Qyz = .5 * (dcentral<D>(qq, qza, 1) + dcentral<D>(qq, qya, 2));
          Qzx = .5 * (dcentral<D>(qq, qxa, 2) + dcentral<D>(qq, qza, 0));
        }
      } else {
        int32_t nb[12];
        corner_neighbors<D>(g, (int32_t)n, nb);
        const int cnt = D == 3 ? 12 : 4;
        bool exist = true, neg = true;
        for (int k = 0; k < cnt; ++k) exist = exist && nb[k] >= 0;
        if (exist) {
          for (int k = 0; k < cnt; ++k) neg = neg && mask[nb[k]] < 0;
          if (neg) {
            const int mm0 = D == 3 ? 8 : 0, pm0 = D == 3 ? 9 : 1, mp0 = D == 3 ? 10 : 2, pp0 = D == 3 ? 11 : 3;
            Qxy = (q[nb[pp0]] + q[nb[mm0]] - q[nb[mp0]] - q[nb[pm0]]) / (qq.d[0] + qq.d[1]) / (qq.d[2] + qq.d[3]);
            if (D == 3) {
              Qyz = (q[nb[7]] + q[nb[4]] - q[nb[6]] - q[nb[5]]) / (qq.d[2] + qq.d[3]) / (qq.d[D == 3 ? 4 : 0] + qq.d[D == 3 ? 5 : 0]);
              Qzx = (q[nb[3]] + q[nb[0]] - q[nb[1]] - q[nb[2]]) / (qq.d[D == 3 ? 4 : 0] + qq.d[D == 3 ? 5 : 0]) / (qq.d[0] + qq.d[1]);
            }
            bqnn[n] = -1;
          }
        }
      }
      if (bqnn[n] < 0) {
        // dxx_central etc.: central second differences of the quadratically corrected neighbours
        // (x_ngbd_with_quadratic_interpolation, src/my_p4est_quad_neighbor_nodes_of_node.cpp:365-390)
        double fz, fn[6], dd[3] = {0, 0, 0};
        ngbd_quadratic(qq, q, &fz, fn);
        for (int a = 0; a < D; ++a) dd[a] = central_second_derivative(fn[2 * a + 1], fz, fn[2 * a], qq.d[2 * a + 1], qq.d[2 * a]);
        const double Qx = qx[n], Qy = qx[N + n];
        const double Nx = nrm[0][n], Ny = nrm[1][n];
        const double Nxx = dcentral<D>(qq, nrm[0], 0), Nyx = dcentral<D>(qq, nrm[1], 0);
        const double Nxy = dcentral<D>(qq, nrm[0], 1), Nyy = dcentral<D>(qq, nrm[1], 1);
        if (D == 3) {
          const double Qz = qx[2 * N + n], Nz = nrm[2][n];
          const double Nzx = dcentral<D>(qq, nrm[2], 0), Nzy = dcentral<D>(qq, nrm[2], 1);
          const double Nxz = dcentral<D>(qq, nrm[0], 2), Nyz = dcentral<D>(qq, nrm[1], 2), Nzz = dcentral<D>(qq, nrm[2], 2);
          qnn[n] = Nx * (Nx * dd[0] + 2. * Ny * Qxy + Qx * Nxx + Qy * Nyx + Qz * Nzx) +
                   Ny * (Ny * dd[1] + 2. * Nz * Qyz + Qx * Nxy + Qy * Nyy + Qz * Nzy) +
                   Nz * (Nz * dd[2] + 2. * Nx * Qzx + Qx * Nxz + Qy * Nyz + Qz * Nzz);
        } else {
          qnn[n] = Nx * (Nx * dd[0] + 2. * Ny * Qxy + Qx * Nxx + Qy * Nyx) + Ny * (Ny * dd[1] + Qx * Nxy + Qy * Nyy);
        }
      } else {
        if (!q_nn_io) qnn[n] = 0;  // left as it was (a fresh vector is zero)
      }
    }
  }
  // marching loops: qnn, then qn, then q (ping-pong; nodes not marched keep their value)
  auto run = [&](std::vector<double>& v, const std::vector<double>& b, const double* src, bool with_src) {
    std::vector<double> tmp(v);
    for (int it = 0; it < iterations; ++it) {
#pragma omp parallel for schedule(dynamic, 1024) num_threads(nthreads)
      for (long long n = 0; n < (long long)N; ++n)
        if (b[n] > 0 && phi[n] < band_extend) tmp[n] = march<D>(Q[n], v.data(), nrm, n, src ? src[n] : 0.0, with_src);
      v.swap(tmp);
    }
  };
  if (order == 2) run(qnn, bqnn, nullptr, false);
  if (order >= 1) run(qn, bqn, order == 2 ? qnn.data() : nullptr, true);
  std::vector<double> cur(q, q + N), tmp(q, q + N), qdd((size_t)D * N);
  for (int it = 0; it < iterations; ++it) {
    compute_derivatives<D>(cx, cur.data(), qdd.data(), nthreads);
#pragma omp parallel for schedule(dynamic, 1024) num_threads(nthreads)
    for (long long n = 0; n < (long long)N; ++n) {
      if (!(mask[n] > -ORA_EPS && phi[n] < band_extend)) continue;
      const Qnnn<D>& qq = Q[n];
      const double dt = (D == 3 ? MIN(MIN(fabs(qq.d[0]), fabs(qq.d[2]), fabs(qq.d[4])), MIN(fabs(qq.d[1]), fabs(qq.d[3]), fabs(qq.d[5])))
                                : MIN(MIN(fabs(qq.d[0]), fabs(qq.d[2])), MIN(fabs(qq.d[1]), fabs(qq.d[3])))) /
                        double(D);
      double gq[3];
      for (int a = 0; a < D; ++a)
        gq[a] = nrm[a][n] > 0 ? (cur[n] - f_linear(qq, 2 * a, cur.data())) / qq.d[2 * a]
                              : (f_linear(qq, 2 * a + 1, cur.data()) - cur[n]) / qq.d[2 * a + 1];
      if (order == 2) {
        for (int a = 0; a < D; ++a) {
          const double* qaa = qdd.data() + (size_t)a * N;
          double qm = f_linear(qq, 2 * a, qaa), qp = f_linear(qq, 2 * a + 1, qaa);
          qm = qaa[n] * qm < 0 ? 0 : (fabs(qaa[n]) < fabs(qm) ? qaa[n] : qm);
          qp = qaa[n] * qp < 0 ? 0 : (fabs(qaa[n]) < fabs(qp) ? qaa[n] : qp);
          if (nrm[a][n] < 0) gq[a] -= .5 * qq.d[2 * a + 1] * qp;
          else gq[a] += .5 * qq.d[2 * a] * qm;
        }
      }
      double sum = nrm[0][n] * gq[0] + nrm[1][n] * gq[1];
      if (D == 3) sum = sum + nrm[2][n] * gq[2];
      const double change = dt * (sum - (order >= 1 ? qn[n] : 0));
      tmp[n] = cur[n] - change;
    }
    cur.swap(tmp);
  }
  memcpy(q, cur.data(), (size_t)N * sizeof(double));
  if (q_n_io && order >= 1) memcpy(q_n_io, qn.data(), (size_t)N * sizeof(double));
  if (q_nn_io && order == 2) memcpy(q_nn_io, qnn.data(), (size_t)N * sizeof(double));
}

// ---- node interpolation ------------------------------------------------------------------------
// PI of src/casl_math.h:15
const double ORA_PI = 3.1415926535897932384626433832795;

// clip_in_domain, non-periodic (src/my_p4est_utils.h:2177-2187)
template <int D>
void clip_in_domain(const Grid<D>& g, double* xyz) {
  for (int a = 0; a < D; ++a)
    if (xyz[a] < g.xyz_min[a] || xyz[a] > g.xyz_max[a]) xyz[a] = MAX(g.xyz_min[a], MIN(g.xyz_max[a], xyz[a]));
}

// find_smallest_quadrant_containing_point + find_quadrant_containing_point, single process,
// non-periodic (src/my_p4est_hierarchy.cpp:264-425, 427-567): the point is scaled to tree units,
// pushed qeps inside the brick, and probed at +-threshold along every axis on which it lies within
// threshold of a cell face; the first probe landing in the finest leaf wins.
template <int D>
int32_t find_smallest_quadrant(const Grid<D>& g, const double* xyz) {
  const double ROOT = (double)Grid<D>::ROOT_LEN;
  const double qeps = (double)1 / ROOT;
  const double threshold = 0.01 * (double)1;
  double xs[3] = {0, 0, 0};
  for (int a = 0; a < D; ++a) {
    xs[a] = xyz[a] - g.xyz_min[a];
    xs[a] /= (g.xyz_max[a] - g.xyz_min[a]) / g.n[a];
  }
  int tr[3] = {0, 0, 0};
  for (int a = 0; a < D; ++a) {
    xs[a] = MAX(qeps, MIN(xs[a], g.n[a] - qeps));
    tr[a] = (int)floor(xs[a]);
  }
  double c[3] = {0, 0, 0};
  bool face[3] = {false, false, false};
  for (int a = 0; a < D; ++a) {
    c[a] = (xs[a] - tr[a]) * ROOT;
    face[a] = (fabs(c[a] - floor(c[a])) < threshold || fabs(ceil(c[a]) - c[a]) < threshold);
  }
  int best = -1, best_level = -1;
  for (int i = (face[0] ? -1 : 0); i < 2; i += 2)
    for (int j = (face[1] ? -1 : 0); j < 2; j += 2)
      for (int k = (D == 3 && face[2] ? -1 : 0); k < (D == 3 ? 2 : 1); k += 2) {
        const int off[3] = {i, j, k};
        double s[3];
        int t[3] = {tr[0], tr[1], tr[2]};
        for (int a = 0; a < D; ++a) {
          s[a] = (off[a] == 0 ? c[a] : c[a] + off[a] * threshold);
          if (s[a] < 0 || s[a] >= ROOT) {
            const int slide = (int)floor(s[a] / ROOT);
            s[a] -= ((double)slide) * ROOT;
            t[a] = tr[a] + slide;
          }
          if (t[a] < 0 || t[a] >= g.n[a]) throw std::runtime_error("oracle: point outside the brick");
        }
        const int tt = g.tree_at(t[0], t[1], D == 3 ? t[2] : 0);
        const int32_t q = descend(g, tt, s);
        if (g.leaves[q].level > best_level) {
          best_level = g.leaves[q].level;
          best = q;
        }
      }
  return best;
}

enum { ORA_LINEAR = 0, ORA_QUADRATIC, ORA_QUADRATIC_NON_OSCILLATORY, ORA_QUADRATIC_NON_OSCILLATORY_CONTINUOUS_V1,
       ORA_QUADRATIC_NON_OSCILLATORY_CONTINUOUS_V2 };

// get_local_interpolation_weights (src/my_p4est_utils.cpp:367-408)
template <int D>
void local_weights(const Grid<D>& g, const Leaf& Q, const double* xyz_global, double* lw, double* sdw) {
  const double* tmin = &g.tv_min[3 * Q.tree];
  const double* tmax = &g.tv_max[3 * Q.tree];
  const double qh = (double)(Grid<D>::ROOT_LEN >> Q.level) / (double)Grid<D>::ROOT_LEN;
  double xyz[3], d_[3][2];
  for (int a = 0; a < D; ++a) {
    const double qmin = (double)Q.x[a] / (double)Grid<D>::ROOT_LEN;
    xyz[a] = (xyz_global[a] - tmin[a]) / (tmax[a] - tmin[a]);
    xyz[a] = (xyz[a] - qmin) / qh;
    d_[a][0] = 1.0 - xyz[a];
    d_[a][1] = xyz[a];
  }
  for (int c = 0; c < Grid<D>::CH; ++c) {
    const int ix = c & 1, iy = (c >> 1) & 1, iz = (c >> 2) & 1;
    lw[c] = (D == 3 ? d_[0][ix] * d_[1][iy] * d_[2][iz] : d_[0][ix] * d_[1][iy]);
  }
  for (int a = 0; a < D; ++a) {
    const double h = (tmax[a] - tmin[a]) * qh;
    sdw[a] = h * h * d_[a][0] * d_[a][1];
  }
}

// the five interpolation kernels (src/my_p4est_utils.cpp:410-576), one function value f[CH] with
// second derivatives fdd[CH][D] at the corners
template <int D>
double interpolate_local(int method, const double* lw, const double* sdw, const double* f, const double (*fdd)[3]) {
  const int CH = Grid<D>::CH;
  double r = 0.0;
  if (method == ORA_LINEAR) {
    for (int j = 0; j < CH; ++j) r += +f[j] * lw[j];
    return r;
  }
  double dd[3] = {0, 0, 0};
  if (method == ORA_QUADRATIC) {
    for (int j = 0; j < CH; ++j) {
      for (int i = 0; i < D; ++i) dd[i] = ((j == 0) ? 0.0 : dd[i]) + fdd[j][i] * lw[j];
      r += f[j] * lw[j];
    }
  } else if (method == ORA_QUADRATIC_NON_OSCILLATORY) {
    for (int j = 0; j < CH; ++j) {
      for (int i = 0; i < D; ++i) dd[i] = (j == 0 ? fdd[j][i] : MINMOD(dd[i], fdd[j][i]));
      r += f[j] * lw[j];
    }
  } else if (method == ORA_QUADRATIC_NON_OSCILLATORY_CONTINUOUS_V1) {
    for (int i = 0; i < D; ++i) {
      dd[i] = 0.0;
      for (int jm = 0; jm < CH; ++jm) {
        if ((jm >> i) & 1) continue;
        const int jp = jm | (1 << i);
        dd[i] += MINMOD(fdd[jm][i], fdd[jp][i]) * (lw[jm] + lw[jp]);
      }
    }
    for (int j = 0; j < CH; ++j) r += f[j] * lw[j];
  } else {
    for (int i = 0; i < D; ++i) {
      double m = 0, p = 0;
      for (int jm = 0; jm < CH; ++jm) {
        if ((jm >> i) & 1) continue;
        const int jp = jm | (1 << i);
        m += fdd[jm][i] * (lw[jm] + lw[jp]);
        p += fdd[jp][i] * (lw[jm] + lw[jp]);
      }
      dd[i] = MINMOD(m, p);
    }
    for (int j = 0; j < CH; ++j) r += f[j] * lw[j];
  }
  if (D == 3)
    r -= 0.5 * (sdw[0] * dd[0] + sdw[1] * dd[1] + sdw[2] * dd[2]);
  else
    r -= 0.5 * (sdw[0] * dd[0] + sdw[1] * dd[1]);
  return r;
}

// my_p4est_interpolation_t::add_point_general + my_p4est_interpolation_nodes_t::interpolate
// (src/my_p4est_interpolation.cpp:68-124, src/my_p4est_interpolation_nodes.cpp:107-288): the leaf
// is located from the clipped point, the weights use the point as given. F: nf fields of N values;
// Fdd: nf x D x N second derivatives (required unless method is linear). out: nf x np.
template <int D>
void interpolate_points(const Ctx& cx, int method, int nf, const double* F, const double* Fdd, int64_t np, const double* xyz,
                        double* out, int nthreads) {
  const Grid<D>& g = *static_cast<const Grid<D>*>(cx.grid);
  const int64_t N = cx.N;
  const int CH = Grid<D>::CH;
#pragma omp parallel for schedule(static) num_threads(nthreads)
  for (int64_t p = 0; p < np; ++p) {
    double xc[3] = {0, 0, 0};
    for (int a = 0; a < D; ++a) xc[a] = xyz[p * D + a];
    clip_in_domain(g, xc);
    const int32_t q = find_smallest_quadrant(g, xc);
    double lw[8], sdw[3];
    local_weights(g, g.leaves[q], xyz + p * D, lw, sdw);
    for (int k = 0; k < nf; ++k) {
      double f[8], fdd[8][3];
      for (int j = 0; j < CH; ++j) {
        const int32_t node = g.local_nodes[(size_t)q * CH + j];
        f[j] = F[(size_t)k * N + node];
        for (int a = 0; a < D; ++a) fdd[j][a] = (method == ORA_LINEAR ? 0.0 : Fdd[((size_t)k * D + a) * N + node]);
      }
      out[(size_t)k * np + p] = interpolate_local<D>(method, lw, sdw, f, fdd);
    }
  }
}

// single-vortex velocity of examples/level_set_advection/main_2d.cpp:116-181, scaled by s (the
// example's sign, or cos(pi t/T))
template <int D>
void vortex(const double* x, double s, double* v) {
  if (D == 3) {
    v[0] = 2.0 * (sin(ORA_PI * x[0]) * sin(ORA_PI * x[0])) * sin(2 * ORA_PI * x[1]) * sin(2 * ORA_PI * x[2]) * s;
    v[1] = -(sin(ORA_PI * x[1]) * sin(ORA_PI * x[1])) * sin(2 * ORA_PI * x[0]) * sin(2 * ORA_PI * x[2]) * s;
    v[2] = -(sin(ORA_PI * x[2]) * sin(ORA_PI * x[2])) * sin(2 * ORA_PI * x[0]) * sin(2 * ORA_PI * x[1]) * s;
  } else {
    v[0] = -(sin(ORA_PI * x[0]) * sin(ORA_PI * x[0])) * sin(2 * ORA_PI * x[1]) * s;
    v[1] = (sin(ORA_PI * x[1]) * sin(ORA_PI * x[1])) * sin(2 * ORA_PI * x[0]) * s;
  }
}

// second derivatives of nf fields (nf x D x N) when the caller gives none
template <int D>
const double* derivatives_of(const Ctx& cx, int nf, const double* F, const double* Fdd, std::vector<double>& store, int nthreads) {
  if (Fdd) return Fdd;
  store.resize((size_t)nf * D * cx.N);
  for (int k = 0; k < nf; ++k) compute_derivatives<D>(cx, F + (size_t)k * cx.N, store.data() + (size_t)k * D * cx.N, nthreads);
  return store.data();
}

// advect_from_n_to_np1(dt, Vec* v, Vec** vxx, phi_n, phi_xx_n, phi_np1) (src/my_p4est_semi_lagrangian.cpp:148-223):
// v at the new nodes, v at x* = x - dt/2 v (clipped), phi at x_d = x - dt v* (clipped).
template <int D>
void sl_advect(const Ctx& cx, int64_t np, const double* xyz, double dt, const double* v, const double* vdd, const double* phi,
               const double* phi_dd, int velo_method, int phi_method, double* phi_np1, int nthreads) {
  const Grid<D>& g = *static_cast<const Grid<D>*>(cx.grid);
  std::vector<double> vs, ps;
  vdd = (velo_method == ORA_LINEAR ? nullptr : derivatives_of<D>(cx, D, v, vdd, vs, nthreads));
  phi_dd = (phi_method == ORA_LINEAR ? nullptr : derivatives_of<D>(cx, 1, phi, phi_dd, ps, nthreads));
  std::vector<double> vt((size_t)D * np), pts((size_t)D * np);
  interpolate_points<D>(cx, velo_method, D, v, vdd, np, xyz, vt.data(), nthreads);
  for (int64_t n = 0; n < np; ++n) {
    double x[3];
    for (int a = 0; a < D; ++a) x[a] = xyz[n * D + a];
    for (int a = 0; a < D; ++a) x[a] -= 0.5 * dt * vt[(size_t)a * np + n];
    clip_in_domain(g, x);
    for (int a = 0; a < D; ++a) pts[n * D + a] = x[a];
  }
  interpolate_points<D>(cx, velo_method, D, v, vdd, np, pts.data(), vt.data(), nthreads);
  for (int64_t n = 0; n < np; ++n) {
    double x[3];
    for (int a = 0; a < D; ++a) x[a] = xyz[n * D + a];
    for (int a = 0; a < D; ++a) x[a] -= dt * vt[(size_t)a * np + n];
    clip_in_domain(g, x);
    for (int a = 0; a < D; ++a) pts[n * D + a] = x[a];
  }
  interpolate_points<D>(cx, phi_method, 1, phi, phi_dd, np, pts.data(), phi_np1, nthreads);
}

// advect_from_n_to_np1(dt_nm1, dt_n, vnm1, vxx_nm1, vn, vxx_n, phi_n, phi_xx_n, phi_np1)
// (src/my_p4est_semi_lagrangian.cpp:225-319): v_n at the new nodes (quadratic), v_n and v_nm1 at
// x* = x - dt_n/2 v_n (clipped) with velo_method on grids n and n-1, phi_n at x_d = x - dt_n v* (clipped),
// v* = (1 + .5 dt_n/dt_nm1) v_n(x*) - .5 dt_n/dt_nm1 v_nm1(x*).
template <int D>
void sl_advect2(const Ctx& cn, const Ctx& cm, int64_t np, const double* xyz, double dt_nm1, double dt_n, const double* vnm1,
                const double* vnm1_dd, const double* vn, const double* vn_dd, const double* phi, const double* phi_dd, int velo_method,
                int phi_method, double* phi_np1, int nthreads) {
  const Grid<D>& g = *static_cast<const Grid<D>*>(cn.grid);
  std::vector<double> vs, ms, ps;
  vn_dd = derivatives_of<D>(cn, D, vn, vn_dd, vs, nthreads);
  vnm1_dd = (velo_method == ORA_LINEAR ? nullptr : derivatives_of<D>(cm, D, vnm1, vnm1_dd, ms, nthreads));
  phi_dd = (phi_method == ORA_LINEAR ? nullptr : derivatives_of<D>(cn, 1, phi, phi_dd, ps, nthreads));
  std::vector<double> vt_n((size_t)D * np), vt_nm1((size_t)D * np), pts((size_t)D * np);
  interpolate_points<D>(cn, ORA_QUADRATIC, D, vn, vn_dd, np, xyz, vt_n.data(), nthreads);
  for (int64_t n = 0; n < np; ++n) {
    double x[3];
    for (int a = 0; a < D; ++a) x[a] = xyz[n * D + a];
    for (int a = 0; a < D; ++a) x[a] -= .5 * dt_n * vt_n[(size_t)a * np + n];
    clip_in_domain(g, x);
    for (int a = 0; a < D; ++a) pts[n * D + a] = x[a];
  }
  interpolate_points<D>(cm, velo_method, D, vnm1, vnm1_dd, np, pts.data(), vt_nm1.data(), nthreads);
  interpolate_points<D>(cn, velo_method, D, vn, velo_method == ORA_LINEAR ? nullptr : vn_dd, np, pts.data(), vt_n.data(), nthreads);
  for (int64_t n = 0; n < np; ++n) {
    double v_star[3], x[3];
    for (int a = 0; a < D; ++a)
      v_star[a] = (1.0 + .5 * dt_n / dt_nm1) * vt_n[(size_t)a * np + n] - 0.5 * dt_n / dt_nm1 * vt_nm1[(size_t)a * np + n];
    for (int a = 0; a < D; ++a) x[a] = xyz[n * D + a];
    for (int a = 0; a < D; ++a) x[a] -= dt_n * v_star[a];
    clip_in_domain(g, x);
    for (int a = 0; a < D; ++a) pts[n * D + a] = x[a];
  }
  interpolate_points<D>(cn, phi_method, 1, phi, phi_dd, np, pts.data(), phi_np1, nthreads);
}

// advect_from_n_to_np1(dt, const CF** v, phi_n, phi_xx_n, phi_np1) (src/my_p4est_semi_lagrangian.cpp:108-146)
// with the single-vortex velocity scaled by vscale.
template <int D>
void sl_advect_vortex(const Ctx& cx, int64_t np, const double* xyz, double dt, double vscale, const double* phi, const double* phi_dd,
                      int phi_method, double* phi_np1, int nthreads) {
  const Grid<D>& g = *static_cast<const Grid<D>*>(cx.grid);
  std::vector<double> ps;
  phi_dd = (phi_method == ORA_LINEAR ? nullptr : derivatives_of<D>(cx, 1, phi, phi_dd, ps, nthreads));
  std::vector<double> pts((size_t)D * np);
  for (int64_t n = 0; n < np; ++n) {
    double x[3], xs[3], v[3];
    for (int a = 0; a < D; ++a) x[a] = xyz[n * D + a];
    vortex<D>(x, vscale, v);
    for (int a = 0; a < D; ++a) xs[a] = x[a] - 0.5 * dt * v[a];
    clip_in_domain(g, xs);
    vortex<D>(xs, vscale, v);
    for (int a = 0; a < D; ++a) pts[n * D + a] = x[a] - dt * v[a];
    clip_in_domain(g, &pts[n * D]);
  }
  interpolate_points<D>(cx, phi_method, 1, phi, phi_dd, np, pts.data(), phi_np1, nthreads);
}

// ---- extension from the interface to the whole domain -----------------------------------------
// pascalTriangle / smoothstep (src/my_p4est_utils.cpp:3350-3370)
double pascal_triangle(int a, int b) {
  double result = 1.;
  for (int i = 0; i < b; ++i) result *= double(a - i) / double(i + 1);
  return result;
}
double smoothstep(int N, double x) {
  if (x <= 0) return 0;
  if (x >= 1) return 1;
  double result = 0;
  for (int n = 0; n <= N; ++n) result += pascal_triangle(-N - 1, n) * pascal_triangle(2 * N + 1, N - n) * pow(x, N + n + 1);
  return result;
}

// node_x_fr_n(n, p4est, nodes) (src/my_p4est_utils.h:1346-1370)
template <int D>
void node_coordinates(const Grid<D>& g, int32_t n, double* xyz) {
  const int t = g.node_tree[n];
  for (int a = 0; a < D; ++a) {
    const int64_t v = g.node_x[(size_t)n * D + a];
    const double r = v == Grid<D>::ROOT_LEN - 1 ? 1.0 : static_cast<double>(v) / static_cast<double>(Grid<D>::ROOT_LEN);
    xyz[a] = (g.tv_max[3 * t + a] - g.tv_min[3 * t + a]) * r + g.tv_min[3 * t + a];
  }
}

// extend_from_interface_to_whole_domain_TVD_one_iteration (src/my_p4est_level_set.cpp:3181-3323), one
// field: Godunov upwinding along sgn(phi) grad(phi)/|grad(phi)| with second-order one-sided differences,
// the neighbour across the interface replaced by the interface value at the subcell distance, Neumann
// walls. qdd: D x N second derivatives of q.
template <int D>
void efi_one_iteration(const Ctx& cx, const double* phi, const double* grad, const double* q, const double* qdd, const double* qi_nb,
                       const double* s_nb, double* q_out, int nthreads) {
  const Qnnn<D>* Q = static_cast<const Qnnn<D>*>(cx.qnnn);
  const int64_t N = cx.N;
  const double zdt = cx.zero_distance_threshold;
#pragma omp parallel for schedule(dynamic, 1024) num_threads(nthreads)
  for (long long n = 0; n < (long long)N; ++n) {
    if (fabs(phi[n]) < zdt) {
      q_out[n] = q[n];
      continue;
    }
    const Qnnn<D>& qq = Q[n];
    double p_000, p_nb[6], q_000, q_nb[6], s[6];
    ngbd_quadratic(qq, phi, &p_000, p_nb);
    ngbd_quadratic(qq, q, &q_000, q_nb);
    for (int dir = 0; dir < 2 * D; ++dir) s[dir] = qq.d[dir];
    for (int dir = 0; dir < 2 * D; ++dir)
      if (p_000 * p_nb[dir] < 0.0) {
        s[dir] = s_nb[(size_t)dir * N + n];
        q_nb[dir] = qi_nb[(size_t)dir * N + n];
      }
    // second derivative of q along each axis at the node and at its two neighbours on that axis
    double dd_000[3], dd_m[3], dd_p[3];
    for (int a = 0; a < D; ++a) {
      double z, nb[6];
      ngbd_quadratic(qq, qdd + (size_t)a * N, &z, nb);
      dd_000[a] = z;
      dd_m[a] = nb[2 * a];
      dd_p[a] = nb[2 * a + 1];
    }
    const uint8_t w = cx.wall[n];
    for (int a = 0; a < D; ++a) {
      if (w & (1 << (2 * a))) {
        s[2 * a] = s[2 * a + 1];
        q_nb[2 * a] = q_nb[2 * a + 1];
        dd_000[a] = dd_m[a] = dd_p[a] = 0.0;
      } else if (w & (1 << (2 * a + 1))) {
        s[2 * a + 1] = s[2 * a];
        q_nb[2 * a + 1] = q_nb[2 * a];
        dd_000[a] = dd_m[a] = dd_p[a] = 0.0;
      }
    }
    double dt = MIN(s[0], s[1]);
    dt = MIN(dt, s[2], s[3]);
    if (D == 3) dt = MIN(dt, s[D == 3 ? 4 : 0], s[D == 3 ? 5 : 0]);
    dt /= ((double)D);
    const double gx = grad[n], gy = grad[N + n], gz = D == 3 ? grad[2 * N + n] : 0.0;
    const double mag = D == 3 ? sqrt(gx * gx + gy * gy + gz * gz) : sqrt(gx * gx + gy * gy);
    const double sg = phi[n] < 0.0 ? -1.0 : +1.0;
    const double nv[3] = {mag > ORA_EPS ? sg * gx / mag : 0.0, mag > ORA_EPS ? sg * gy / mag : 0.0,
                          mag > ORA_EPS ? sg * gz / mag : 0.0};
    double t[3];
    for (int a = 0; a < D; ++a) {
      const double qm = (q_000 - q_nb[2 * a]) / s[2 * a] + 0.5 * s[2 * a] * MINMOD(dd_m[a], dd_000[a]);
      const double qp = (q_nb[2 * a + 1] - q_000) / s[2 * a + 1] - 0.5 * s[2 * a + 1] * MINMOD(dd_p[a], dd_000[a]);
      t[a] = nv[a] * (nv[a] > 0.0 ? qm : qp);
    }
    q_out[n] = q_000 - dt * (D == 3 ? (t[0] + t[1] + t[D == 3 ? 2 : 0]) : (t[0] + t[1]));
  }
}

// extend_from_interface_to_whole_domain_TVD(phi, qi, q, iterations, mask, band_zero, band_smooth, cf = NULL,
// grad_phi) (src/my_p4est_level_set.cpp:3325-3767) for one field with the interpolation method used on
// the interface (interpolation_on_interface, quadratic_non_oscillatory_continuous_v2 by default):
// interface values along each grid line crossing the interface, q started from qi within 1.5 dl of the
// interface, then `iterations` TVD-RK2 steps. grad_in (D x N) may be null (first derivatives of phi).
// cf: the caller's interface values, asked one crossing at a time in the reference's order (node by
// node, then direction), as (*cf)(n, dir, dist) is in src/my_p4est_level_set.cpp:3488-3585; q then
// starts at zero.
typedef int (*ora_values_fn)(void* ctx, int64_t count, const int32_t* nodes, const int32_t* dirs, const double* dists, double* values);
template <int D>
void extend_from_interface(const Ctx& cx, const double* phi, const double* qi, double* q, int iterations, const double* mask,
                           double band_zero, double band_smooth, const double* grad_in, int method, int nthreads,
                           ora_values_fn cf = nullptr, void* cf_ctx = nullptr) {
  const Grid<D>& g = *static_cast<const Grid<D>*>(cx.grid);
  const Qnnn<D>* Q = static_cast<const Qnnn<D>*>(cx.qnnn);
  const int64_t N = cx.N;
  int max_lvl = 0;
  for (const Leaf& l : g.leaves) max_lvl = MAX(max_lvl, (int)l.level);
  double dl = g.tree_dim[0] / pow(2., (double)max_lvl);
  for (int a = 1; a < D; ++a) dl = MAX(dl, g.tree_dim[a] / pow(2., (double)max_lvl));
  std::vector<double> qdd((size_t)D * N), grad_store, pdd((size_t)D * N);
  compute_derivatives<D>(cx, qi, qdd.data(), nthreads);
  const double* grad = grad_in;
  if (!grad) {
    grad_store.resize((size_t)D * N);
    first_derivatives<D>(cx, phi, grad_store.data(), nthreads);
    grad = grad_store.data();
  }
  compute_derivatives<D>(cx, phi, pdd.data(), nthreads);
  for (int64_t n = 0; n < N; ++n)
    q[n] = cf ? 0 : ((mask ? MAX(mask[n], fabs(phi[n])) : fabs(phi[n])) < 1.5 * dl ? qi[n] : 0);
  // interface values and distances along the 2D directions
  std::vector<double> qi_nb((size_t)2 * D * N), s_nb((size_t)2 * D * N);
  std::vector<uint8_t> cross((size_t)N, 0);
  std::vector<std::vector<double>> pts(2 * D);
  std::vector<std::vector<int32_t>> who(2 * D);
  for (int64_t n = 0; n < N; ++n) {
    const Qnnn<D>& qq = Q[n];
    double x[3];
    node_coordinates(g, (int32_t)n, x);
    double p_000, p_nb[6];
    ngbd_quadratic(qq, phi, &p_000, p_nb);
    for (int dir = 0; dir < 2 * D; ++dir) {
      const int a = dir / 2;
      const double* paa = pdd.data() + (size_t)a * N;
      if (p_000 * p_nb[dir] < 0.0) {
        double dist = interface_Location_With_Second_Order_Derivative(0, qq.d[dir], p_000, p_nb[dir], paa[n], f_linear(qq, dir, paa));
        dist = MAX(dist, ORA_EPS);
        if (cf) {
          const int32_t nn = (int32_t)n, dd_ = dir;
          double v = 0;
          if (cf(cf_ctx, 1, &nn, &dd_, &dist, &v) != 0) throw std::runtime_error("oracle: cf failed");
          qi_nb[(size_t)dir * N + n] = v;
        } else {
          for (int b = 0; b < D; ++b) pts[dir].push_back(b == a ? ((dir & 1) ? x[b] + dist : x[b] - dist) : x[b]);
          who[dir].push_back((int32_t)n);
        }
        s_nb[(size_t)dir * N + n] = dist;
        cross[n] |= (uint8_t)(1u << dir);
      } else {
        qi_nb[(size_t)dir * N + n] = qi[n];
        s_nb[(size_t)dir * N + n] = qq.d[dir];
      }
    }
  }
  const double a_ = band_zero * dl, b_ = band_smooth * dl;
  for (int dir = 0; dir < 2 * D; ++dir) {
    const int64_t np = (int64_t)who[dir].size();
    std::vector<double> v((size_t)np), m((size_t)np);
    interpolate_points<D>(cx, method, 1, qi, qdd.data(), np, pts[dir].data(), v.data(), nthreads);
    if (mask) interpolate_points<D>(cx, ORA_LINEAR, 1, mask, nullptr, np, pts[dir].data(), m.data(), nthreads);
    for (int64_t k = 0; k < np; ++k) {
      const int32_t n = who[dir][k];
      double val = v[k];
      if (mask) val *= 1. - smoothstep(1, (m[k] - a_) / b_);
      qi_nb[(size_t)dir * N + n] = val;
    }
  }
  std::vector<double> q1((size_t)N), q2((size_t)N);
  for (int it = 0; it < iterations; ++it) {
    compute_derivatives<D>(cx, q, qdd.data(), nthreads);
    efi_one_iteration<D>(cx, phi, grad, q, qdd.data(), qi_nb.data(), s_nb.data(), q1.data(), nthreads);
    compute_derivatives<D>(cx, q1.data(), qdd.data(), nthreads);
    efi_one_iteration<D>(cx, phi, grad, q1.data(), qdd.data(), qi_nb.data(), s_nb.data(), q2.data(), nthreads);
    for (int64_t n = 0; n < N; ++n) q[n] = .5 * (q[n] + q2[n]);
  }
}


template <int D>
Ctx* build_from_leaves(const int* n_xyz, const double* lo, const double* hi, int64_t nleaves, const int32_t* tree,
                       const int32_t* level, const int32_t* xyz) {
  Grid<D>* g = new Grid<D>();
  setup_brick(*g, n_xyz, lo, hi);
  g->leaves.resize(nleaves);
  for (int64_t i = 0; i < nleaves; ++i) {
    g->leaves[i].tree = tree[i];
    g->leaves[i].level = level[i];
    for (int a = 0; a < 3; ++a) g->leaves[i].x[a] = xyz[3 * i + a];
  }
  build_hierarchy(*g);
  build_nodes(*g);
  const int64_t N = (int64_t)g->node_tree.size();
  g->qnnn.resize(N);
  g->wall.resize(N);
  int bad = 0;
#pragma omp parallel for schedule(dynamic, 4096) reduction(+ : bad)
  for (long long i = 0; i < (long long)N; ++i) {  // independent per node
    if (construct_neighbors(*g, (int32_t)i, g->qnnn[i])) ++bad;
    g->wall[i] = wall_of(*g, (int32_t)i);
  }
  if (bad) {
    delete g;
    throw std::runtime_error("oracle: incomplete node neighbourhood");
  }
  Ctx* cx = new Ctx();
  cx->dim = D;
  cx->N = N;
  cx->qnnn = g->qnnn.data();
  cx->wall = g->wall.data();
  cx->grid = g;
  double m = g->tree_dim[0];
  for (int a = 1; a < D; ++a) m = MIN(m, g->tree_dim[a]);
  cx->zero_distance_threshold = ORA_EPS * (D == 3 ? MIN(g->tree_dim[0], g->tree_dim[1], g->tree_dim[2]) : MIN(g->tree_dim[0], g->tree_dim[1]));
  return cx;
}

template <typename Fn>
int guard(Fn&& fn) {
  try {
    fn();
    return 0;
  } catch (const std::exception& e) {
    g_err = e.what();
    return 1;
  }
}

}  // namespace

extern "C" {

const char* ora_last_error(void) { return g_err.c_str(); }
size_t ora_qnnn_record_bytes(int dim) { return dim == 2 ? sizeof(Qnnn<2>) : sizeof(Qnnn<3>); }

int ora_grid_from_leaves(int dim, const int* n_xyz, const double* lo, const double* hi, int64_t nleaves, const int32_t* tree,
                         const int32_t* level, const int32_t* xyz, void** out) {
  return guard([&] {
    *out = dim == 2 ? (void*)build_from_leaves<2>(n_xyz, lo, hi, nleaves, tree, level, xyz)
                    : (void*)build_from_leaves<3>(n_xyz, lo, hi, nleaves, tree, level, xyz);
  });
}

// Borrow neighbour records built elsewhere (same layout; kept alive by the caller) and copy the wall
// mask; tree_dims gives the tree sizes for zero_distance_threshold.
int ora_grid_from_qnnn(int dim, int64_t N, const void* qnnn, const uint8_t* wall, const double* tree_dims, void** out) {
  return guard([&] {
    Ctx* cx = new Ctx();
    cx->dim = dim;
    cx->N = N;
    cx->qnnn = const_cast<void*>(qnnn);  // borrowed: the caller keeps the records alive
    cx->wall_store.assign(wall, wall + N);
    cx->wall = cx->wall_store.data();
    cx->grid = nullptr;
    cx->zero_distance_threshold =
        ORA_EPS * (dim == 3 ? MIN(tree_dims[0], tree_dims[1], tree_dims[2]) : MIN(tree_dims[0], tree_dims[1]));
    *out = cx;
  });
}

void ora_grid_destroy(void* h) {
  Ctx* cx = static_cast<Ctx*>(h);
  if (!cx) return;
  if (cx->grid) {
    if (cx->dim == 2) delete static_cast<Grid<2>*>(cx->grid);
    else delete static_cast<Grid<3>*>(cx->grid);
  }
  delete cx;
}

int64_t ora_grid_num_nodes(void* h) { return static_cast<Ctx*>(h)->N; }
double ora_zero_distance_threshold(void* h) { return static_cast<Ctx*>(h)->zero_distance_threshold; }

// owner tree and clamped logical coordinates (3 per node) of the oracle's own numbering
int ora_grid_nodes(void* h, int32_t* tree, int64_t* xyz) {
  return guard([&] {
    Ctx* cx = static_cast<Ctx*>(h);
    if (!cx->grid) throw std::runtime_error("grid built from records has no node coordinates");
    const int D = cx->dim;
    const std::vector<int32_t>& nt = D == 2 ? static_cast<Grid<2>*>(cx->grid)->node_tree : static_cast<Grid<3>*>(cx->grid)->node_tree;
    const std::vector<int64_t>& nx = D == 2 ? static_cast<Grid<2>*>(cx->grid)->node_x : static_cast<Grid<3>*>(cx->grid)->node_x;
    for (int64_t n = 0; n < cx->N; ++n) {
      tree[n] = nt[n];
      for (int a = 0; a < 3; ++a) xyz[3 * n + a] = a < D ? nx[(size_t)n * D + a] : 0;
    }
  });
}

int ora_grid_export_qnnn(void* h, void* out) {
  return guard([&] {
    Ctx* cx = static_cast<Ctx*>(h);
    memcpy(out, cx->qnnn, ora_qnnn_record_bytes(cx->dim) * cx->N);
  });
}

int ora_grid_wall_mask(void* h, uint8_t* out) {
  return guard([&] {
    Ctx* cx = static_cast<Ctx*>(h);
    memcpy(out, cx->wall, cx->N);
  });
}

int ora_compute_derivatives(void* h, const double* f, double* fdd, int nthreads) {
  return guard([&] {
    Ctx* cx = static_cast<Ctx*>(h);
    if (cx->dim == 2) compute_derivatives<2>(*cx, f, fdd, nthreads);
    else compute_derivatives<3>(*cx, f, fdd, nthreads);
  });
}

int ora_reinitialize_masked(void* h, double* phi, const double* mask, int order_space, int order_pseudotime, double limit_high,
                            double limit_low, int iters, int nthreads) {
  return guard([&] {
    if (order_space < 1 || order_space > 2 || order_pseudotime < 1 || order_pseudotime > 2)
      throw std::invalid_argument("valid orders of accuracy are 1 and 2 only");
    Ctx* cx = static_cast<Ctx*>(h);
    if (cx->dim == 2) reinitialize<2>(*cx, phi, order_space, order_pseudotime, limit_high, limit_low, iters, nthreads, mask);
    else reinitialize<3>(*cx, phi, order_space, order_pseudotime, limit_high, limit_low, iters, nthreads, mask);
  });
}

int ora_reinitialize(void* h, double* phi, int order_space, int order_pseudotime, double limit_high, double limit_low, int iters,
                     int nthreads) {
  return guard([&] {
    if (order_space < 1 || order_space > 2 || order_pseudotime < 1 || order_pseudotime > 2)
      throw std::invalid_argument("valid orders of accuracy are 1 and 2 only");
    Ctx* cx = static_cast<Ctx*>(h);
    if (cx->dim == 2) reinitialize<2>(*cx, phi, order_space, order_pseudotime, limit_high, limit_low, iters, nthreads);
    else reinitialize<3>(*cx, phi, order_space, order_pseudotime, limit_high, limit_low, iters, nthreads);
  });
}

int ora_advect_in_normal_direction(void* h, const double* vn, const double* vn_np1, double* phi, double dt, double* phi_dd,
                                   int nthreads) {
  return guard([&] {
    Ctx* cx = static_cast<Ctx*>(h);
    if (cx->dim == 2) advect_normal<2>(*cx, vn, vn_np1, phi, dt, phi_dd, nthreads);
    else advect_normal<3>(*cx, vn, vn_np1, phi, dt, phi_dd, nthreads);
  });
}

// CF overload's time step: dt = MIN over nodes of 0.8*fabs(s_min/vn) (src/my_p4est_level_set.cpp:752-776)
int ora_advect_cfl_dt(void* h, const double* vn, double* dt_out) {
  return guard([&] {
    Ctx* cx = static_cast<Ctx*>(h);
    double dt = DBL_MAX;
    for (int64_t n = 0; n < cx->N; ++n) {
      double smin;
      if (cx->dim == 2) {
        const Qnnn<2>& q = static_cast<const Qnnn<2>*>(cx->qnnn)[n];
        smin = MIN(MIN(fabs(q.d[1]), fabs(q.d[0])), MIN(fabs(q.d[3]), fabs(q.d[2])));
      } else {
        const Qnnn<3>& q = static_cast<const Qnnn<3>*>(cx->qnnn)[n];
        smin = MIN(MIN(fabs(q.d[1]), fabs(q.d[0])), MIN(fabs(q.d[3]), fabs(q.d[2])), MIN(fabs(q.d[5]), fabs(q.d[4])));
      }
      dt = MIN(dt, 0.8 * fabs(smin / vn[n]));
    }
    *dt_out = dt;
  });
}

int ora_interpolate(void* h, int method, int nfields, const double* F, const double* Fdd, int64_t npts, const double* xyz,
                    double* out, int nthreads) {
  return guard([&] {
    Ctx* cx = static_cast<Ctx*>(h);
    if (!cx->grid) throw std::runtime_error("interpolation needs a grid built from leaves");
    if (method < 0 || method > 4) throw std::invalid_argument("unknown interpolation method");
    std::vector<double> store;
    if (cx->dim == 2) {
      const double* dd = method == ORA_LINEAR ? nullptr : derivatives_of<2>(*cx, nfields, F, Fdd, store, nthreads);
      interpolate_points<2>(*cx, method, nfields, F, dd, npts, xyz, out, nthreads);
    } else {
      const double* dd = method == ORA_LINEAR ? nullptr : derivatives_of<3>(*cx, nfields, F, Fdd, store, nthreads);
      interpolate_points<3>(*cx, method, nfields, F, dd, npts, xyz, out, nthreads);
    }
  });
}

// leaf chosen by the point location for each point (after clipping)
int ora_locate(void* h, int64_t npts, const double* xyz, int32_t* leaf) {
  return guard([&] {
    Ctx* cx = static_cast<Ctx*>(h);
    if (!cx->grid) throw std::runtime_error("point location needs a grid built from leaves");
    for (int64_t p = 0; p < npts; ++p) {
      double x[3] = {0, 0, 0};
      for (int a = 0; a < cx->dim; ++a) x[a] = xyz[p * cx->dim + a];
      if (cx->dim == 2) {
        clip_in_domain(*static_cast<Grid<2>*>(cx->grid), x);
        leaf[p] = find_smallest_quadrant(*static_cast<Grid<2>*>(cx->grid), x);
      } else {
        clip_in_domain(*static_cast<Grid<3>*>(cx->grid), x);
        leaf[p] = find_smallest_quadrant(*static_cast<Grid<3>*>(cx->grid), x);
      }
    }
  });
}

int ora_sl_advect(void* h, int64_t npts, const double* xyz, double dt, const double* v, const double* vdd, const double* phi,
                  const double* phi_dd, int velo_method, int phi_method, double* phi_np1, int nthreads) {
  return guard([&] {
    Ctx* cx = static_cast<Ctx*>(h);
    if (!cx->grid) throw std::runtime_error("semi-Lagrangian step needs a grid built from leaves");
    if (cx->dim == 2) sl_advect<2>(*cx, npts, xyz, dt, v, vdd, phi, phi_dd, velo_method, phi_method, phi_np1, nthreads);
    else sl_advect<3>(*cx, npts, xyz, dt, v, vdd, phi, phi_dd, velo_method, phi_method, phi_np1, nthreads);
  });
}

// One sweep over the nodes [first, first + count) only (the per-rank work of a Morton-range split):
// compute_derivatives, and one reinitialize_one_iteration stage (phi_0_dd / phi_n_dd null: first order in
// space). The limits are the caller's phi_0 range, widened as reinitialize_within_range_of_phi_0 does.
int ora_compute_derivatives_range(void* h, const double* f, double* out, int64_t first, int64_t count, int nthreads) {
  return guard([&] {
    Ctx* cx = static_cast<Ctx*>(h);
    if (first < 0 || count < 0 || first + count > cx->N) throw std::runtime_error("node range out of bounds");
    if (cx->dim == 2) compute_derivatives<2>(*cx, f, out, nthreads, first, count);
    else compute_derivatives<3>(*cx, f, out, nthreads, first, count);
  });
}

// One advect_in_normal_direction_one_iteration sweep over the nodes [first, first + count) only (the per-rank work of
// a Morton-range split): phi_np1 = phi_n - dt vn |grad phi_n| there, dd the minmod terms' second derivatives.
int ora_advect_stage_range(void* h, const double* vn, double dt, const double* dd, const double* phi_n, double* phi_np1, int64_t first,
                           int64_t count, int nthreads) {
  return guard([&] {
    Ctx* cx = static_cast<Ctx*>(h);
    if (first < 0 || count < 0 || first + count > cx->N) throw std::runtime_error("node range out of bounds");
    if (cx->dim == 2) advect_one_iteration<2>(*cx, vn, dt, dd, phi_n, phi_np1, nthreads, first, count);
    else advect_one_iteration<3>(*cx, vn, dt, dd, phi_n, phi_np1, nthreads, first, count);
  });
}

int ora_reinit_stage_range(void* h, double* phi_np1, const double* phi_0, const double* phi_n, double limit_high, double limit_low,
                           const double* phi_0_dd, const double* phi_n_dd, int64_t first, int64_t count, int nthreads) {
  return guard([&] {
    Ctx* cx = static_cast<Ctx*>(h);
    if (first < 0 || count < 0 || first + count > cx->N) throw std::runtime_error("node range out of bounds");
    if (cx->dim == 2)
      reinitialize_one_iteration<2>(*cx, phi_np1, phi_0, phi_n, limit_high, limit_low, phi_0_dd, phi_n_dd, nthreads, first, count);
    else
      reinitialize_one_iteration<3>(*cx, phi_np1, phi_0, phi_n, limit_high, limit_low, phi_0_dd, phi_n_dd, nthreads, first, count);
  });
}

int ora_sl_advect2(void* h_n, void* h_nm1, int64_t npts, const double* xyz, double dt_nm1, double dt_n, const double* vnm1,
                   const double* vnm1_dd, const double* vn, const double* vn_dd, const double* phi, const double* phi_dd, int velo_method,
                   int phi_method, double* phi_np1, int nthreads) {
  return guard([&] {
    Ctx* cn = static_cast<Ctx*>(h_n);
    Ctx* cm = static_cast<Ctx*>(h_nm1);
    if (!cn->grid || !cm->grid) throw std::runtime_error("semi-Lagrangian step needs grids built from leaves");
    if (cn->dim != cm->dim) throw std::runtime_error("grids of one dimension required");
    if (cn->dim == 2)
      sl_advect2<2>(*cn, *cm, npts, xyz, dt_nm1, dt_n, vnm1, vnm1_dd, vn, vn_dd, phi, phi_dd, velo_method, phi_method, phi_np1, nthreads);
    else
      sl_advect2<3>(*cn, *cm, npts, xyz, dt_nm1, dt_n, vnm1, vnm1_dd, vn, vn_dd, phi, phi_dd, velo_method, phi_method, phi_np1, nthreads);
  });
}

int ora_sl_advect_vortex(void* h, int64_t npts, const double* xyz, double dt, double vscale, const double* phi, const double* phi_dd,
                         int phi_method, double* phi_np1, int nthreads) {
  return guard([&] {
    Ctx* cx = static_cast<Ctx*>(h);
    if (!cx->grid) throw std::runtime_error("semi-Lagrangian step needs a grid built from leaves");
    if (cx->dim == 2) sl_advect_vortex<2>(*cx, npts, xyz, dt, vscale, phi, phi_dd, phi_method, phi_np1, nthreads);
    else sl_advect_vortex<3>(*cx, npts, xyz, dt, vscale, phi, phi_dd, phi_method, phi_np1, nthreads);
  });
}

int ora_first_derivatives(void* h, const double* f, double* out, int nthreads) {
  return guard([&] {
    Ctx* cx = static_cast<Ctx*>(h);
    if (cx->dim == 2) first_derivatives<2>(*cx, f, out, nthreads);
    else first_derivatives<3>(*cx, f, out, nthreads);
  });
}

int ora_compute_normals(void* h, const double* phi, double* out, int nthreads) {
  return guard([&] {
    Ctx* cx = static_cast<Ctx*>(h);
    if (cx->dim == 2) {
      first_derivatives<2>(*cx, phi, out, nthreads);
      normalize<2>(cx->N, out);
    } else {
      first_derivatives<3>(*cx, phi, out, nthreads);
      normalize<3>(cx->N, out);
    }
  });
}

int ora_mean_curvature_from_normals(void* h, const double* normals, double* kappa, int nthreads) {
  return guard([&] {
    Ctx* cx = static_cast<Ctx*>(h);
    if (cx->dim == 2) curvature_from_normals<2>(*cx, normals, kappa, nthreads);
    else curvature_from_normals<3>(*cx, normals, kappa, nthreads);
  });
}

int ora_normals_and_mean_curvature(void* h, const double* phi, double* normals, double* kappa, int nthreads) {
  return guard([&] {
    Ctx* cx = static_cast<Ctx*>(h);
    if (cx->dim == 2) normals_and_curvature<2>(*cx, phi, normals, kappa, nthreads);
    else normals_and_curvature<3>(*cx, phi, normals, kappa, nthreads);
  });
}

int ora_extend_over_interface_ex(void* h, const double* phi, const double* mask, double* q, int iterations, int order, double band_use,
                                 double band_extend, const double* normals, int nonzero_guess, double* q_n, double* q_nn, int nthreads) {
  return guard([&] {
    Ctx* cx = static_cast<Ctx*>(h);
    if (!cx->grid) throw std::runtime_error("extension needs a grid built from leaves");
    if (order < 0 || order > 2) throw std::invalid_argument("order must be 0, 1 or 2");
    if (cx->dim == 2)
      extend_over_interface<2>(*cx, phi, mask, q, iterations, order, band_use, band_extend, normals, nthreads, nonzero_guess != 0, q_n, q_nn);
    else
      extend_over_interface<3>(*cx, phi, mask, q, iterations, order, band_use, band_extend, normals, nthreads, nonzero_guess != 0, q_n, q_nn);
  });
}

int ora_extend_over_interface(void* h, const double* phi, const double* mask, double* q, int iterations, int order, double band_use,
                              double band_extend, const double* normals, int nthreads) {
  return guard([&] {
    Ctx* cx = static_cast<Ctx*>(h);
    if (!cx->grid) throw std::runtime_error("extension needs a grid built from leaves");
    if (order < 0 || order > 2) throw std::invalid_argument("order must be 0, 1 or 2");
    if (cx->dim == 2) extend_over_interface<2>(*cx, phi, mask, q, iterations, order, band_use, band_extend, normals, nthreads);
    else extend_over_interface<3>(*cx, phi, mask, q, iterations, order, band_use, band_extend, normals, nthreads);
  });
}

int ora_extend_from_interface(void* h, const double* phi, const double* qi, double* q, int iterations, const double* mask,
                              double band_zero, double band_smooth, const double* grad, int method, int nthreads) {
  return guard([&] {
    Ctx* cx = static_cast<Ctx*>(h);
    if (!cx->grid) throw std::runtime_error("extension needs a grid built from leaves");
    if (cx->dim == 2) extend_from_interface<2>(*cx, phi, qi, q, iterations, mask, band_zero, band_smooth, grad, method, nthreads);
    else extend_from_interface<3>(*cx, phi, qi, q, iterations, mask, band_zero, band_smooth, grad, method, nthreads);
  });
}

int ora_extend_from_interface_cf(void* h, const double* phi, const double* qi, double* q, int iterations, ora_values_fn cf, void* ctx,
                                 const double* grad, int nthreads) {
  return guard([&] {
    Ctx* cx = static_cast<Ctx*>(h);
    if (!cx->grid) throw std::runtime_error("extension needs a grid built from leaves");
    if (cx->dim == 2) extend_from_interface<2>(*cx, phi, qi, q, iterations, nullptr, 0.0, 1.0, grad, 4, nthreads, cf, ctx);
    else extend_from_interface<3>(*cx, phi, qi, q, iterations, nullptr, 0.0, 1.0, grad, 4, nthreads, cf, ctx);
  });
}

// interface_Location / interface_Location_With_Second_Order_Derivative (src/casl_math.cpp:55-97)
double ora_interface_location(double a, double b, double fa, double fb) { return interface_Location(a, b, fa, fb); }
double ora_interface_location_2nd(double a, double b, double fa, double fb, double fxxa, double fxxb) {
  return interface_Location_With_Second_Order_Derivative(a, b, fa, fb, fxxa, fxxb);
}

// velocity of the single vortex at points (D per point), D x np output
int ora_vortex(int dim, int64_t npts, const double* xyz, double vscale, double* v) {
  return guard([&] {
    for (int64_t p = 0; p < npts; ++p) {
      double x[3] = {0, 0, 0}, w[3];
      for (int a = 0; a < dim; ++a) x[a] = xyz[p * dim + a];
      if (dim == 2) vortex<2>(x, vscale, w);
      else vortex<3>(x, vscale, w);
      for (int a = 0; a < dim; ++a) v[(size_t)a * npts + p] = w[a];
    }
  });
}

}  // extern "C"
