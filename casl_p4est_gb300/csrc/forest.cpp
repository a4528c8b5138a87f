// Host forest implementation (see forest.hpp for what it stands in for).
#include "forest.hpp"

#include <algorithm>
#include <cstring>
#ifdef _OPENMP
#include <omp.h>
#include <parallel/algorithm>
#endif

namespace lsg {

void sort_u64(std::vector<uint64_t>& v) {
#ifdef _OPENMP
  if (v.size() > (size_t)1 << 16) {
    __gnu_parallel::sort(v.begin(), v.end());
    return;
  }
#endif
  std::sort(v.begin(), v.end());
}

// Trees of a brick are numbered along a Morton curve of their (i,j,k) position, as
// p4est_connectivity_new_brick does; vertex coordinates follow my_p4est_brick_new
// (src/my_p4est_tools.c:138-168): xyz_min + (i+ii)*dx with dx = (xyz_max - xyz_min)/n.
void Brick::init(int dim_, const int* n_, const double* xyz_min_, const double* xyz_max_, const int* periodic_) {
  dim = dim_;
  for (int a = 0; a < 3; ++a) {
    n[a] = (a < dim) ? n_[a] : 1;
    xyz_min[a] = (a < dim) ? xyz_min_[a] : 0.0;
    xyz_max[a] = (a < dim) ? xyz_max_[a] : 0.0;
    periodic[a] = (a < dim && periodic_) ? periodic_[a] : 0;
    if (n[a] < 1) throw std::invalid_argument("brick: number of trees per axis must be >= 1");
    if (a < dim && !(xyz_max[a] > xyz_min[a])) throw std::invalid_argument("brick: xyz_max must exceed xyz_min");
  }
  num_trees = n[0] * n[1] * n[2];
  std::vector<std::pair<uint64_t, int>> order;
  order.reserve(num_trees);
  for (int k = 0; k < n[2]; ++k)
    for (int j = 0; j < n[1]; ++j)
      for (int i = 0; i < n[0]; ++i) {
        uint64_t key = spread3((uint64_t)i) | (spread3((uint64_t)j) << 1) | (spread3((uint64_t)k) << 2);
        order.push_back({key, (n[0] * n[1] * k + n[0] * j + i)});
      }
  std::sort(order.begin(), order.end());
  ijk_to_tree.assign(num_trees, -1);
  tree_ijk.assign(3 * (size_t)num_trees, 0);
  tmin.assign(3 * (size_t)num_trees, 0.0);
  tmax.assign(3 * (size_t)num_trees, 0.0);
  double dxyz[3];
  for (int a = 0; a < 3; ++a) dxyz[a] = (xyz_max[a] - xyz_min[a]) / (double)n[a];
  for (int t = 0; t < num_trees; ++t) {
    int lin = order[t].second;
    int ijk[3] = {lin % n[0], (lin / n[0]) % n[1], lin / (n[0] * n[1])};
    ijk_to_tree[lin] = t;
    for (int a = 0; a < 3; ++a) {
      tree_ijk[3 * t + a] = ijk[a];
      if (a < dim) {
        tmin[3 * t + a] = xyz_min[a] + (ijk[a] + 0) * dxyz[a];
        tmax[3 * t + a] = xyz_min[a] + (ijk[a] + 1) * dxyz[a];
      }
    }
  }
}

template <int D>
void Forest<D>::init(const int* n, const double* xyz_min, const double* xyz_max, const int* periodic) {
  brick.init(D, n, xyz_min, xyz_max, periodic);
  for (int a = 0; a < D; ++a)
    if (brick.periodic[a]) throw std::invalid_argument("periodic bricks are not supported by this build of the host forest");
  if (brick.num_trees > max_trees_for_keys<D>()) throw std::invalid_argument("too many trees for 64-bit node keys");
  std::vector<Quad> roots;
  std::vector<uint64_t> keys;
  for (int t = 0; t < brick.num_trees; ++t) {
    Quad q;
    q.x[0] = q.x[1] = q.x[2] = 0;
    q.tree = t;
    q.level = 0;
    roots.push_back(q);
    keys.push_back(((uint64_t)t) << tree_shift<D>());
  }
  leaves.replace(std::move(roots));
  leaf_key.replace(std::move(keys));
  drop_nodes();
}

template <int D>
void Forest<D>::refine(const uint8_t* tags) {
  const size_t nl = leaves.size();
  std::vector<size_t> offset(nl + 1, 0);
  for (size_t i = 0; i < nl; ++i) {
    if (tags[i] && leaves[i].level >= DD::QMAXLEVEL) throw std::invalid_argument("refine: quadrant already at the maximum level");
    offset[i + 1] = offset[i] + (tags[i] ? DD::CHILDREN : 1);
  }
  std::vector<Quad> out(offset[nl]);
  std::vector<uint64_t> keys(offset[nl]);
#pragma omp parallel for schedule(static)
  for (long long ii = 0; ii < (long long)nl; ++ii) {
    const size_t i = (size_t)ii;
    const Quad& q = leaves[i];
    size_t o = offset[i];
    if (!tags[i]) {
      out[o] = q;
      keys[o] = leaf_key[i];
      continue;
    }
    const int32_t h = quadrant_len(DD::MAXLEVEL, q.level + 1);
    for (int c = 0; c < DD::CHILDREN; ++c) {
      Quad ch = q;
      ch.level = q.level + 1;
      for (int a = 0; a < D; ++a) ch.x[a] = q.x[a] + (((c >> a) & 1) ? h : 0);
      out[o + c] = ch;
      keys[o + c] = (((uint64_t)ch.tree) << tree_shift<D>()) | morton<D>(ch.x);
    }
  }
  leaves.replace(std::move(out));
  leaf_key.replace(std::move(keys));
  drop_nodes();
}

template <int D>
bool Forest<D>::family_at(size_t i, const uint8_t* tags) const {
  const size_t nl = leaves.size();
  const Quad& q = leaves[i];
  if (q.level == 0 || i + DD::CHILDREN > nl) return false;
  const int32_t hp = quadrant_len(DD::MAXLEVEL, q.level - 1);
  for (int a = 0; a < D; ++a)
    if (q.x[a] % hp != 0) return false;
  const int32_t h = quadrant_len(DD::MAXLEVEL, q.level);
  for (int c = 0; c < DD::CHILDREN; ++c) {
    const Quad& s = leaves[i + c];
    if (s.level != q.level || s.tree != q.tree || !tags[i + c]) return false;
    for (int a = 0; a < D; ++a)
      if (s.x[a] != q.x[a] + (((c >> a) & 1) ? h : 0)) return false;
  }
  return true;
}

template <int D>
void Forest<D>::coarsen(const uint8_t* tags) {
  const size_t nl = leaves.size();
  std::vector<Quad> out;
  std::vector<uint64_t> keys;
  out.reserve(nl);
  keys.reserve(nl);
  size_t i = 0;
  while (i < nl) {
    const Quad& q = leaves[i];
    const bool family = family_at(i, tags);
    if (family) {
      Quad p = q;
      p.level = q.level - 1;
      out.push_back(p);
      keys.push_back(leaf_key[i]);
      i += DD::CHILDREN;
    } else {
      out.push_back(q);
      keys.push_back(leaf_key[i]);
      ++i;
    }
  }
  leaves.replace(std::move(out));
  leaf_key.replace(std::move(keys));
  drop_nodes();
}

// Exclusive prefix sum of cnt[0..n) into off[0..n], off[n] = total; OpenMP blocks of the range each
// sum their part, then add the totals of the blocks before them.
static void exclusive_scan_sizes(const uint8_t* cnt, size_t n, std::vector<size_t>& off) {
  off.assign(n + 1, 0);
#ifdef _OPENMP
  const int nt = n > ((size_t)1 << 15) ? omp_get_max_threads() : 1;
#else
  const int nt = 1;
#endif
  std::vector<size_t> part((size_t)nt + 1, 0);
#pragma omp parallel num_threads(nt)
  {
#ifdef _OPENMP
    const int t = omp_get_thread_num();
#else
    const int t = 0;
#endif
    const size_t lo = n * (size_t)t / (size_t)nt, hi = n * (size_t)(t + 1) / (size_t)nt;
    size_t sum = 0;
    for (size_t i = lo; i < hi; ++i) sum += cnt[i];
    part[(size_t)t + 1] = sum;
#pragma omp barrier
#pragma omp single
    for (int k = 0; k < nt; ++k) part[(size_t)k + 1] += part[(size_t)k];
    size_t run = part[(size_t)t];
    for (size_t i = lo; i < hi; ++i) {
      off[i] = run;
      run += cnt[i];
    }
  }
  off[n] = part[(size_t)nt];
}

// The sequential pass (coarsen every complete family tagged -1 in linear order, then refine the
// surviving leaves tagged +1) in three parallel sweeps. Families cannot overlap in a linear forest
// and a family can only start at its first child, so testing every leaf independently finds the same
// families as the sequential scan; each leaf then emits 0 (inside a family), 1 or CHILDREN leaves at
// an offset from a prefix sum, in the sequential output order.
template <int D>
bool Forest<D>::coarsen_then_refine(const int8_t* tag) {
  constexpr int C = DD::CHILDREN;
  const size_t nl = leaves.size();
  std::vector<uint8_t> ctag(nl), fam(nl), cnt(nl);
#pragma omp parallel for schedule(static)
  for (long long ii = 0; ii < (long long)nl; ++ii) ctag[(size_t)ii] = tag[ii] < 0;
#pragma omp parallel for schedule(static)
  for (long long ii = 0; ii < (long long)nl; ++ii) fam[(size_t)ii] = family_at((size_t)ii, ctag.data()) ? 1 : 0;
  int changed = 0;
#pragma omp parallel for schedule(static) reduction(| : changed)
  for (long long ii = 0; ii < (long long)nl; ++ii) {
    const size_t i = (size_t)ii;
    bool inside = false;
    for (int c = 1; c < C && !inside; ++c) inside = i >= (size_t)c && fam[i - (size_t)c];
    if (fam[i]) {
      cnt[i] = 1;
      changed = 1;
    } else if (inside) {
      cnt[i] = 0;
    } else if (tag[i] > 0) {
      if (leaves[i].level >= DD::QMAXLEVEL) changed |= 2;
      cnt[i] = (uint8_t)C;
      changed |= 1;
    } else {
      cnt[i] = 1;
    }
  }
  if (changed & 2) throw std::invalid_argument("refine: quadrant already at the maximum level");
  if (!changed) return false;  // same leaves: the node numbering (and its device copy) still holds
  std::vector<size_t> off;
  exclusive_scan_sizes(cnt.data(), nl, off);
  std::vector<Quad> out(off[nl]);
  std::vector<uint64_t> keys(off[nl]);
#pragma omp parallel for schedule(static)
  for (long long ii = 0; ii < (long long)nl; ++ii) {
    const size_t i = (size_t)ii;
    const size_t o = off[i];
    const Quad& q = leaves[i];
    if (cnt[i] == 0) continue;
    if (fam[i]) {
      Quad pq = q;
      pq.level = q.level - 1;
      out[o] = pq;
      keys[o] = leaf_key[i];  // the parent starts where its first child does
    } else if (cnt[i] == 1) {
      out[o] = q;
      keys[o] = leaf_key[i];
    } else {
      const int32_t h = quadrant_len(DD::MAXLEVEL, q.level + 1);
      for (int c = 0; c < C; ++c) {
        Quad ch = q;
        ch.level = q.level + 1;
        for (int a = 0; a < D; ++a) ch.x[a] = q.x[a] + (((c >> a) & 1) ? h : 0);
        out[o + (size_t)c] = ch;
        keys[o + (size_t)c] = (((uint64_t)ch.tree) << tree_shift<D>()) | morton<D>(ch.x);
      }
    }
  }
  leaves.replace(std::move(out));
  leaf_key.replace(std::move(keys));
  drop_nodes();
  return true;
}

template <int D>
void Forest<D>::tag_refine_coarsen(int min_lvl, int max_lvl, double lip, double band, const double* phi, int8_t* tag) const {
  if (!nodes_built) throw std::invalid_argument("refine_and_coarsen: the forest's nodes are not built");
  const size_t nl = leaves.size();
  const std::vector<int32_t>& ln = nd->host().local_nodes;
#pragma omp parallel for schedule(static)
  for (long long ii = 0; ii < (long long)nl; ++ii) {
    const Quad& qd = leaves[(size_t)ii];
    if (qd.level < min_lvl) {
      tag[ii] = 1;
      continue;
    }
    if (qd.level > max_lvl) {
      tag[ii] = -1;
      continue;
    }
    double f[DD::CHILDREN];
    for (int c = 0; c < DD::CHILDREN; ++c) f[c] = phi[ln[(size_t)ii * DD::CHILDREN + c]];
    const double* tmn = &brick.tmin[3 * qd.tree];
    const double* tmx = &brick.tmax[3 * qd.tree];
    const double dmin = (double)quadrant_len(DD::MAXLEVEL, qd.level) / (double)DD::ROOT_LEN;
    const double lmax_len = (double)quadrant_len(DD::MAXLEVEL, max_lvl) / (double)DD::ROOT_LEN;
    const double dx = (tmx[0] - tmn[0]) * dmin;
    const double dy = (tmx[1] - tmn[1]) * dmin;
    double smallest_dxyz_max = max2((tmx[0] - tmn[0]), (tmx[1] - tmn[1])) * lmax_len;
    double d;
    if (D == 3) {
      const double dz = (tmx[2] - tmn[2]) * dmin;
      smallest_dxyz_max = max2(smallest_dxyz_max, (tmx[2] - tmn[2]) * lmax_len);
      d = sqrt(dx * dx + dy * dy + dz * dz);
    } else {
      d = sqrt(dx * dx + dy * dy);
    }
    const double band_real = band * smallest_dxyz_max;
    bool refine = false, coarsen = true;
    for (int i = 0; i < DD::CHILDREN; ++i) {
      refine = refine || (qd.level < max_lvl &&
                          (fabs(f[i]) - band_real <= 0.5 * lip * d ||
                           (i == 0 ? false : ((f[i] > 0.0 && f[0] <= 0.0) || (f[i] <= 0.0 && f[0] > 0.0)))));
      coarsen = coarsen && qd.level > min_lvl && fabs(f[i]) - band_real >= 1.0 * lip * d &&
                (i == 0 ? true : ((f[i] > 0.0 && f[0] > 0.0) || (f[i] <= 0.0 && f[0] <= 0.0)));
    }
    tag[ii] = refine ? 1 : (coarsen ? -1 : 0);
  }
}

template <int D>
void Forest<D>::set_leaves(size_t n, const int32_t* tree, const int32_t* level, const int32_t* xyz) {
  std::vector<Quad> ls(n);
  std::vector<uint64_t> keys(n);
  int32_t expect_tree = 0;
  uint64_t expect_key = 0;
  for (size_t i = 0; i < n; ++i) {
    Quad q;
    q.tree = tree[i];
    q.level = level[i];
    for (int a = 0; a < 3; ++a) q.x[a] = a < D ? xyz[3 * i + a] : 0;
    if (q.tree < 0 || q.tree >= brick.num_trees || q.level < 0 || q.level > DD::QMAXLEVEL)
      throw std::invalid_argument("set_leaves: tree or level out of range");
    const int32_t h = quadrant_len(DD::MAXLEVEL, q.level);
    for (int a = 0; a < D; ++a)
      if (q.x[a] < 0 || q.x[a] >= DD::ROOT_LEN || q.x[a] % h != 0) throw std::invalid_argument("set_leaves: misaligned leaf");
    const uint64_t m = morton<D>(q.x);
    if (q.tree != expect_tree || m != expect_key)
      throw std::invalid_argument("set_leaves: leaves must form a complete forest in tree-major Morton order");
    const uint64_t next = m + (uint64_t(1) << (D * (DD::MAXLEVEL - q.level)));
    if (next == (uint64_t(1) << (D * DD::MAXLEVEL))) {
      ++expect_tree;
      expect_key = 0;
    } else {
      expect_key = next;
    }
    ls[i] = q;
    keys[i] = (((uint64_t)q.tree) << tree_shift<D>()) | m;
  }
  if (expect_tree != brick.num_trees || expect_key != 0) throw std::invalid_argument("set_leaves: the leaves do not cover every tree");
  leaves.replace(std::move(ls));
  leaf_key.replace(std::move(keys));
  drop_nodes();
}

template <int D>
bool Forest<D>::global_to_tree(const int64_t* G, int32_t& tree, int32_t* x) const {
  int ijk[3] = {0, 0, 0};
  for (int a = 0; a < D; ++a) {
    const int64_t L = (int64_t)brick.n[a] * DD::ROOT_LEN;
    if (G[a] < 0 || G[a] >= L) return false;
    ijk[a] = (int)(G[a] / DD::ROOT_LEN);
    x[a] = (int32_t)(G[a] - (int64_t)ijk[a] * DD::ROOT_LEN);
  }
  tree = brick.tree_at(ijk);
  return true;
}

template <int D>
int32_t Forest<D>::find_leaf(int32_t tree, const int32_t* x) const {
  const uint64_t key = (((uint64_t)tree) << tree_shift<D>()) | morton<D>(x);
  auto it = std::upper_bound(leaf_key.begin(), leaf_key.end(), key);
  if (it == leaf_key.begin()) return -1;
  const int32_t idx = (int32_t)((it - leaf_key.begin()) - 1);
  const Quad& q = leaves[idx];
  if (q.tree != tree) return -1;
  const int32_t h = quadrant_len(DD::MAXLEVEL, q.level);
  for (int a = 0; a < D; ++a)
    if (x[a] < q.x[a] || x[a] >= q.x[a] + h) return -1;
  return idx;
}

// Every leaf corner becomes a node (src/my_p4est_nodes.h:55-63). A corner shared by several trees
// is owned by the lowest tree id that touches it and is clamped inside that tree
// (p4est_node_canonicalize, src/my_p4est_nodes.c); nodes are sorted by (owner tree, Morton index)
// (src/my_p4est_nodes.c:606-627).
template <int D>
void Forest<D>::build_nodes() {
  const size_t nl = leaves.size();
  std::vector<uint64_t> corner_key(nl * DD::CHILDREN);
  auto canon = [&](const Quad& q, int c) -> uint64_t {
    int64_t G[3] = {0, 0, 0};
    const int32_t h = quadrant_len(DD::MAXLEVEL, q.level);
    for (int a = 0; a < D; ++a)
      G[a] = (int64_t)brick.tree_ijk[3 * q.tree + a] * DD::ROOT_LEN + q.x[a] + (((c >> a) & 1) ? h : 0);
    // candidate trees along each axis
    int cand[3][2];
    int ncand[3] = {1, 1, 1};
    for (int a = 0; a < 3; ++a) cand[a][0] = cand[a][1] = 0;
    for (int a = 0; a < D; ++a) {
      const int64_t L = (int64_t)brick.n[a] * DD::ROOT_LEN;
      int64_t t = G[a] / DD::ROOT_LEN;
      if (G[a] == L) {
        cand[a][0] = (int)(t - 1);
      } else if (G[a] % DD::ROOT_LEN == 0 && G[a] > 0) {
        cand[a][0] = (int)(t - 1);
        cand[a][1] = (int)t;
        ncand[a] = 2;
      } else {
        cand[a][0] = (int)t;
      }
    }
    int32_t owner = -1;
    int owner_ijk[3] = {0, 0, 0};
    for (int k = 0; k < ncand[2]; ++k)
      for (int j = 0; j < ncand[1]; ++j)
        for (int i = 0; i < ncand[0]; ++i) {
          int ijk[3] = {cand[0][i], cand[1][j], cand[2][k]};
          int32_t t = brick.tree_at(ijk);
          if (owner < 0 || t < owner) {
            owner = t;
            owner_ijk[0] = ijk[0];
            owner_ijk[1] = ijk[1];
            owner_ijk[2] = ijk[2];
          }
        }
    int32_t xl[3] = {0, 0, 0};
    for (int a = 0; a < D; ++a) {
      int64_t v = G[a] - (int64_t)owner_ijk[a] * DD::ROOT_LEN;
      if (v == DD::ROOT_LEN) v = DD::ROOT_LEN - 1;  // p4est_node_clamp_inside
      xl[a] = (int32_t)v;
    }
    return (((uint64_t)owner) << tree_shift<D>()) | morton<D>(xl);
  };
#pragma omp parallel for schedule(static)
  for (long long ii = 0; ii < (long long)nl; ++ii)
    for (int c = 0; c < DD::CHILDREN; ++c) corner_key[(size_t)ii * DD::CHILDREN + c] = canon(leaves[(size_t)ii], c);
  auto A = std::make_shared<NodeArrays>();
  std::vector<uint64_t>& node_key = A->node_key;
  std::vector<int32_t>& node_tree = A->node_tree;
  std::vector<int32_t>& node_x = A->node_x;
  std::vector<int32_t>& local_nodes = A->local_nodes;
  node_key = corner_key;
  sort_u64(node_key);
  node_key.erase(std::unique(node_key.begin(), node_key.end()), node_key.end());
  const size_t nn = node_key.size();
  if (nn >= (size_t)INT32_MAX) throw std::runtime_error("too many nodes for 32-bit node indices");
  node_tree.resize(nn);
  node_x.resize(nn * D);
  const uint64_t mask = (((uint64_t)1) << tree_shift<D>()) - 1;
#pragma omp parallel for schedule(static)
  for (long long ii = 0; ii < (long long)nn; ++ii) {
    const uint64_t key = node_key[(size_t)ii];
    node_tree[(size_t)ii] = (int32_t)(key >> tree_shift<D>());
    const uint64_t m = key & mask;
    for (int a = 0; a < D; ++a) {
      uint64_t v = 0;
      for (int b = 0; b < DD::MAXLEVEL; ++b) v |= ((m >> (D * b + a)) & 1ull) << b;
      node_x[(size_t)ii * D + a] = (int32_t)v;
    }
  }
  local_nodes.resize(nl * DD::CHILDREN);
#pragma omp parallel for schedule(static)
  for (long long ii = 0; ii < (long long)(nl * DD::CHILDREN); ++ii) {
    auto it = std::lower_bound(node_key.begin(), node_key.end(), corner_key[(size_t)ii]);
    local_nodes[(size_t)ii] = (int32_t)(it - node_key.begin());
  }
  A->count = nn;
  nd = A;
  nodes_built = true;
  device.reset();
}

template <int D>
void Forest<D>::node_xyz(int32_t n, double* xyz) const {
  const NodeArrays& A = nd->host();
  const int32_t t = A.node_tree[n];
  for (int a = 0; a < D; ++a) {
    const int32_t v = A.node_x[(size_t)D * n + a];
    const double r = (v == DD::ROOT_LEN - 1) ? 1.0 : (double)v / (double)DD::ROOT_LEN;
    xyz[a] = (brick.tmax[3 * t + a] - brick.tmin[3 * t + a]) * r + brick.tmin[3 * t + a];
  }
}

template <int D>
int Forest<D>::max_level() const {
  int l = 0;
  for (const Quad& q : leaves) l = std::max(l, (int)q.level);
  return l;
}
template <int D>
int Forest<D>::min_level() const {
  int l = DD::MAXLEVEL;
  for (const Quad& q : leaves) l = std::min(l, (int)q.level);
  return l;
}

template <int D>
void Forest<D>::dxyz_min(double* dxyz) const {
  const int l = max_level();
  for (int a = 0; a < D; ++a) dxyz[a] = (brick.tmax[a] - brick.tmin[a]) / (double)(1 << l);
}

template struct Forest<2>;
template struct Forest<3>;

}  // namespace lsg
