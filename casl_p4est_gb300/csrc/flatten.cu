// Device flattener: the node-neighbour tables built on the GPU from the grid, so that a new grid
// (every step of a semi-Lagrangian regrid) does not wait on the host.
//
//   FP64 tables   construct_neighbors (src/my_p4est_node_neighbors.cpp:114-1201) per node through a
//                 view over device arrays, then the same row fill as the host flattener
//                 (fill_row64): one thread per node; correction records numbered by an exclusive
//                 scan in node order, as the host numbers them.
//   mixed tables  the classification, geometry classes and device node order of the host's
//                 build_tables32, restated with sorts and scans (see the second half of this file).
//
// Compiled with -fmad=false: every double expression rounds as the host flattener's
// (-ffp-contract=off) does, so the FP64 tables are bit-identical to the host's.
#include <cub/cub.cuh>

#include <algorithm>
#include <cstring>
#include <vector>

#include "flatten.hpp"
#include "tables.hpp"

namespace lsg {

// The grid as construct_neighbors_v reads it, over device arrays.
template <int D>
struct DeviceForestView {
  DForest<D> F;
  __device__ int32_t node_tree(int32_t n) const { return F.node_tree[n]; }
  __device__ int32_t node_x(int32_t n, int a) const { return F.node_x[(int64_t)D * n + a]; }
  __device__ void node_unclamped(int32_t n, int32_t* x) const {
    for (int a = 0; a < D; ++a) {
      const int32_t v = F.node_x[(int64_t)D * n + a];
      x[a] = (v == Dim<D>::ROOT_LEN - 1) ? Dim<D>::ROOT_LEN : v;
    }
  }
  __device__ int nt(int a) const { return F.n[a]; }
  __device__ int tree_ijk(int32_t t, int a) const { return F.tree_ijk[3 * t + a]; }
  __device__ int32_t tree_at(const int* ijk) const {
    return F.ijk_to_tree[(int64_t)F.n[0] * F.n[1] * (D == 3 ? ijk[2] : 0) + (int64_t)F.n[0] * ijk[1] + ijk[0]];
  }
  __device__ double tmin(int32_t t, int a) const { return F.tmin[3 * t + a]; }
  __device__ double tmax(int32_t t, int a) const { return F.tmax[3 * t + a]; }
  // leaf of `tree` containing the logical point X: coarse-cell table, then a binary search on the keys
  __device__ int32_t find_leaf(int32_t tree, const int32_t* X) const {
    int32_t c[3] = {0, 0, 0};
    for (int a = 0; a < D; ++a) c[a] = X[a] >> (Dim<D>::MAXLEVEL - F.L0);
    const int64_t idx = (int64_t)tree * F.ncoarse + (int64_t)morton<D>(c);
    int32_t lo = F.ctab[idx], hi = F.ctab[idx + 1];
    const uint64_t key = ((uint64_t)tree << tree_shift<D>()) | morton<D>(X);
    while (lo < hi) {
      const int32_t mid = (lo + hi + 1) >> 1;
      if (F.key[mid] <= key)
        lo = mid;
      else
        hi = mid - 1;
    }
    if (leaf_tree(lo) != tree) return -1;
    const int32_t h = quadrant_len(Dim<D>::MAXLEVEL, F.level[lo]);
    for (int a = 0; a < D; ++a) {
      const int32_t x0 = leaf_x(lo, a);
      if (X[a] < x0 || X[a] >= x0 + h) return -1;
    }
    return lo;
  }
  __device__ int leaf_level(int32_t q) const { return F.level[q]; }
  __device__ int32_t leaf_tree(int32_t q) const { return (int32_t)(F.key[q] >> tree_shift<D>()); }
  __device__ int32_t leaf_x(int32_t q, int a) const {
    int32_t x[3] = {0, 0, 0};
    unmorton<D>(F.key[q] & ((uint64_t(1) << tree_shift<D>()) - 1), x);
    return x[a];
  }
  __device__ int32_t local_node(int32_t q, int c) const { return F.local_nodes[(int64_t)Dim<D>::CHILDREN * q + c]; }
};

namespace {

constexpr int TPB = 256;

// irregular-group outputs of the mixed tables
struct DMixedOut {
  uint32_t* i_meta;
  uint32_t* i_cls;
  int32_t* i_nbr;
  float* i_wf;
  float* i_d;
  float* i_q;
  int32_t* i_cidx;
  double* i_wf64;
  double* i_d64;
  double* i_q64;
};
inline unsigned nblocks(int64_t n) { return (unsigned)((n + TPB - 1) / TPB); }

template <int D>
__global__ void __launch_bounds__(TPB) k_rows64(DForest<D> F, int32_t* __restrict__ nbr, double* __restrict__ w, double* __restrict__ nrm,
                                                double* __restrict__ d, double* __restrict__ q, uint8_t* __restrict__ wall,
                                                double* __restrict__ smin, int32_t* __restrict__ needs, double* __restrict__ cross,
                                                int* __restrict__ failed) {
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t N = F.N;
  if (n >= N) return;
  const DeviceForestView<D> V{F};
  Qnnn<D> rec;
  if (construct_neighbors_v<D>(V, (int32_t)n, rec)) {
    atomicAdd(failed, 1);
    needs[n] = 0;
    return;
  }
  const bool need = fill_row64<D>(rec, N, n, nbr, w, nrm, d, q, smin);
  needs[n] = need ? 1 : 0;
  // the cross terms of a node that needs a correction record, at its node index until the records
  // are numbered
  if (need) cross_terms<D>(rec, cross + (int64_t)6 * n);
  wall[n] = (uint8_t)wall_mask_v<D>(V, (int32_t)n);
}

// correction records numbered in node order (the exclusive scan of the needs flags)
__global__ void __launch_bounds__(TPB) k_crec64(int64_t N, const int32_t* __restrict__ needs, const int32_t* __restrict__ scan,
                                                const double* __restrict__ cross, int32_t* __restrict__ cidx, double* __restrict__ crec) {
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  if (!needs[n]) {
    cidx[n] = -1;
    return;
  }
  const int32_t r = scan[n];
  cidx[n] = r;
  for (int i = 0; i < 6; ++i) crec[(int64_t)6 * r + i] = cross[(int64_t)6 * n + i];
}

// ---- mixed tables -------------------------------------------------------------------------------
// level code of every neighbour distance: l with tree_size * 2^-l == d exactly (-1 if none), and the
// smallest code present (the base level)
template <int D>
__global__ void __launch_bounds__(TPB) k_lvl_codes(const double* __restrict__ d, int64_t N, double ts0, double ts1, double ts2,
                                                   int8_t* __restrict__ code, int* __restrict__ base_min) {
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int best = 64;
  for (int dir = 0; dir < 2 * D && n < N; ++dir) {
    const double dv = d[(int64_t)dir * N + n];
    const int a = dir >> 1;
    const double size = a == 0 ? ts0 : (a == 1 ? ts1 : ts2);
    int8_t c = -1;
    if (dv > 0) {
      int l = 0;
      double h = size;
      while (h > dv && l < 63) {
        h *= 0.5;
        ++l;
      }
      if (h == dv) {
        c = (int8_t)l;
        best = min(best, l);
      }
    }
    code[(int64_t)dir * N + n] = c;
  }
  // one atomic per warp
  for (int o = 16; o > 0; o >>= 1) best = min(best, __shfl_xor_sync(0xffffffffu, best, o));
  if ((threadIdx.x & 31) == 0 && best < 64) atomicMin(base_min, best);
}

// regular: no wall, no correction, one face node with weight 1 and no third-order factor per
// direction, every level code within [base, base + 15]; face-node counts of every node
template <int D>
__global__ void __launch_bounds__(TPB) k_classify(DTab64<D> T, const int8_t* __restrict__ code, int base, uint8_t* __restrict__ is_reg,
                                                  uint32_t* __restrict__ icount, int32_t* __restrict__ irr_flag) {
  constexpr int H = Dim<D>::HALF;
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t N = T.N;
  if (n >= N) return;
  uint32_t counts = 0;
  bool regular = T.wall[n] == 0 && T.cidx[n] < 0;
  for (int dir = 0; dir < 2 * D; ++dir) {
    int cnt = 0;
    for (int k = 0; k < H; ++k)
      if (T.nbr[(int64_t)(dir * H + k) * N + n] >= 0) cnt = k + 1;
    counts |= (uint32_t)(cnt - 1) << (2 * dir);
    if (cnt != 1) regular = false;
    for (int j = 0; j < D - 1; ++j)
      if (T.q[(int64_t)(dir * (D - 1) + j) * N + n] != 0.0) regular = false;
    const int lc = code[(int64_t)dir * N + n];
    if (lc < base || lc > base + 15) regular = false;
  }
  icount[n] = counts;
  is_reg[n] = regular ? 1 : 0;
  irr_flag[n] = regular ? 0 : 1;
}

// first position of every class in the hash-grouped order
__global__ void __launch_bounds__(TPB) k_class_starts(const int32_t* __restrict__ flag, const int32_t* __restrict__ excl, int64_t nI,
                                                      int32_t* __restrict__ start) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nI && flag[i]) start[excl[i]] = (int32_t)i;
}

// renumber the classes (new id and shift of each class's block of the irregular order)
__global__ void __launch_bounds__(TPB) k_class_renumber(const int32_t* __restrict__ irr_node, int64_t nI, const int32_t* __restrict__ newid,
                                                        const int32_t* __restrict__ shift, int32_t* __restrict__ node_cls,
                                                        int32_t* __restrict__ irr_rank) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nI) return;
  const int32_t n = irr_node[k];
  const int32_t c = node_cls[n];
  node_cls[n] = newid[c];
  irr_rank[n] += shift[c];
}

__device__ __forceinline__ uint64_t mix64(uint64_t h) {
  h ^= h >> 33;
  h *= 0xff51afd7ed558ccdull;
  h ^= h >> 33;
  h *= 0xc4ceb9fe1a85ec53ull;
  h ^= h >> 33;
  return h;
}

// geometry class record of every irregular node (slot k = its rank among the irregular nodes in
// node order), with a hash of its bits for grouping equal records
template <int D>
__global__ void __launch_bounds__(TPB) k_records(DTab64<D> T, const uint8_t* __restrict__ is_reg, const uint32_t* __restrict__ icount,
                                                 const int32_t* __restrict__ irr_pos, double* __restrict__ rec, uint64_t* __restrict__ hash,
                                                 int32_t* __restrict__ slot, int32_t* __restrict__ irr_node) {
  constexpr int H = Dim<D>::HALF;
  constexpr int CW = cls_words<D>();
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t N = T.N;
  if (n >= N || is_reg[n]) return;
  const int32_t k = irr_pos[n];
  const uint32_t counts = icount[n];
  double r[CW];
  for (int w = 0; w < CW; ++w) r[w] = 0.0;
  const uint32_t meta = counts | ((T.cidx[n] >= 0) ? (1u << 16) : 0u) | ((uint32_t)T.wall[n] << 24);
  r[0] = (double)meta;
  for (int dir = 0; dir < 2 * D; ++dir) {
    const int cnt = (int)((counts >> (2 * dir)) & 3) + 1;
    r[1 + dir] = T.d[(int64_t)dir * N + n];
    const double nr = T.nrm[(int64_t)dir * N + n];
    for (int kk = 0; kk < H; ++kk) r[1 + 2 * D + dir * H + kk] = kk < cnt ? T.w[(int64_t)(dir * H + kk) * N + n] / nr : 0.0;
    for (int j = 0; j < D - 1; ++j) r[1 + 2 * D + 2 * D * H + dir * (D - 1) + j] = T.q[(int64_t)(dir * (D - 1) + j) * N + n];
  }
  double* cm = r + 1 + 2 * D + 2 * D * H + 2 * D * (D - 1);
  for (int c = 0; c < D; ++c) {
    double e[3] = {0, 0, 0};
    e[c] = 1.0;
    if (T.cidx[n] >= 0) apply_correction<D>(T.crec + (int64_t)6 * T.cidx[n], e);
    for (int rr = 0; rr < D; ++rr) cm[rr * D + c] = e[rr];
  }
  uint64_t h = 0x9E3779B97F4A7C15ull;
  for (int w = 0; w < CW; ++w) {
    const uint64_t b = (uint64_t)__double_as_longlong(r[w]);
    rec[(int64_t)k * CW + w] = r[w];
    h = mix64(h ^ b) + 0x9E3779B97F4A7C15ull;
  }
  hash[k] = h;
  slot[k] = k;
  irr_node[k] = (int32_t)n;
}

// first of each run of equal records in hash order
template <int D>
__global__ void __launch_bounds__(TPB) k_class_flags(const double* __restrict__ rec, const int32_t* __restrict__ sorted_slot, int64_t nI,
                                                     int32_t* __restrict__ flag) {
  constexpr int CW = cls_words<D>();
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nI) return;
  int f = 1;
  if (i > 0) {
    const double* a = rec + (int64_t)sorted_slot[i] * CW;
    const double* b = rec + (int64_t)sorted_slot[i - 1] * CW;
    f = 0;
    for (int w = 0; w < CW; ++w)
      if (__double_as_longlong(a[w]) != __double_as_longlong(b[w])) f = 1;
  }
  flag[i] = f;
}

// class index of every irregular node, the class records (FP64, and FP32 with the meta word as bits),
// and each irregular node's rank in (class, node) order
template <int D>
__global__ void __launch_bounds__(TPB) k_class_write(const double* __restrict__ rec, const int32_t* __restrict__ sorted_slot,
                                                     const int32_t* __restrict__ irr_node, const int32_t* __restrict__ flag,
                                                     const int32_t* __restrict__ excl, int64_t nI, double* __restrict__ cls64,
                                                     float* __restrict__ cls32, int32_t* __restrict__ node_cls, int32_t* __restrict__ irr_rank) {
  constexpr int CW = cls_words<D>();
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nI) return;
  const int32_t c = excl[i] + flag[i] - 1;
  const int32_t k = sorted_slot[i];
  const int32_t n = irr_node[k];
  node_cls[n] = c;
  irr_rank[n] = (int32_t)i;
  if (flag[i]) {
    const double* r = rec + (int64_t)k * CW;
    for (int w = 0; w < CW; ++w) {
      cls64[(int64_t)c * CW + w] = r[w];
      cls32[(int64_t)c * CW + w] = (float)r[w];
    }
    const uint32_t meta = (uint32_t)r[0];
    cls32[(int64_t)c * CW] = __uint_as_float(meta);
  }
}

// regular nodes: second neighbour along each direction (the face node's own face node further out,
// when the face node is regular and points back), outer level codes, and the uniform flag
// (every own and outer code equal); face nodes without a recorded second neighbour join the extended
// second-derivative set. meta2: far codes | all << 31 | uniform << 30.
template <int D>
__global__ void __launch_bounds__(TPB) k_regular_info(DTab64<D> T, const int8_t* __restrict__ code, int base, const uint8_t* __restrict__ is_reg,
                                                      uint32_t* __restrict__ meta2, uint8_t* __restrict__ in_x) {
  constexpr int H = Dim<D>::HALF;
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t N = T.N;
  if (n >= N || !is_reg[n]) return;
  uint32_t far = 0;
  bool all = true;
  for (int dir = 0; dir < 2 * D; ++dir) {
    const int32_t j = T.nbr[(int64_t)(dir * H) * N + n];
    const int back = dir ^ 1;
    if (is_reg[j] && T.nbr[(int64_t)(back * H) * N + j] == (int32_t)n) {
      far |= ((uint32_t)(code[(int64_t)dir * N + j] - base) & 15u) << (4 * dir);
    } else {
      all = false;
      if (is_reg[j]) in_x[j] = 1;
    }
  }
  bool uniform = all;
  const int c0 = code[n] - base;
  for (int dir = 0; dir < 2 * D && uniform; ++dir)
    uniform = (code[(int64_t)dir * N + n] - base) == c0 && (int)((far >> (4 * dir)) & 15u) == c0;
  meta2[n] = far | (all ? (1u << 31) : 0u) | (uniform ? (1u << 30) : 0u);
}

// regular face nodes of irregular nodes join the extended set
template <int D>
__global__ void __launch_bounds__(TPB) k_mark_irregular(DTab64<D> T, const uint8_t* __restrict__ is_reg, uint8_t* __restrict__ in_x) {
  constexpr int NS = 2 * D * Dim<D>::HALF;
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t N = T.N;
  if (n >= N || is_reg[n]) return;
  for (int sl = 0; sl < NS; ++sl) {
    const int32_t j = T.nbr[(int64_t)sl * N + n];
    if (j >= 0 && is_reg[j]) in_x[j] = 1;
  }
}

// device order key: regular groups [uniform outside the set | uniform in the set | other in the set |
// other outside] in node order, then the irregular nodes by (class, node)
__global__ void __launch_bounds__(TPB) k_perm_keys(const uint8_t* __restrict__ is_reg, const uint32_t* __restrict__ meta2,
                                                   const uint8_t* __restrict__ in_x, const int32_t* __restrict__ irr_rank, int64_t N,
                                                   uint64_t* __restrict__ keys, int32_t* __restrict__ vals,
                                                   unsigned long long* __restrict__ counts) {
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  uint64_t group = 5;  // none: past the end
  if (n < N) {
    uint64_t pos;
    if (is_reg[n]) {
      const bool uni = (meta2[n] >> 30) & 1u, inset = in_x[n] != 0;
      group = uni ? (inset ? 1 : 0) : (inset ? 2 : 3);
      pos = (uint64_t)n;
    } else {
      group = 4;
      pos = (uint64_t)irr_rank[n];
    }
    keys[n] = (group << 40) | pos;
    vals[n] = (int32_t)n;
  }
  // group sizes: one atomic per warp and group
  for (int g = 0; g < 5; ++g) {
    const unsigned c = __popc(__ballot_sync(0xffffffffu, group == (uint64_t)g));
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(counts + g, (unsigned long long)c);
  }
}

__global__ void __launch_bounds__(TPB) k_iperm(const int32_t* __restrict__ perm, int64_t N, int32_t* __restrict__ iperm) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < N) iperm[perm[i]] = (int32_t)i;
}

template <int D>
__global__ void __launch_bounds__(TPB) k_fill_regular(DTab64<D> T, const int8_t* __restrict__ code, int base,
                                                      const uint8_t* __restrict__ is_reg, const uint32_t* __restrict__ meta2n,
                                                      const int32_t* __restrict__ perm, const int32_t* __restrict__ iperm, int64_t nR,
                                                      uint32_t* __restrict__ r_meta, int32_t* __restrict__ r_nbr, int32_t* __restrict__ r_nbr2,
                                                      uint32_t* __restrict__ r_meta2) {
  constexpr int H = Dim<D>::HALF;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nR) return;
  const int64_t N = T.N;
  const int64_t n = perm[i];
  uint32_t codes = 0;
  for (int dir = 0; dir < 2 * D; ++dir) {
    codes |= (uint32_t)(code[(int64_t)dir * N + n] - base) << (4 * dir);
    const int32_t j = T.nbr[(int64_t)(dir * H) * N + n];
    r_nbr[(int64_t)dir * nR + i] = iperm[j];
    const bool two = is_reg[j] && T.nbr[(int64_t)((dir ^ 1) * H) * N + j] == (int32_t)n;
    r_nbr2[(int64_t)dir * nR + i] = two ? iperm[T.nbr[(int64_t)(dir * H) * N + j]] : -1;
  }
  r_meta[i] = codes;
  r_meta2[i] = meta2n[n];
}

template <int D>
__global__ void __launch_bounds__(TPB) k_fill_irregular(DTab64<D> T, const uint32_t* __restrict__ icount, const int32_t* __restrict__ node_cls,
                                                        const int32_t* __restrict__ perm, const int32_t* __restrict__ iperm, int64_t nR,
                                                        DMixedOut O) {
  constexpr int H = Dim<D>::HALF;
  const int64_t N = T.N;
  const int64_t nI = N - nR;
  const int64_t ii = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (ii >= nI) return;
  const int64_t n = perm[nR + ii];
  uint32_t meta = icount[n];
  if (T.cidx[n] >= 0) meta |= 1u << 16;
  meta |= (uint32_t)T.wall[n] << 24;
  O.i_meta[ii] = meta;
  O.i_cls[ii] = (uint32_t)node_cls[n];
  for (int dir = 0; dir < 2 * D; ++dir) {
    const int cnt = (int)((icount[n] >> (2 * dir)) & 3) + 1;
    const double nr = T.nrm[(int64_t)dir * N + n];
    for (int k = 0; k < H; ++k) {
      const int32_t nb = T.nbr[(int64_t)(dir * H + k) * N + n];
      O.i_nbr[(int64_t)(dir * H + k) * nI + ii] = k < cnt ? iperm[nb] : iperm[T.nbr[(int64_t)(dir * H) * N + n]];
      const double wn = k < cnt ? T.w[(int64_t)(dir * H + k) * N + n] / nr : 0.0;
      O.i_wf[(int64_t)(dir * H + k) * nI + ii] = (float)wn;
      O.i_wf64[(int64_t)(dir * H + k) * nI + ii] = wn;
    }
    O.i_d[(int64_t)dir * nI + ii] = (float)T.d[(int64_t)dir * N + n];
    O.i_d64[(int64_t)dir * nI + ii] = T.d[(int64_t)dir * N + n];
    for (int j = 0; j < D - 1; ++j) {
      O.i_q[(int64_t)(dir * (D - 1) + j) * nI + ii] = (float)T.q[(int64_t)(dir * (D - 1) + j) * N + n];
      O.i_q64[(int64_t)(dir * (D - 1) + j) * nI + ii] = T.q[(int64_t)(dir * (D - 1) + j) * N + n];
    }
  }
  O.i_cidx[ii] = T.cidx[n];
}

// correction matrices: correct_naive_second_derivatives applied to the unit vectors
template <int D>
__global__ void __launch_bounds__(TPB) k_corr(const double* __restrict__ crec, int64_t R, float* __restrict__ corr, double* __restrict__ corr64) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= R) return;
  for (int c = 0; c < D; ++c) {
    double e[3] = {0, 0, 0};
    e[c] = 1.0;
    apply_correction<D>(crec + 6 * r, e);
    for (int rr = 0; rr < D; ++rr) {
      corr[(int64_t)D * D * r + D * rr + c] = (float)e[rr];
      corr64[(int64_t)D * D * r + D * rr + c] = e[rr];
    }
  }
}

// ---- node numbering ----------------------------------------------------------------------------
// canonical key of every leaf corner: the corner in global logical coordinates, owned by the lowest
// tree touching it and clamped inside that tree (p4est_node_canonicalize / p4est_node_clamp_inside)
template <int D>
__global__ void __launch_bounds__(TPB) k_corner_keys(const uint64_t* __restrict__ leaf_key, const int8_t* __restrict__ level, int64_t nl,
                                                     int n0, int n1, int n2, const int32_t* __restrict__ tree_ijk,
                                                     const int32_t* __restrict__ ijk_to_tree, uint64_t* __restrict__ corner_key) {
  using DD = Dim<D>;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nl * DD::CHILDREN) return;
  const int64_t ii = e / DD::CHILDREN;
  const int c = (int)(e % DD::CHILDREN);
  const uint64_t lk = leaf_key[ii];
  const int32_t tree = (int32_t)(lk >> tree_shift<D>());
  int32_t x[3] = {0, 0, 0};
  unmorton<D>(lk & ((uint64_t(1) << tree_shift<D>()) - 1), x);
  const int32_t h = quadrant_len(DD::MAXLEVEL, level[ii]);
  const int nn[3] = {n0, n1, n2};
  int64_t G[3] = {0, 0, 0};
  for (int a = 0; a < D; ++a) G[a] = (int64_t)tree_ijk[3 * tree + a] * DD::ROOT_LEN + x[a] + (((c >> a) & 1) ? h : 0);
  int cand[3][2] = {{0, 0}, {0, 0}, {0, 0}};
  int ncand[3] = {1, 1, 1};
  for (int a = 0; a < D; ++a) {
    const int64_t L = (int64_t)nn[a] * DD::ROOT_LEN;
    const int64_t t = G[a] / DD::ROOT_LEN;
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
        const int ijk[3] = {cand[0][i], cand[1][j], cand[2][k]};
        const int32_t t = ijk_to_tree[(int64_t)n0 * n1 * ijk[2] + (int64_t)n0 * ijk[1] + ijk[0]];
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
    if (v == DD::ROOT_LEN) v = DD::ROOT_LEN - 1;
    xl[a] = (int32_t)v;
  }
  corner_key[e] = (((uint64_t)owner) << tree_shift<D>()) | morton<D>(xl);
}

template <int D>
__global__ void __launch_bounds__(TPB) k_decode_nodes(const uint64_t* __restrict__ node_key, int64_t nn, int32_t* __restrict__ node_tree,
                                                      int32_t* __restrict__ node_x) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nn) return;
  const uint64_t key = node_key[i];
  node_tree[i] = (int32_t)(key >> tree_shift<D>());
  int32_t x[3] = {0, 0, 0};
  unmorton<D>(key & ((uint64_t(1) << tree_shift<D>()) - 1), x);
  for (int a = 0; a < D; ++a) node_x[i * D + a] = x[a];
}

// node index of every leaf corner: position of its key among the sorted unique node keys
__global__ void __launch_bounds__(TPB) k_local_nodes(const uint64_t* __restrict__ corner_key, int64_t nc, const uint64_t* __restrict__ node_key,
                                                     int64_t nn, int32_t* __restrict__ local_nodes) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nc) return;
  const uint64_t k = corner_key[e];
  int64_t lo = 0, hi = nn;
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (node_key[mid] < k)
      lo = mid + 1;
    else
      hi = mid;
  }
  local_nodes[e] = (int32_t)lo;
}

// splitting_criteria_tag_t::tag_quadrant from the node values (same rule as Forest::tag_refine_coarsen)
template <int D>
__global__ void __launch_bounds__(TPB) k_tag_leaves(const uint64_t* __restrict__ leaf_key, const int8_t* __restrict__ level, int64_t nl,
                                                    const int32_t* __restrict__ local_nodes, const double* __restrict__ tmin_,
                                                    const double* __restrict__ tmax_, const double* __restrict__ phi, int min_lvl, int max_lvl,
                                                    double lip, double band, int8_t* __restrict__ tag) {
  using DD = Dim<D>;
  const int64_t ii = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (ii >= nl) return;
  const int lv = level[ii];
  if (lv < min_lvl) {
    tag[ii] = 1;
    return;
  }
  if (lv > max_lvl) {
    tag[ii] = -1;
    return;
  }
  const int32_t tree = (int32_t)(leaf_key[ii] >> tree_shift<D>());
  double f[DD::CHILDREN];
  for (int c = 0; c < DD::CHILDREN; ++c) f[c] = phi[local_nodes[ii * DD::CHILDREN + c]];
  const double* tmn = tmin_ + 3 * tree;
  const double* tmx = tmax_ + 3 * tree;
  const double dmin = (double)quadrant_len(DD::MAXLEVEL, lv) / (double)DD::ROOT_LEN;
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
    refine = refine || (lv < max_lvl && (fabs(f[i]) - band_real <= 0.5 * lip * d ||
                                         (i == 0 ? false : ((f[i] > 0.0 && f[0] <= 0.0) || (f[i] <= 0.0 && f[0] > 0.0)))));
    coarsen = coarsen && lv > min_lvl && fabs(f[i]) - band_real >= 1.0 * lip * d &&
              (i == 0 ? true : ((f[i] > 0.0 && f[0] > 0.0) || (f[i] <= 0.0 && f[0] <= 0.0)));
  }
  tag[ii] = refine ? 1 : (coarsen ? -1 : 0);
}

}  // namespace

// One device allocation carved into the temporaries of a build (one allocator call instead of one per
// temporary). Pieces start on 256-byte boundaries.
struct Arena {
  DevBuf<uint8_t> buf;
  size_t off = 0;
  template <typename T>
  static size_t bytes(size_t n) {
    return (n * sizeof(T) + 255) & ~(size_t)255;
  }
  void reserve(size_t total) {
    buf.alloc(total + 256);
    off = 0;
  }
  template <typename T>
  T* take(size_t n) {
    const size_t b = bytes<T>(n);
    if (off + b > buf.n) throw std::logic_error("device flattener: scratch arena too small");
    T* p = reinterpret_cast<T*>(buf.p + off);
    off += b;
    return p;
  }
};

// exclusive prefix sum of n int32 values (CUB)
static void exclusive_sum(const int32_t* in, int32_t* out, int64_t n, void* temp, size_t temp_bytes, cudaStream_t s) {
  if (n == 0) return;
  size_t bytes = 0;
  cub::DeviceScan::ExclusiveSum(nullptr, bytes, in, out, (int)n, s);
  if (bytes > temp_bytes) throw std::logic_error("device flattener: scan scratch too small");
  cuda_check(cub::DeviceScan::ExclusiveSum(temp, bytes, in, out, (int)n, s), "exclusive scan");
}

// total of a 0/1 flag array given its exclusive scan
static int64_t scan_total(const int32_t* flags, const int32_t* excl, int64_t n, cudaStream_t s) {
  if (n == 0) return 0;
  int32_t a = 0, b = 0;
  cuda_check(cudaMemcpyAsync(&a, flags + n - 1, sizeof(int32_t), cudaMemcpyDeviceToHost, s), "D2H");
  cuda_check(cudaMemcpyAsync(&b, excl + n - 1, sizeof(int32_t), cudaMemcpyDeviceToHost, s), "D2H");
  cuda_check(cudaStreamSynchronize(s), "scan total");
  return (int64_t)a + b;
}

template <int D>
int64_t build_tables64_device(const DForest<D>& F, const Tab64Dev<D>& out, cudaStream_t s) {
  constexpr int NS = 2 * D * Dim<D>::HALF;
  const int64_t N = F.N;
  out.nbr->alloc((size_t)NS * N);
  out.w->alloc((size_t)NS * N);
  out.nrm->alloc((size_t)2 * D * N);
  out.d->alloc((size_t)2 * D * N);
  out.q->alloc((size_t)2 * D * (D - 1) * N);
  out.cidx->alloc((size_t)N);
  out.wall->alloc((size_t)N);
  out.smin->alloc((size_t)N);
  size_t tb = 0;
  cub::DeviceScan::ExclusiveSum(nullptr, tb, (const int32_t*)nullptr, (int32_t*)nullptr, (int)N, s);
  tb += 1;
  Arena A;
  A.reserve(2 * Arena::bytes<int32_t>((size_t)N + 1) + Arena::bytes<double>((size_t)6 * N + 1) + Arena::bytes<int>(1) +
            Arena::bytes<uint8_t>(tb));
  int32_t* needs = A.take<int32_t>((size_t)N + 1);
  int32_t* scan = A.take<int32_t>((size_t)N + 1);
  double* cross = A.take<double>((size_t)6 * N + 1);
  int* failed = A.take<int>(1);
  void* temp = A.take<uint8_t>(tb);
  cuda_check(cudaMemsetAsync(failed, 0, sizeof(int), s), "memset");
  if (N) k_rows64<D><<<nblocks(N), TPB, 0, s>>>(F, out.nbr->p, out.w->p, out.nrm->p, out.d->p, out.q->p, out.wall->p, out.smin->p, needs,
                                                cross, failed);
  cuda_check(cudaGetLastError(), "device flattener rows");
  exclusive_sum(needs, scan, N, temp, tb, s);
  int nfail = 0;
  cuda_check(cudaMemcpyAsync(&nfail, failed, sizeof(int), cudaMemcpyDeviceToHost, s), "D2H");
  const int64_t R = scan_total(needs, scan, N, s);
  if (nfail) throw std::runtime_error("node neighbours: incomplete stencil in a single-process forest");
  out.crec->alloc((size_t)6 * R + 6);
  if (N) k_crec64<<<nblocks(N), TPB, 0, s>>>(N, needs, scan, cross, out.cidx->p, out.crec->p);
  cuda_check(cudaGetLastError(), "device flattener corrections");
  cuda_check(cudaStreamSynchronize(s), "device flattener");
  return R;
}

template <int D>
void build_mixed_device(const DTab64<D>& T, int64_t R, const double* ts, MixedDev<D>& M, cudaStream_t s) {
  constexpr int H = Dim<D>::HALF;
  constexpr int NS = 2 * D * H;
  constexpr int CW = cls_words<D>();
  const int64_t N = T.N;
  // temporaries sized by N, carved from one allocation
  size_t tb1 = 0, tsort = 0;
  cub::DeviceScan::ExclusiveSum(nullptr, tb1, (const int32_t*)nullptr, (int32_t*)nullptr, (int)N, s);
  cub::DeviceRadixSort::SortPairs(nullptr, tsort, (const uint64_t*)nullptr, (uint64_t*)nullptr, (const int32_t*)nullptr, (int32_t*)nullptr,
                                  (int)N, 0, 43, s);
  tb1 = std::max(tb1, tsort) + 1;
  const size_t N1 = (size_t)N + 1;
  Arena A;
  A.reserve(Arena::bytes<int8_t>((size_t)2 * D * N + 1) + Arena::bytes<int>(1) + 2 * Arena::bytes<uint8_t>(N1) +
            2 * Arena::bytes<uint32_t>(N1) + 5 * Arena::bytes<int32_t>(N1) + 2 * Arena::bytes<uint64_t>(N1) +
            Arena::bytes<unsigned long long>(5) + Arena::bytes<uint8_t>(tb1));
  int8_t* code = A.take<int8_t>((size_t)2 * D * N + 1);
  int* base_min = A.take<int>(1);
  uint8_t* is_reg = A.take<uint8_t>(N1);
  uint8_t* in_x = A.take<uint8_t>(N1);
  uint32_t* icount = A.take<uint32_t>(N1);
  uint32_t* meta2n = A.take<uint32_t>(N1);
  int32_t* irr_flag = A.take<int32_t>(N1);
  int32_t* irr_pos = A.take<int32_t>(N1);
  int32_t* node_cls = A.take<int32_t>(N1);
  int32_t* irr_rank = A.take<int32_t>(N1);
  int32_t* vals = A.take<int32_t>(N1);
  uint64_t* keys = A.take<uint64_t>(N1);
  uint64_t* keys_sorted = A.take<uint64_t>(N1);
  unsigned long long* counts = A.take<unsigned long long>(5);
  void* temp1 = A.take<uint8_t>(tb1);
  // base level
  int h_base = 64;
  cuda_check(cudaMemcpyAsync(base_min, &h_base, sizeof(int), cudaMemcpyHostToDevice, s), "H2D");
  if (N) k_lvl_codes<D><<<nblocks(N), TPB, 0, s>>>(T.d, N, ts[0], ts[1], D == 3 ? ts[2] : 1.0, code, base_min);
  cuda_check(cudaMemcpyAsync(&h_base, base_min, sizeof(int), cudaMemcpyDeviceToHost, s), "D2H");
  cuda_check(cudaStreamSynchronize(s), "base level");
  const int base = h_base == 64 ? 0 : h_base;
  M.base = base;
  // classification
  if (N) k_classify<D><<<nblocks(N), TPB, 0, s>>>(T, code, base, is_reg, icount, irr_flag);
  exclusive_sum(irr_flag, irr_pos, N, temp1, tb1, s);
  const int64_t nI = scan_total(irr_flag, irr_pos, N, s);
  const int64_t nR = N - nI;
  // geometry classes: records, grouped by hash (stable: node order inside a group), runs of equal records;
  // temporaries sized by the irregular count, carved from a second allocation
  size_t tb2 = 0, tcls = 0;
  cub::DeviceScan::ExclusiveSum(nullptr, tb2, (const int32_t*)nullptr, (int32_t*)nullptr, (int)nI, s);
  cub::DeviceRadixSort::SortPairs(nullptr, tcls, (const uint64_t*)nullptr, (uint64_t*)nullptr, (const int32_t*)nullptr, (int32_t*)nullptr,
                                  (int)nI, 0, 64, s);
  tb2 = std::max(tb2, tcls) + 1;
  const size_t I1 = (size_t)nI + 1;
  Arena B;
  B.reserve(Arena::bytes<double>((size_t)nI * CW + 1) + 2 * Arena::bytes<uint64_t>(I1) + 5 * Arena::bytes<int32_t>(I1) +
            Arena::bytes<uint8_t>(tb2));
  double* rec = B.take<double>((size_t)nI * CW + 1);
  uint64_t* hash = B.take<uint64_t>(I1);
  uint64_t* hash_sorted = B.take<uint64_t>(I1);
  int32_t* slot = B.take<int32_t>(I1);
  int32_t* slot_sorted = B.take<int32_t>(I1);
  int32_t* irr_node = B.take<int32_t>(I1);
  int32_t* flag = B.take<int32_t>(I1);
  int32_t* excl = B.take<int32_t>(I1);
  void* temp2 = B.take<uint8_t>(tb2);
  int64_t ncls = 0;
  if (nI) {
    k_records<D><<<nblocks(N), TPB, 0, s>>>(T, is_reg, icount, irr_pos, rec, hash, slot, irr_node);
    cuda_check(cub::DeviceRadixSort::SortPairs(temp2, tcls, hash, hash_sorted, slot, slot_sorted, (int)nI, 0, 64, s), "class sort");
    k_class_flags<D><<<nblocks(nI), TPB, 0, s>>>(rec, slot_sorted, nI, flag);
    exclusive_sum(flag, excl, nI, temp2, tb2, s);
    ncls = scan_total(flag, excl, nI, s);
  }
  M.cls32->alloc((size_t)ncls * CW + 1);
  DevBuf<double> cls64;
  cls64.alloc((size_t)ncls * CW + 1);
  if (nI)
    k_class_write<D><<<nblocks(nI), TPB, 0, s>>>(rec, slot_sorted, irr_node, flag, excl, nI, cls64.p, M.cls32->p, node_cls, irr_rank);
  // classes renumbered in the host build's order (records compared as bytes), which also orders the
  // irregular group: each class's block of (class, node) positions moves as a whole
  if (ncls > 1) {
    std::vector<double> h64((size_t)ncls * CW);
    std::vector<float> h32((size_t)ncls * CW);
    std::vector<int32_t> start((size_t)ncls);
    DevBuf<int32_t> dstart, dnew, dshift;
    dstart.alloc((size_t)ncls);
    k_class_starts<<<nblocks(nI), TPB, 0, s>>>(flag, excl, nI, dstart.p);
    cuda_check(cudaGetLastError(), "class starts");
    cuda_check(cudaMemcpyAsync(h64.data(), cls64.p, h64.size() * sizeof(double), cudaMemcpyDeviceToHost, s), "D2H");
    cuda_check(cudaMemcpyAsync(h32.data(), M.cls32->p, h32.size() * sizeof(float), cudaMemcpyDeviceToHost, s), "D2H");
    cuda_check(cudaMemcpyAsync(start.data(), dstart.p, start.size() * sizeof(int32_t), cudaMemcpyDeviceToHost, s), "D2H");
    cuda_check(cudaStreamSynchronize(s), "class records");
    std::vector<int32_t> order((size_t)ncls), newid((size_t)ncls), shift((size_t)ncls);
    for (int64_t c = 0; c < ncls; ++c) order[(size_t)c] = (int32_t)c;
    std::sort(order.begin(), order.end(), [&](int32_t a, int32_t b) {
      return memcmp(&h64[(size_t)a * CW], &h64[(size_t)b * CW], CW * sizeof(double)) < 0;
    });
    std::vector<float> n32(h32.size());
    int64_t pos = 0;
    for (int64_t p = 0; p < ncls; ++p) {
      const int32_t c = order[(size_t)p];
      const int64_t cnt = (c + 1 < ncls ? start[(size_t)c + 1] : nI) - start[(size_t)c];
      newid[(size_t)c] = (int32_t)p;
      shift[(size_t)c] = (int32_t)(pos - start[(size_t)c]);
      pos += cnt;
      memcpy(&n32[(size_t)p * CW], &h32[(size_t)c * CW], CW * sizeof(float));
    }
    dnew.upload(newid, s);
    dshift.upload(shift, s);
    cuda_check(cudaMemcpyAsync(M.cls32->p, n32.data(), n32.size() * sizeof(float), cudaMemcpyHostToDevice, s), "H2D");
    k_class_renumber<<<nblocks(nI), TPB, 0, s>>>(irr_node, nI, dnew.p, dshift.p, node_cls, irr_rank);
    cuda_check(cudaGetLastError(), "class renumbering");
    cuda_check(cudaStreamSynchronize(s), "class renumbering");  // the host vectors above go out of scope
  }
  M.ncls = ncls;
  // regular nodes: second neighbours, uniform flag, extended set
  cuda_check(cudaMemsetAsync(in_x, 0, N1, s), "memset");
  cuda_check(cudaMemsetAsync(meta2n, 0, N1 * sizeof(uint32_t), s), "memset");
  cuda_check(cudaMemsetAsync(counts, 0, 5 * sizeof(unsigned long long), s), "memset");
  if (N) {
    k_regular_info<D><<<nblocks(N), TPB, 0, s>>>(T, code, base, is_reg, meta2n, in_x);
    k_mark_irregular<D><<<nblocks(N), TPB, 0, s>>>(T, is_reg, in_x);
  }
  // device order
  M.perm->alloc((size_t)N);
  M.iperm->alloc((size_t)N);
  if (N) {
    k_perm_keys<<<nblocks(N), TPB, 0, s>>>(is_reg, meta2n, in_x, irr_rank, N, keys, vals, counts);
    cuda_check(cub::DeviceRadixSort::SortPairs(temp1, tsort, keys, keys_sorted, vals, M.perm->p, (int)N, 0, 43, s), "order sort");
    k_iperm<<<nblocks(N), TPB, 0, s>>>(M.perm->p, N, M.iperm->p);
  }
  unsigned long long g[5] = {0, 0, 0, 0, 0};
  cuda_check(cudaMemcpyAsync(g, counts, sizeof(g), cudaMemcpyDeviceToHost, s), "D2H");
  cuda_check(cudaStreamSynchronize(s), "group counts");
  if ((int64_t)(g[0] + g[1] + g[2] + g[3]) != nR || (int64_t)g[4] != nI) throw std::runtime_error("device flattener: group counts");
  M.nR = nR;
  M.nI = nI;
  M.nU = (int64_t)(g[0] + g[1]);
  M.x_first = (int64_t)g[0];
  M.nX = (int64_t)(g[1] + g[2]);
  // regular group
  M.r_meta->alloc((size_t)nR + 1);
  M.r_nbr->alloc((size_t)2 * D * nR + 1);
  M.r_nbr2->alloc((size_t)2 * D * nR + 1);
  M.r_meta2->alloc((size_t)nR + 1);
  if (nR)
    k_fill_regular<D><<<nblocks(nR), TPB, 0, s>>>(T, code, base, is_reg, meta2n, M.perm->p, M.iperm->p, nR, M.r_meta->p, M.r_nbr->p,
                                                  M.r_nbr2->p, M.r_meta2->p);
  // irregular group
  M.i_meta->alloc((size_t)nI + 1);
  M.i_cls->alloc((size_t)nI + 1);
  M.i_nbr->alloc((size_t)NS * nI + 1);
  M.i_wf->alloc((size_t)NS * nI + 1);
  M.i_d->alloc((size_t)2 * D * nI + 1);
  M.i_q->alloc((size_t)2 * D * (D - 1) * nI + 1);
  M.i_cidx->alloc((size_t)nI + 1);
  M.i_wf64->alloc((size_t)NS * nI + 1);
  M.i_d64->alloc((size_t)2 * D * nI + 1);
  M.i_q64->alloc((size_t)2 * D * (D - 1) * nI + 1);
  DMixedOut O{M.i_meta->p, M.i_cls->p, M.i_nbr->p, M.i_wf->p, M.i_d->p, M.i_q->p, M.i_cidx->p, M.i_wf64->p, M.i_d64->p, M.i_q64->p};
  if (nI) k_fill_irregular<D><<<nblocks(nI), TPB, 0, s>>>(T, icount, node_cls, M.perm->p, M.iperm->p, nR, O);
  // correction matrices
  M.corr->alloc((size_t)D * D * R + 1);
  M.corr64->alloc((size_t)D * D * R + 1);
  if (R) k_corr<D><<<nblocks(R), TPB, 0, s>>>(T.crec, R, M.corr->p, M.corr64->p);
  cuda_check(cudaGetLastError(), "device flattener (mixed)");
  cuda_check(cudaStreamSynchronize(s), "device flattener (mixed)");
}

template <int D>
__global__ void __launch_bounds__(TPB) k_node_xyz(const int32_t* __restrict__ node_tree, const int32_t* __restrict__ node_x, int64_t nn,
                                                  const double* __restrict__ tmin, const double* __restrict__ tmax, double* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nn) return;
  const int32_t t = node_tree[i];
  for (int a = 0; a < D; ++a) {
    const int32_t v = node_x[i * D + a];
    const double r = (v == Dim<D>::ROOT_LEN - 1) ? 1.0 : (double)v / (double)Dim<D>::ROOT_LEN;
    out[i * D + a] = (tmax[3 * t + a] - tmin[3 * t + a]) * r + tmin[3 * t + a];
  }
}

template <int D>
static void upload_leaves_and_brick(const Forest<D>& F, ForestDevice<D>& X, cudaStream_t s) {
  X.nl = (int64_t)F.leaves.size();
  X.leaf_key.upload(F.leaf_key.vec(), s);
  std::vector<int8_t> lvl((size_t)X.nl);
  for (int64_t q = 0; q < X.nl; ++q) lvl[(size_t)q] = (int8_t)F.leaves[(size_t)q].level;
  X.level.upload(lvl, s);
  X.tree_ijk.upload(F.brick.tree_ijk, s);
  X.ijk_to_tree.upload(F.brick.ijk_to_tree, s);
  X.tmin.upload(F.brick.tmin, s);
  X.tmax.upload(F.brick.tmax, s);
  cuda_check(cudaStreamSynchronize(s), "forest upload");  // the host level copy goes out of scope
}

template <int D>
ForestDevice<D>& forest_device(Forest<D>& F, cudaStream_t s) {
  if (F.device) return *static_cast<ForestDevice<D>*>(F.device.get());
  if (!F.nodes_built) throw std::invalid_argument("the forest's nodes are not built");
  auto X = std::make_shared<ForestDevice<D>>();
  upload_leaves_and_brick(F, *X, s);
  X->nn = (int64_t)F.num_nodes();
  const NodeArrays& A = F.nd->host();
  X->node_key.upload(A.node_key, s);
  X->node_tree.upload(A.node_tree, s);
  X->node_x.upload(A.node_x, s);
  X->local_nodes.upload(A.local_nodes, s);
  cuda_check(cudaStreamSynchronize(s), "forest upload");
  F.device = X;
  return *X;
}

template <int D>
void build_nodes_device(Forest<D>& F, cudaStream_t s) {
  using DD = Dim<D>;
  auto X = std::make_shared<ForestDevice<D>>();
  upload_leaves_and_brick(F, *X, s);
  const int64_t nl = X->nl, nc = nl * DD::CHILDREN;
  size_t b1 = 0, b2 = 0;
  cub::DeviceRadixSort::SortKeys(nullptr, b1, (const uint64_t*)nullptr, (uint64_t*)nullptr, (int)nc, 0, 64, s);
  cub::DeviceSelect::Unique(nullptr, b2, (const uint64_t*)nullptr, (uint64_t*)nullptr, (int64_t*)nullptr, (int)nc, s);
  const size_t tb = std::max(b1, b2) + 1;
  Arena A;
  A.reserve(2 * Arena::bytes<uint64_t>((size_t)nc + 1) + Arena::bytes<int64_t>(1) + Arena::bytes<uint8_t>(tb));
  uint64_t* corner = A.take<uint64_t>((size_t)nc + 1);
  uint64_t* sorted = A.take<uint64_t>((size_t)nc + 1);
  int64_t* nsel = A.take<int64_t>(1);
  void* temp = A.take<uint8_t>(tb);
  X->node_key.alloc((size_t)nc + 1);
  if (nc) {
    k_corner_keys<D><<<nblocks(nc), TPB, 0, s>>>(X->leaf_key.p, X->level.p, nl, F.brick.n[0], F.brick.n[1], F.brick.n[2], X->tree_ijk.p,
                                                 X->ijk_to_tree.p, corner);
    cuda_check(cub::DeviceRadixSort::SortKeys(temp, b1, corner, sorted, (int)nc, 0, 64, s), "corner sort");
    cuda_check(cub::DeviceSelect::Unique(temp, b2, sorted, X->node_key.p, nsel, (int)nc, s), "corner unique");
  }
  int64_t nn = 0;
  if (nc) cuda_check(cudaMemcpyAsync(&nn, nsel, sizeof(int64_t), cudaMemcpyDeviceToHost, s), "D2H");
  cuda_check(cudaStreamSynchronize(s), "node count");
  if (nn >= (int64_t)INT32_MAX) throw std::runtime_error("too many nodes for 32-bit node indices");
  X->nn = nn;
  X->node_tree.alloc((size_t)nn + 1);
  X->node_x.alloc((size_t)nn * D + 1);
  X->local_nodes.alloc((size_t)nc + 1);
  if (nn) k_decode_nodes<D><<<nblocks(nn), TPB, 0, s>>>(X->node_key.p, nn, X->node_tree.p, X->node_x.p);
  if (nc) k_local_nodes<<<nblocks(nc), TPB, 0, s>>>(corner, nc, X->node_key.p, nn, X->local_nodes.p);
  cuda_check(cudaGetLastError(), "device node numbering");
  // the host copies of the arrays are made on first host use
  auto H = std::make_shared<NodeArrays>();
  H->count = (size_t)nn;
  std::shared_ptr<const ForestDevice<D>> Xc = X;
  H->fetch = [Xc, nn, nc](NodeArrays& A) {
    A.node_key.resize((size_t)nn);
    A.node_tree.resize((size_t)nn);
    A.node_x.resize((size_t)nn * D);
    A.local_nodes.resize((size_t)nc);
    if (nn) {
      cuda_check(cudaMemcpy(A.node_key.data(), Xc->node_key.p, (size_t)nn * 8, cudaMemcpyDeviceToHost), "D2H");
      cuda_check(cudaMemcpy(A.node_tree.data(), Xc->node_tree.p, (size_t)nn * 4, cudaMemcpyDeviceToHost), "D2H");
      cuda_check(cudaMemcpy(A.node_x.data(), Xc->node_x.p, (size_t)nn * D * 4, cudaMemcpyDeviceToHost), "D2H");
    }
    if (nc) cuda_check(cudaMemcpy(A.local_nodes.data(), Xc->local_nodes.p, (size_t)nc * 4, cudaMemcpyDeviceToHost), "D2H");
  };
  cuda_check(cudaStreamSynchronize(s), "device node numbering");
  F.nd = H;
  F.nodes_built = true;
  F.device = X;
}

__global__ void __launch_bounds__(TPB) k_concat_index(const int32_t* __restrict__ src, int64_t n, int64_t total,
                                                      int32_t* __restrict__ dst, int64_t Ndst, int64_t off, int32_t add) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= total) return;
  const int64_t p = e / n, i = e - p * n;
  const int32_t v = src[e];
  dst[p * Ndst + off + i] = v >= 0 ? v + add : v;
}

void concat_index_planes(const int32_t* src, int64_t n, int planes, int32_t* dst, int64_t Ndst, int64_t off, int32_t add,
                         cudaStream_t s) {
  const int64_t total = n * planes;
  if (total) k_concat_index<<<nblocks(total), TPB, 0, s>>>(src, n, total, dst, Ndst, off, add);
  cuda_check(cudaGetLastError(), "index concatenation");
}

template <int D>
__global__ void __launch_bounds__(TPB) k_coarse_table(const uint64_t* __restrict__ key, int64_t nl, int64_t ncells, int64_t ncoarse, int L0,
                                                      int32_t* __restrict__ ctab) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i > ncells) return;
  if (i == ncells) {
    ctab[i] = (int32_t)(nl - 1);
    return;
  }
  const uint64_t t = (uint64_t)(i / ncoarse), c = (uint64_t)(i % ncoarse);
  const uint64_t k = (t << tree_shift<D>()) | (c << (D * (Dim<D>::MAXLEVEL - L0)));
  int64_t lo = 0, hi = nl - 1;  // the last leaf with key <= k, else 0
  while (lo < hi) {
    const int64_t mid = (lo + hi + 1) >> 1;
    if (key[mid] <= k)
      lo = mid;
    else
      hi = mid - 1;
  }
  ctab[i] = (int32_t)lo;
}

template <int D>
void coarse_table_device(const uint64_t* leaf_key, int64_t nl, int nt, int L0, int32_t* ctab, cudaStream_t s) {
  const int64_t ncoarse = int64_t(1) << (D * L0), ncells = (int64_t)nt * ncoarse;
  k_coarse_table<D><<<nblocks(ncells + 1), TPB, 0, s>>>(leaf_key, nl, ncells, ncoarse, L0, ctab);
  cuda_check(cudaGetLastError(), "coarse cell table");
}

template <int D>
void node_xyz_device(Forest<D>& F, double* out, cudaStream_t s) {
  ForestDevice<D>& X = forest_device(F, s);
  if (X.nn) k_node_xyz<D><<<nblocks(X.nn), TPB, 0, s>>>(X.node_tree.p, X.node_x.p, X.nn, X.tmin.p, X.tmax.p, out);
  cuda_check(cudaGetLastError(), "node coordinates");
}

template <int D>
bool refine_and_coarsen_device(Forest<D>& F, int min_lvl, int max_lvl, double lip, double band, const double* phi, cudaStream_t s) {
  ForestDevice<D>& X = forest_device(F, s);
  DevBuf<int8_t> tag;
  tag.alloc((size_t)X.nl + 1);
  if (X.nl)
    k_tag_leaves<D><<<nblocks(X.nl), TPB, 0, s>>>(X.leaf_key.p, X.level.p, X.nl, X.local_nodes.p, X.tmin.p, X.tmax.p, phi, min_lvl, max_lvl,
                                                  lip, band, tag.p);
  cuda_check(cudaGetLastError(), "device tags");
  std::vector<int8_t> h((size_t)X.nl);
  if (X.nl) cuda_check(cudaMemcpyAsync(h.data(), tag.p, (size_t)X.nl, cudaMemcpyDeviceToHost, s), "D2H");
  cuda_check(cudaStreamSynchronize(s), "tag download");
  return F.coarsen_then_refine(h.data());
}

#define LSG_INST(D)                                                                          \
  template void build_nodes_device<D>(Forest<D>&, cudaStream_t);                             \
  template ForestDevice<D>& forest_device<D>(Forest<D>&, cudaStream_t);                      \
  template void node_xyz_device<D>(Forest<D>&, double*, cudaStream_t);                       \
  template void coarse_table_device<D>(const uint64_t*, int64_t, int, int, int32_t*, cudaStream_t); \
  template bool refine_and_coarsen_device<D>(Forest<D>&, int, int, double, double, const double*, cudaStream_t); \
  template int64_t build_tables64_device<D>(const DForest<D>&, const Tab64Dev<D>&, cudaStream_t); \
  template void build_mixed_device<D>(const DTab64<D>&, int64_t, const double*, MixedDev<D>&, cudaStream_t);
LSG_INST(2)
LSG_INST(3)
#undef LSG_INST

}  // namespace lsg
