// Flattener, mixed-precision part: FP32 tables in a device node order of their own.
//
// Nodes are renumbered on the device into two groups so that every warp runs one code path and
// reads only what it uses:
//   regular    every direction has a single face node (weight exactly 1), no cross-term correction,
//              no third-order correction, not on a wall, and every neighbour distance equals a cell
//              size tree_size * 2^-level with level in [base_level, base_level + 15];
//              per node: 6 (4 in 2D) neighbour indices and one 32-bit word of 4-bit level codes.
//   irregular  everything else (hanging faces, walls, corrections), sorted by their pattern
//              (face-node counts, correction flag, wall bits) and then by node index, so that warps
//              see uniform patterns; per node the full stencil: counts word, face-node indices,
//              normalised weights w/nrm, distances, third-order factors and an optional 3x3 (2x2)
//              correction matrix (every branch of correct_naive_second_derivatives is linear in the
//              naive second derivatives, so it is evaluated in FP64 on the unit vectors).
// Regular nodes come first, each group keeps the node order (tree-major Morton) of the grid.
#include <algorithm>
#include <parallel/algorithm>
#include <cstring>
#include <stdexcept>

#include "tables.hpp"

namespace lsg {


template <int D>
void build_tables32(const Tables64<D>& T, const double* tree_size, Tables32<D>& M) {
  constexpr int H = Dim<D>::HALF;
  constexpr int NS = 2 * D * H;
  const int64_t N = T.N;
  M.N = N;
  // base level: the coarsest cell size present among all neighbour distances
  int base = 64;
  std::vector<int> lvl_code((size_t)2 * D * N, -1);
#pragma omp parallel for schedule(static) reduction(min : base)
  for (long long nn = 0; nn < (long long)N; ++nn) {
    for (int dir = 0; dir < 2 * D; ++dir) {
      const double dv = T.d[(size_t)dir * N + nn];
      const double size = tree_size[dir >> 1];
      if (!(dv > 0)) continue;
      int l = 0;
      double h = size;
      while (h > dv && l < 63) {
        h *= 0.5;
        ++l;
      }
      if (h == dv) {
        lvl_code[(size_t)dir * N + nn] = l;
        base = std::min(base, l);
      }
    }
  }
  if (base == 64) base = 0;
  M.base_level = base;
  for (int a = 0; a < D; ++a)
    for (int c = 0; c < 16; ++c) M.level_size[a * 16 + c] = (float)ldexp(tree_size[a], -(base + c));

  // classification and geometry classes of the irregular nodes
  constexpr int CW = cls_words<D>();
  std::vector<uint8_t> is_reg((size_t)N, 0);
  std::vector<uint32_t> icount((size_t)N);
#pragma omp parallel for schedule(static)
  for (long long nn = 0; nn < (long long)N; ++nn) {
    const size_t n = (size_t)nn;
    uint32_t counts = 0;
    bool regular = T.wall[n] == 0 && T.cidx[n] < 0;
    for (int dir = 0; dir < 2 * D; ++dir) {
      int cnt = 0;
      for (int k = 0; k < H; ++k)
        if (T.nbr[(size_t)(dir * H + k) * N + n] >= 0) cnt = k + 1;
      counts |= (uint32_t)(cnt - 1) << (2 * dir);
      if (cnt != 1) regular = false;
      for (int j = 0; j < D - 1; ++j)
        if (T.q[(size_t)(dir * (D - 1) + j) * N + n] != 0.0) regular = false;
      const int lc = lvl_code[(size_t)dir * N + n];
      if (lc < base || lc > base + 15) regular = false;
    }
    icount[n] = counts;
    is_reg[n] = regular ? 1 : 0;
  }
  // class record of every irregular node (compact: slot k of irr_nodes[k])
  std::vector<int64_t> irr_nodes;
  for (int64_t n = 0; n < N; ++n)
    if (!is_reg[n]) irr_nodes.push_back(n);
  const int64_t nIrr = (int64_t)irr_nodes.size();
  std::vector<double> rec((size_t)nIrr * CW);
#pragma omp parallel for schedule(static)
  for (long long kk = 0; kk < (long long)nIrr; ++kk) {
    const size_t n = (size_t)irr_nodes[(size_t)kk];
    const uint32_t counts = icount[n];
    double* r = &rec[(size_t)kk * CW];
    for (int w = 0; w < CW; ++w) r[w] = 0.0;
    uint32_t meta = counts | ((T.cidx[n] >= 0) ? (1u << 16) : 0u) | ((uint32_t)T.wall[n] << 24);
    r[0] = (double)meta;
    for (int dir = 0; dir < 2 * D; ++dir) {
      const int cnt = (int)((counts >> (2 * dir)) & 3) + 1;
      r[1 + dir] = T.d[(size_t)dir * N + n];
      const double nrm = T.nrm[(size_t)dir * N + n];
      for (int k = 0; k < H; ++k) r[1 + 2 * D + dir * H + k] = k < cnt ? T.w[(size_t)(dir * H + k) * N + n] / nrm : 0.0;
      for (int j = 0; j < D - 1; ++j) r[1 + 2 * D + 2 * D * H + dir * (D - 1) + j] = T.q[(size_t)(dir * (D - 1) + j) * N + n];
    }
    double* cm = r + 1 + 2 * D + 2 * D * H + 2 * D * (D - 1);
    for (int c = 0; c < D; ++c) {
      double e[3] = {0, 0, 0};
      e[c] = 1.0;
      if (T.cidx[n] >= 0) apply_correction<D>(&T.crec[6 * (size_t)T.cidx[n]], e);
      for (int rr = 0; rr < D; ++rr) cm[rr * D + c] = e[rr];
    }
  }
  // deduplicate class records (exact double keys): sort record slots by (record bytes, node)
  std::vector<int64_t> slots((size_t)nIrr);
  for (int64_t k = 0; k < nIrr; ++k) slots[(size_t)k] = k;
  __gnu_parallel::sort(slots.begin(), slots.end(), [&](int64_t x, int64_t y) {
    const int c = memcmp(&rec[(size_t)x * CW], &rec[(size_t)y * CW], CW * sizeof(double));
    return c != 0 ? c < 0 : x < y;
  });
  std::vector<int64_t> order((size_t)nIrr);
  for (int64_t i = 0; i < nIrr; ++i) order[(size_t)i] = irr_nodes[(size_t)slots[(size_t)i]];
  std::vector<int32_t> node_cls((size_t)N, -1);
  M.cls64.clear();
  int64_t ncls = 0;
  for (size_t i = 0; i < order.size(); ++i) {
    const double* ri = &rec[(size_t)slots[i] * CW];
    if (i == 0 || memcmp(ri, &rec[(size_t)slots[i - 1] * CW], CW * sizeof(double)) != 0) {
      M.cls64.insert(M.cls64.end(), ri, ri + CW);
      ++ncls;
    }
    node_cls[order[i]] = (int32_t)(ncls - 1);
  }
  M.ncls = ncls;
  M.cls32.resize(M.cls64.size());
  for (size_t i = 0; i < M.cls64.size(); ++i) M.cls32[i] = (float)M.cls64[i];
  // meta words are bit patterns, not values
  for (int64_t c = 0; c < ncls; ++c) {
    const uint32_t meta = (uint32_t)M.cls64[(size_t)c * CW];
    memcpy(&M.cls32[(size_t)c * CW], &meta, sizeof(uint32_t));
  }
  // device order: regular nodes (node order), then irregular nodes by (class, node)
  M.perm.resize((size_t)N);
  M.iperm.resize((size_t)N);
  int64_t nR = 0;
  for (int64_t n = 0; n < N; ++n)
    if (is_reg[n]) M.perm[nR++] = (int32_t)n;
  {
    int64_t i = nR;
    for (int64_t n : order) M.perm[i++] = (int32_t)n;
  }
  for (int64_t i = 0; i < N; ++i) M.iperm[M.perm[i]] = (int32_t)i;
  M.nR = nR;
  const int64_t nI = N - nR;
  M.nI = nI;
  // regular group
  M.r_meta.assign((size_t)nR, 0u);
  M.r_nbr.assign((size_t)2 * D * nR, 0);
#pragma omp parallel for schedule(static)
  for (long long ii = 0; ii < (long long)nR; ++ii) {
    const size_t n = (size_t)M.perm[ii];
    uint32_t codes = 0;
    for (int dir = 0; dir < 2 * D; ++dir) {
      codes |= (uint32_t)(lvl_code[(size_t)dir * N + n] - base) << (4 * dir);
      M.r_nbr[(size_t)dir * nR + ii] = M.iperm[T.nbr[(size_t)(dir * H) * N + n]];
    }
    M.r_meta[ii] = codes;
  }
  M.r_nbr2.assign((size_t)2 * D * nR, -1);
  M.r_meta2.assign((size_t)nR, 0u);
#pragma omp parallel for schedule(static)
  for (long long ii = 0; ii < (long long)nR; ++ii) {
    uint32_t far = 0;
    bool all = true;
    for (int dir = 0; dir < 2 * D; ++dir) {
      const int32_t j = M.r_nbr[(size_t)dir * nR + ii];
      const int back = dir ^ 1;
      if (j < nR && M.r_nbr[(size_t)back * nR + j] == (int32_t)ii) {
        M.r_nbr2[(size_t)dir * nR + ii] = M.r_nbr[(size_t)dir * nR + j];
        far |= ((M.r_meta[j] >> (4 * dir)) & 15u) << (4 * dir);
      } else {
        all = false;
      }
    }
    // uniform: every own and outer distance has the same level code
    bool uniform = all;
    const uint32_t c0 = M.r_meta[ii] & 15u;
    for (int dir = 0; dir < 2 * D && uniform; ++dir)
      uniform = ((M.r_meta[ii] >> (4 * dir)) & 15u) == c0 && ((far >> (4 * dir)) & 15u) == c0;
    M.r_meta2[ii] = far | (all ? (1u << 31) : 0u) | (uniform ? (1u << 30) : 0u);
  }

  // uniform regular nodes first (node order kept within each part); indices are remapped
  {
    std::vector<int32_t> new_of_old((size_t)nR), old_of_new;
    old_of_new.reserve((size_t)nR);
    for (int64_t ii = 0; ii < nR; ++ii)
      if ((M.r_meta2[ii] >> 30) & 1u) old_of_new.push_back((int32_t)ii);
    M.nU = (int64_t)old_of_new.size();
    for (int64_t ii = 0; ii < nR; ++ii)
      if (!((M.r_meta2[ii] >> 30) & 1u)) old_of_new.push_back((int32_t)ii);
    for (int64_t k = 0; k < nR; ++k) new_of_old[old_of_new[k]] = (int32_t)k;
    auto remap = [&](int32_t j) -> int32_t { return (j >= 0 && j < nR) ? new_of_old[j] : j; };
    std::vector<uint32_t> meta_n((size_t)nR), meta2_n((size_t)nR);
    std::vector<int32_t> nbr_n((size_t)2 * D * nR), nbr2_n((size_t)2 * D * nR);
    std::vector<int32_t> perm_n((size_t)nR);
    for (int64_t k = 0; k < nR; ++k) {
      const int64_t o = old_of_new[k];
      meta_n[k] = M.r_meta[o];
      meta2_n[k] = M.r_meta2[o];
      perm_n[k] = M.perm[o];
      for (int dir = 0; dir < 2 * D; ++dir) {
        nbr_n[(size_t)dir * nR + k] = remap(M.r_nbr[(size_t)dir * nR + o]);
        nbr2_n[(size_t)dir * nR + k] = remap(M.r_nbr2[(size_t)dir * nR + o]);
      }
    }
    M.r_meta.swap(meta_n);
    M.r_meta2.swap(meta2_n);
    M.r_nbr.swap(nbr_n);
    M.r_nbr2.swap(nbr2_n);
    for (int64_t k = 0; k < nR; ++k) M.perm[k] = perm_n[k];
    for (int64_t i = 0; i < N; ++i) M.iperm[M.perm[i]] = (int32_t)i;
  }
  // irregular group
  M.i_meta.assign((size_t)nI, 0u);
  M.i_nbr.assign((size_t)NS * nI, 0);
  M.i_wf.assign((size_t)NS * nI, 0.0f);
  M.i_d.assign((size_t)2 * D * nI, 0.0f);
  M.i_q.assign((size_t)2 * D * (D - 1) * nI, 0.0f);
  M.i_cidx.assign((size_t)nI, -1);
  M.i_cls.assign((size_t)nI, 0u);
  M.i_wf64.assign((size_t)NS * nI, 0.0);
  M.i_d64.assign((size_t)2 * D * nI, 0.0);
  M.i_q64.assign((size_t)2 * D * (D - 1) * nI, 0.0);
#pragma omp parallel for schedule(static)
  for (long long ii = 0; ii < (long long)nI; ++ii) {
    const size_t n = (size_t)M.perm[nR + ii];
    uint32_t meta = icount[n];
    if (T.cidx[n] >= 0) meta |= 1u << 16;
    meta |= (uint32_t)T.wall[n] << 24;
    M.i_meta[ii] = meta;
    M.i_cls[ii] = (uint32_t)node_cls[n];
    for (int dir = 0; dir < 2 * D; ++dir) {
      const int cnt = (int)((icount[n] >> (2 * dir)) & 3) + 1;
      const double nrm = T.nrm[(size_t)dir * N + n];
      for (int k = 0; k < H; ++k) {
        const int32_t nb = T.nbr[(size_t)(dir * H + k) * N + n];
        M.i_nbr[(size_t)(dir * H + k) * nI + ii] = k < cnt ? M.iperm[nb] : M.iperm[T.nbr[(size_t)(dir * H) * N + n]];
        const double wn = k < cnt ? T.w[(size_t)(dir * H + k) * N + n] / nrm : 0.0;
        M.i_wf[(size_t)(dir * H + k) * nI + ii] = (float)wn;
        M.i_wf64[(size_t)(dir * H + k) * nI + ii] = wn;
      }
      M.i_d[(size_t)dir * nI + ii] = (float)T.d[(size_t)dir * N + n];
      M.i_d64[(size_t)dir * nI + ii] = T.d[(size_t)dir * N + n];
      for (int j = 0; j < D - 1; ++j) {
        M.i_q[(size_t)(dir * (D - 1) + j) * nI + ii] = (float)T.q[(size_t)(dir * (D - 1) + j) * N + n];
        M.i_q64[(size_t)(dir * (D - 1) + j) * nI + ii] = T.q[(size_t)(dir * (D - 1) + j) * N + n];
      }
    }
    M.i_cidx[ii] = T.cidx[n];
  }
  // extended second-derivative set: regular face nodes of irregular nodes, and face nodes of regular
  // nodes whose second neighbour is not recorded (irregular nodes are always in the set)
  {
    std::vector<uint8_t> inx((size_t)nR, 0);
#pragma omp parallel for schedule(static)
    for (long long ii = 0; ii < (long long)nI; ++ii)
      for (int s_ = 0; s_ < NS; ++s_) {
        const int32_t j = M.i_nbr[(size_t)s_ * nI + ii];
        if (j < nR) {
#pragma omp atomic write
          inx[j] = 1;
        }
      }
#pragma omp parallel for schedule(static)
    for (long long ii = 0; ii < (long long)nR; ++ii)
      for (int dir = 0; dir < 2 * D; ++dir)
        if (M.r_nbr2[(size_t)dir * nR + ii] < 0) {
          const int32_t j = M.r_nbr[(size_t)dir * nR + ii];
          if (j < nR) {
#pragma omp atomic write
            inx[j] = 1;
          }
        }
    // regular order [uniform, not in the set | uniform in the set | other in the set | other]: the
    // regular part of the extended set becomes one contiguous range (coalesced second-derivative
    // writes, no index list) and the uniform nodes stay in front
    std::vector<int32_t> old_of_new;
    old_of_new.reserve((size_t)nR);
    for (int pass = 0; pass < 4; ++pass)
      for (int64_t j = 0; j < nR; ++j) {
        const bool uni = j < M.nU, inset = inx[(size_t)j] != 0;
        const int cls = uni ? (inset ? 1 : 0) : (inset ? 2 : 3);
        if (cls == pass) old_of_new.push_back((int32_t)j);
      }
    std::vector<int32_t> new_of_old((size_t)nR);
    for (int64_t k = 0; k < nR; ++k) new_of_old[(size_t)old_of_new[(size_t)k]] = (int32_t)k;
    auto remap = [&](int32_t j) -> int32_t { return (j >= 0 && j < nR) ? new_of_old[(size_t)j] : j; };
    std::vector<uint32_t> meta_n((size_t)nR), meta2_n((size_t)nR);
    std::vector<int32_t> nbr_n((size_t)2 * D * nR), nbr2_n((size_t)2 * D * nR), perm_n((size_t)nR);
#pragma omp parallel for schedule(static)
    for (long long k = 0; k < (long long)nR; ++k) {
      const int64_t o = old_of_new[(size_t)k];
      meta_n[(size_t)k] = M.r_meta[(size_t)o];
      meta2_n[(size_t)k] = M.r_meta2[(size_t)o];
      perm_n[(size_t)k] = M.perm[(size_t)o];
      for (int dir = 0; dir < 2 * D; ++dir) {
        nbr_n[(size_t)dir * nR + k] = remap(M.r_nbr[(size_t)dir * nR + o]);
        nbr2_n[(size_t)dir * nR + k] = remap(M.r_nbr2[(size_t)dir * nR + o]);
      }
    }
#pragma omp parallel for schedule(static)
    for (long long q = 0; q < (long long)((size_t)NS * nI); ++q) M.i_nbr[(size_t)q] = remap(M.i_nbr[(size_t)q]);
    M.r_meta.swap(meta_n);
    M.r_meta2.swap(meta2_n);
    M.r_nbr.swap(nbr_n);
    M.r_nbr2.swap(nbr2_n);
    for (int64_t k = 0; k < nR; ++k) M.perm[(size_t)k] = perm_n[(size_t)k];
    for (int64_t i = 0; i < N; ++i) M.iperm[(size_t)M.perm[(size_t)i]] = (int32_t)i;
    int64_t uni_out = 0, nset = 0;
    for (int64_t j = 0; j < nR; ++j) {
      if (inx[(size_t)j]) ++nset;
      else if (j < M.nU) ++uni_out;
    }
    M.x_first = uni_out;
    M.x_list.resize((size_t)nset);
    for (int64_t k = 0; k < nset; ++k) M.x_list[(size_t)k] = (int32_t)(uni_out + k);
  }
  const size_t R = T.crec.size() / 6;
  M.corr.assign((size_t)D * D * R, 0.0f);
  M.corr64.assign((size_t)D * D * R, 0.0);
  for (size_t r = 0; r < R; ++r) {
    for (int c = 0; c < D; ++c) {
      double e[3] = {0, 0, 0};
      e[c] = 1.0;
      apply_correction<D>(&T.crec[6 * r], e);
      for (int rr = 0; rr < D; ++rr) {
        M.corr[(size_t)D * D * r + D * rr + c] = (float)e[rr];
        M.corr64[(size_t)D * D * r + D * rr + c] = e[rr];
      }
    }
  }
}

template void build_tables32<2>(const Tables64<2>&, const double*, Tables32<2>&);
template void build_tables32<3>(const Tables64<3>&, const double*, Tables32<3>&);

}  // namespace lsg
