// Flattened node-neighbour tables (host side of the flattener).
//
// The flattener turns the per-node quad_neighbor_nodes_of_node_t records into structure-of-arrays
// tables, indexed [slot * N + node] so that consecutive threads read consecutive words:
//
//   slot = dir * HALF + k   one of the HALF face nodes of direction dir
//
// FP64 tables keep every quantity the reference derives from the stencil geometry with exactly the
// reference's floating-point expressions, precomputed once per grid:
//   w      get_linear_interpolation_weights (src/my_p4est_quad_neighbor_nodes_of_node.h:222-245):
//          w_mm = d_p0*d_0p, w_pm = d_m0*d_0p, w_mp = d_p0*d_0m, w_pp = d_m0*d_0m (2D: d_p0, d_m0)
//   nrm    the matching normalisation (d_m0+d_p0)*(d_0m+d_0p) (2D: d_m0+d_p0)
//   q      the third-order neighbour correction factors 0.5*d_m0*d_p0 and 0.5*d_0m*d_0p
//          (ngbd_with_quadratic_interpolation, .h:1514-1545)
//   m      the second-derivative cross-term coefficients m12..m32
//          (correct_naive_second_derivatives, src/my_p4est_quad_neighbor_nodes_of_node.cpp:44-56)
// Face nodes whose weight is exactly zero are dropped and the remaining ones are stored in the order
// the reference sums them (pp, pm, mp, mm in 3D; pm, mm in 2D), so the device sum is the reference
// sum without its +-0 terms. A slot holding -1 is unused.
//
// Mixed-precision tables hold the same stencil with all divisions folded into FP32 coefficients.
#pragma once
#include <stdint.h>

#include <vector>

#include "neighbors.hpp"

namespace lsg {

// Correction record: the six cross-term coefficients (2D uses m12, m21) of one node whose stencil
// has at least one coefficient with |m| >= EPS.
enum { CM12 = 0, CM13 = 1, CM21 = 2, CM23 = 3, CM31 = 4, CM32 = 5 };

template <int D>
struct Tables64 {
  static constexpr int H = Dim<D>::HALF;
  static constexpr int NS = 2 * D * H;  // face-node slots per node
  int64_t N = 0;
  std::vector<int32_t> nbr;   // NS * N
  std::vector<double> w;      // NS * N
  std::vector<double> nrm;    // 2D * N
  std::vector<double> d;      // 2D * N
  std::vector<double> q;      // 2D*(D-1) * N, [dir*(D-1) + j]
  std::vector<int32_t> cidx;  // N (-1: no cross-term correction)
  std::vector<double> crec;   // 6 * R
  std::vector<uint8_t> wall;  // N, bit dir set on a domain wall
  std::vector<double> smin;   // N, min |d| over directions (CFL of advect_in_normal_direction)
};

template <int D>
void build_tables64(const Forest<D>& F, Tables64<D>& T);

// Correction records of the first derivatives (correct_naive_first_derivatives,
// src/my_p4est_quad_neighbor_nodes_of_node.cpp:575-640): for every node whose naive central first
// derivative along some axis a needs the second derivative along a tangential axis, gidx[n] is a
// record index; the record holds the D*(D-1) weights dd_correction_weight_to_naive_first_derivative
// ([a*(D-1) + j], j-th axis other than a) and gmask bit a*(D-1)+j says which are applied.
template <int D>
void build_gradient_tables(const Forest<D>& F, std::vector<int32_t>& gidx, std::vector<double>& grec, std::vector<uint8_t>& gmask);

// Edge-diagonal neighbours of every node as my_p4est_node_neighbors_t::get_all_neighbors finds them
// (src/my_p4est_node_neighbors.cpp:2001-2153): 3D m0m p0m m0p p0p 0mm 0pm 0mp 0pp mm0 pm0 mp0 pp0,
// 2D mm0 pm0 mp0 pp0; -1 where absent. [k * N + n].
template <int D>
void build_corner_neighbors(const Forest<D>& F, std::vector<int32_t>& out);

// Tables of the disjoint union of several grids: node indices of part k are offset by the node count
// of the parts before it (the union's node order is the parts' node orders one after the other).
template <int D>
void concat_tables64(const std::vector<const Tables64<D>*>& parts, Tables64<D>& out);

template <int D>
struct Tables32 {
  int64_t N = 0, nR = 0, nI = 0;
  int64_t nU = 0;                   // regular nodes 0 .. nU-1 have uniform stencils (see r_meta2 bit 30)
  int base_level = 0;
  float level_size[3 * 16] = {0};   // [axis*16 + code] cell size tree_size * 2^-(base_level + code)
  std::vector<int32_t> perm;        // device index -> node
  std::vector<int32_t> iperm;       // node -> device index
  // regular group (device indices 0 .. nR-1)
  std::vector<uint32_t> r_meta;     // nR: 4-bit level code per direction
  std::vector<int32_t> r_nbr;       // 2D * nR, device indices
  // second neighbour along each direction (the face node's own face node further out), valid when
  // the face node is regular and its opposite face node is this node; -1 otherwise
  std::vector<int32_t> r_nbr2;      // 2D * nR
  std::vector<uint32_t> r_meta2;    // nR: 4-bit level code of the face node's outer distance per direction,
                                    //     bit 31 set when every direction has a second neighbour
  // irregular group (device indices nR .. N-1, stored at [i - nR]), sorted by geometry class
  std::vector<uint32_t> i_meta;     // nI: counts (2 bits/dir), bit 16 correction, bits 24.. walls
  std::vector<uint32_t> i_cls;      // nI: geometry class (index into cls32/cls64)
  std::vector<int32_t> i_nbr;       // NS * nI, device indices
  // geometry classes of the irregular nodes: meta word, then per direction d, normalised weights,
  // third-order factors, then the correction matrix (identity when none), as floats (cls32) and doubles
  // (cls64); CLS_WORDS(D) entries per class
  std::vector<float> cls32;
  std::vector<double> cls64;
  int64_t ncls = 0;
  // nodes whose second derivatives are computed by the extended pass: the irregular nodes and every
  // face node that the fused stage cannot rebuild from a second neighbour (regular ones listed here)
  std::vector<int32_t> x_list;     // x_first, x_first + 1, ... (the regular part of the set is contiguous)
  int64_t x_first = 0;
  std::vector<float> i_wf;          // NS * nI
  std::vector<float> i_d;           // 2D * nI
  std::vector<float> i_q;           // 2D*(D-1) * nI
  std::vector<int32_t> i_cidx;      // nI
  std::vector<float> corr;          // D*D * R, row-major: corrected = corr * naive
  // FP64 copies of the irregular coefficients, for the FP64 subcell step of the mixed path
  std::vector<double> i_wf64, i_d64, i_q64, corr64;
};

template <int D>
void build_tables32(const Tables64<D>& T, const double* tree_size, Tables32<D>& M);

// class record layout: [0] meta (bits), [1 + dir] d, [1 + 2D + dir*H + k] wf, [1 + 2D + 2D*H + dir*(D-1) + j] q,
// [1 + 2D + 2D*H + 2D*(D-1) + r*D + c] correction
template <int D>
LSG_HD constexpr int cls_words() { return 1 + 2 * D + 2 * D * Dim<D>::HALF + 2 * D * (D - 1) + D * D; }

// Cross-term coefficients of one record, exactly as correct_naive_second_derivatives computes them.
template <int D>
inline void cross_terms(const Qnnn<D>& q, double* m) {
  for (int i = 0; i < 6; ++i) m[i] = 0.0;
  // m_ab: correction of the naive second derivative along axis a by the one along axis b, built from
  // the offsets of the two neighbours along a, in the tangential axis b.
  auto mab = [&](int a, int j) -> double {
    const int dm = 2 * a, dp = 2 * a + 1;
    return q.dt[dm][2 * j] * q.dt[dm][2 * j + 1] / q.d[dm] / (q.d[dp] + q.d[dm]) +
           q.dt[dp][2 * j] * q.dt[dp][2 * j + 1] / q.d[dp] / (q.d[dp] + q.d[dm]);
  };
  m[CM12] = mab(0, 0);
  m[CM21] = mab(1, 0);
  if (D == 3) {
    m[CM13] = mab(0, 1);
    m[CM23] = mab(1, 1);
    m[CM31] = mab(2, 0);
    m[CM32] = mab(2, 1);
  }
}

}  // namespace lsg
