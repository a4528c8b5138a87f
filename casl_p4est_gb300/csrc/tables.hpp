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
LSG_HD void cross_terms(const Qnnn<D>& q, double* m) {
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

// correct_naive_second_derivatives (src/my_p4est_quad_neighbor_nodes_of_node.cpp:44-298) applied to the
// naive second derivatives Dv from the six cross-term coefficients m, every branch (host and device).
template <int D>
LSG_HD void apply_correction(const double* m, double* Dv) {
  auto z = [](double v) { return fabs(v) < EPS; };
  if (D == 2) {
    const double m12 = m[CM12], m21 = m[CM21];
    if (z(m12)) {
      if (!z(m21)) Dv[1] = Dv[1] - m21 * Dv[0];
    } else if (z(m21)) {
      Dv[0] = Dv[0] - m12 * Dv[1];
    } else {
      const double idet = 1.0 / (1.0 - m12 * m21);
      const double nx = Dv[0], ny = Dv[1];
      Dv[0] = nx * idet - ny * (m12 * idet);
      Dv[1] = ny * idet - nx * (m21 * idet);
    }
    return;
  }
  const double m12 = m[CM12], m13 = m[CM13], m21 = m[CM21], m23 = m[CM23], m31 = m[CM31], m32 = m[CM32];
  double &Dxx = Dv[0], &Dyy = Dv[1], &Dzz = Dv[2];
  if (z(m12) && z(m13)) {
    if (z(m23)) {
      if (!z(m21)) Dyy -= m21 * Dxx;
      if (!z(m31)) Dzz -= m31 * Dxx;
      if (!z(m32)) Dzz -= m32 * Dyy;
    } else if (z(m32)) {
      if (!z(m31)) Dzz -= m31 * Dxx;
      Dyy -= m23 * Dzz;
      if (!z(m21)) Dyy -= m21 * Dxx;
    } else {
      const double idet = 1.0 / (1.0 - m23 * m32);
      const bool m21z = z(m21), m31z = z(m31);
      const double nDyy = Dyy, nDzz = Dzz;
      Dyy = ((m21z ? nDyy : (nDyy - m21 * Dxx)) - m23 * (m31z ? nDzz : (nDzz - m31 * Dxx))) * idet;
      Dzz = ((m31z ? nDzz : (nDzz - m31 * Dxx)) - m32 * (m21z ? nDyy : (nDyy - m21 * Dxx))) * idet;
    }
  } else if (z(m21) && z(m23)) {
    if (z(m13)) {
      if (!z(m12)) Dxx -= m12 * Dyy;
      if (!z(m31)) Dzz -= m31 * Dxx;
      if (!z(m32)) Dzz -= m32 * Dyy;
    } else if (z(m31)) {
      if (!z(m32)) Dzz -= m32 * Dyy;
      Dxx -= m13 * Dzz;
      if (!z(m12)) Dxx -= m12 * Dyy;
    } else {
      const double idet = 1.0 / (1.0 - m13 * m31);
      const bool m12z = z(m12), m32z = z(m32);
      const double nDxx = Dxx, nDzz = Dzz;
      Dxx = ((m12z ? nDxx : (nDxx - m12 * Dyy)) - m13 * (m32z ? nDzz : (nDzz - m32 * Dyy))) * idet;
      Dzz = ((m32z ? nDzz : (nDzz - m32 * Dyy)) - m31 * (m12z ? nDxx : (nDxx - m12 * Dyy))) * idet;
    }
  } else if (z(m31) && z(m32)) {
    if (z(m12)) {
      if (!z(m13)) Dxx -= m13 * Dzz;
      if (!z(m21)) Dyy -= m21 * Dxx;
      if (!z(m23)) Dyy -= m23 * Dzz;
    } else if (z(m21)) {
      if (!z(m23)) Dyy -= m23 * Dzz;
      Dxx -= m12 * Dyy;
      if (!z(m13)) Dxx -= m13 * Dzz;
    } else {
      const double idet = 1.0 / (1.0 - m12 * m21);
      const bool m13z = z(m13), m23z = z(m23);
      const double nDxx = Dxx, nDyy = Dyy;
      Dxx = ((m13z ? nDxx : (nDxx - m13 * Dzz)) - m12 * (m23z ? nDyy : (nDyy - m23 * Dzz))) * idet;
      Dyy = ((m23z ? nDyy : (nDyy - m23 * Dzz)) - m21 * (m13z ? nDxx : (nDxx - m13 * Dzz))) * idet;
    }
  } else {
    const double idet = 1.0 / (1.0 + m12 * m23 * m31 + m13 * m21 * m32 - m12 * m21 - m13 * m31 - m23 * m32);
    const double nDxx = Dxx, nDyy = Dyy, nDzz = Dzz;
    Dxx = (nDxx * (idet * (1.0 - m23 * m32)) + nDyy * (idet * (m32 * m13 - m12)) + nDzz * (idet * (m12 * m23 - m13)));
    Dyy = (nDxx * (idet * (m31 * m23 - m21)) + nDyy * (idet * (1.0 - m31 * m13)) + nDzz * (idet * (m21 * m13 - m23)));
    Dzz = (nDxx * (idet * (m21 * m32 - m31)) + nDyy * (idet * (m31 * m12 - m32)) + nDzz * (idet * (1.0 - m21 * m12)));
  }
}

// Order in which interpolate_linearly sums the face nodes (.h:290-306): pp, pm, mp, mm (3D); pm, mm (2D).
template <int D>
LSG_HD int eval_slot(int e) {
  if (D == 2) return e == 0 ? 1 : 0;
  return e == 0 ? 3 : (e == 1 ? 1 : (e == 2 ? 2 : 0));
}

// One node's row of the FP64 tables from its record (the same code on the host and the device):
// face nodes with a nonzero weight in summation order, unused slots -1 / 0; normalisations,
// distances, third-order factors, the smallest |d| (smin). Returns whether the node needs a
// cross-term correction record.
template <int D>
LSG_HD bool fill_row64(const Qnnn<D>& q, int64_t N, int64_t n, int32_t* nbr, double* w, double* nrm, double* d, double* qf,
                       double* smin) {
  constexpr int H = Dim<D>::HALF;
  for (int dir = 0; dir < 2 * D; ++dir) {
    const double dm0 = q.dt[dir][0], dp0 = q.dt[dir][1];
    const double d0m = (D == 3) ? q.dt[dir][2] : 0.0, d0p = (D == 3) ? q.dt[dir][3] : 0.0;
    double wk[4] = {0, 0, 0, 0};
    double nr;
    if (D == 2) {
      wk[0] = dp0;  // mm
      wk[1] = dm0;  // pm
      nr = dm0 + dp0;
    } else {
      wk[0] = dp0 * d0p;  // mm
      wk[1] = dm0 * d0p;  // pm
      wk[2] = dp0 * d0m;  // mp
      wk[3] = dm0 * d0m;  // pp
      nr = (dm0 + dp0) * (d0m + d0p);
    }
    int o = 0;
    for (int e = 0; e < H; ++e) {
      const int k = eval_slot<D>(e);
      if (wk[k] == 0.0) continue;
      nbr[(int64_t)(dir * H + o) * N + n] = q.nb[dir][k];
      w[(int64_t)(dir * H + o) * N + n] = wk[k];
      ++o;
    }
    for (; o < H; ++o) {
      nbr[(int64_t)(dir * H + o) * N + n] = -1;
      w[(int64_t)(dir * H + o) * N + n] = 0.0;
    }
    nrm[(int64_t)dir * N + n] = nr;
    d[(int64_t)dir * N + n] = q.d[dir];
    for (int j = 0; j < D - 1; ++j) qf[(int64_t)(dir * (D - 1) + j) * N + n] = 0.5 * q.dt[dir][2 * j] * q.dt[dir][2 * j + 1];
  }
  double s = min2(fabs(q.d[1]), fabs(q.d[0]));
  s = (D == 3) ? min3(s, min2(fabs(q.d[3]), fabs(q.d[2])), min2(fabs(q.d[5 % (2 * D)]), fabs(q.d[4 % (2 * D)])))
               : min2(s, min2(fabs(q.d[3]), fabs(q.d[2])));
  smin[n] = s;
  double m[6];
  cross_terms<D>(q, m);
  bool any = false;
  for (int i = 0; i < 6; ++i) any = any || !(fabs(m[i]) < EPS);
  return any;
}

}  // namespace lsg
