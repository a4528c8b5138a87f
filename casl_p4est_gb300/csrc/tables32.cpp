// Flattener, mixed-precision part: FP32 coefficient tables derived from the FP64 ones.
//
// Per node, read unconditionally by the mixed kernels (3D: 52 bytes):
//   meta   bits 2*dir..2*dir+1: number of face nodes of direction dir minus one
//          bit 16: the node has a cross-term correction (index in cidx, matrix in corr)
//          bits 24..29: wall mask
//   nbr    slot 0 of every direction (shared with the FP64 tables)
//   d      distance per direction
// Read only for directions with more than one face node: the other nbr slots, the normalised
// weights wf = w/nrm and the third-order factors q. The cross-term correction of
// correct_naive_second_derivatives is linear in the naive second derivatives, so every branch of it
// becomes one 3x3 (2x2) matrix, evaluated in FP64 on the unit vectors and stored in FP32.
#include <stdexcept>

#include "tables.hpp"

namespace lsg {

template <int D>
static void apply_correction_host(const double* m, double* Dv) {
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

template <int D>
void build_tables32(const Tables64<D>& T, Tables32<D>& M) {
  constexpr int H = Dim<D>::HALF;
  constexpr int NS = 2 * D * H;
  const int64_t N = T.N;
  M.N = N;
  M.meta.assign((size_t)N, 0u);
  M.wf.assign((size_t)NS * N, 0.0f);
  M.d.assign((size_t)2 * D * N, 0.0f);
  M.q.assign((size_t)2 * D * (D - 1) * N, 0.0f);
  const size_t R = T.crec.size() / 6;
  M.corr.assign((size_t)D * D * R, 0.0f);
#pragma omp parallel for schedule(static)
  for (long long nn = 0; nn < (long long)N; ++nn) {
    const size_t n = (size_t)nn;
    uint32_t meta = 0;
    for (int dir = 0; dir < 2 * D; ++dir) {
      int cnt = 0;
      for (int k = 0; k < H; ++k)
        if (T.nbr[(size_t)(dir * H + k) * N + n] >= 0) cnt = k + 1;
      meta |= (uint32_t)(cnt - 1) << (2 * dir);
      const double nrm = T.nrm[(size_t)dir * N + n];
      for (int k = 0; k < cnt; ++k) M.wf[(size_t)(dir * H + k) * N + n] = (float)(T.w[(size_t)(dir * H + k) * N + n] / nrm);
      M.d[(size_t)dir * N + n] = (float)T.d[(size_t)dir * N + n];
      for (int j = 0; j < D - 1; ++j) M.q[(size_t)(dir * (D - 1) + j) * N + n] = (float)T.q[(size_t)(dir * (D - 1) + j) * N + n];
    }
    if (T.cidx[n] >= 0) meta |= 1u << 16;
    meta |= (uint32_t)T.wall[n] << 24;
    M.meta[n] = meta;
  }
  for (size_t r = 0; r < R; ++r) {
    for (int c = 0; c < D; ++c) {
      double e[3] = {0, 0, 0};
      e[c] = 1.0;
      apply_correction_host<D>(&T.crec[6 * r], e);
      for (int rr = 0; rr < D; ++rr) M.corr[(size_t)D * D * r + D * rr + c] = (float)e[rr];
    }
  }
}

template void build_tables32<2>(const Tables64<2>&, Tables32<2>&);
template void build_tables32<3>(const Tables64<3>&, Tables32<3>&);

}  // namespace lsg
