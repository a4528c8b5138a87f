// FP64 level-set kernels that evaluate every floating-point expression in the reference's order.
// This translation unit is compiled with -fmad=false so that no multiply-add is contracted, which
// makes each result the IEEE double the reference's C++ produces for the same inputs.
//
// One thread per node. Restated reference routines:
//   laplace + correct_naive_second_derivatives  src/my_p4est_quad_neighbor_nodes_of_node.h:615-635,
//                                               src/my_p4est_quad_neighbor_nodes_of_node.cpp:44-298
//   ngbd_with_quadratic_interpolation          .h:1514-1545
//   reinitialize_one_iteration                 src/my_p4est_level_set.cpp:59-288
//   interface_Location[_With_Second_Order_Derivative]  src/casl_math.cpp:55-97
//   advect_in_normal_direction_one_iteration   src/my_p4est_level_set.cpp:559-654
//   CFL of the CF overload                     src/my_p4est_level_set.cpp:745-783
#include <algorithm>

#include <cub/cub.cuh>

#include "kernels.h"
#include "stencil64.cuh"
#include "tables.hpp"

namespace lsg {

namespace {

using namespace st64;
constexpr int TPB = 256;

template <int D>
__global__ void __launch_bounds__(TPB, 8) k_dd64(DTab64<D> T, const double* __restrict__ f, double* __restrict__ dd, int64_t first,
                                              int64_t last) {
  const int64_t n = first + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= last) return;
  double Dv[D];
  laplace64<D>(T, n, f, Dv);
#pragma unroll
  for (int a = 0; a < D; ++a) dd[(int64_t)a * T.N + n] = Dv[a];
}

// Everything reinitialize_one_iteration derives from phi_0 alone: anchoring, range limits, sign,
// and the subcell distances of the interface-adjacent nodes (src/my_p4est_level_set.cpp:84-211).
template <int D>
__global__ void __launch_bounds__(TPB) k_reinit_prep64(DTab64<D> T, const double* __restrict__ phi0, const double* __restrict__ dd0,
                                                       double zdt, double lim_lo, double lim_hi, int order_space,
                                                       uint16_t* __restrict__ status, double* __restrict__ s_near, int64_t first,
                                                       int64_t last) {
  const int64_t n = first + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t N = T.N;
  if (n >= last) return;
  const double p0 = phi0[n];
  if (fabs(p0) < zdt) {
    status[n] = ST_ANCHORED;
    return;
  }
  if (!(lim_lo < p0 && p0 < lim_hi)) {
    status[n] = ST_OUTSIDE;
    return;
  }
  double Dv[D];
#pragma unroll
  for (int a = 0; a < D; ++a) Dv[a] = dd0[(int64_t)a * N + n];
  double fn[2 * D];
  bool near = false;
#pragma unroll
  for (int dir = 0; dir < 2 * D; ++dir) {
    fn[dir] = quad_nb64<D>(T, dir, n, phi0, Dv);
    near = near || product_negative(p0, fn[dir]);
  }
  uint16_t st = positive(p0) ? ST_POSITIVE : 0;
  if (near) {
    st |= ST_NEAR;
    double s[2 * D];
#pragma unroll
    for (int dir = 0; dir < 2 * D; ++dir) s[dir] = T.d[(int64_t)dir * N + n];
#pragma unroll
    for (int dir = 0; dir < 2 * D; ++dir) {
      if (!product_negative(p0, fn[dir])) continue;
      st |= (uint16_t)(1u << (ST_CUT_SHIFT + dir));
      const int axis = dir >> 1;
      if (dir & 1) {
        if (order_space > 1)
          s[dir] = interface_location_2nd(0.0, s[dir], p0, fn[dir], Dv[axis], lin64<D>(T, dir, n, dd0 + (int64_t)axis * N));
        else
          s[dir] = interface_location(0.0, s[dir], p0, fn[dir]);
      } else {
        if (order_space > 1)
          s[dir] = -interface_location_2nd(-s[dir], 0.0, fn[dir], p0, lin64<D>(T, dir, n, dd0 + (int64_t)axis * N), Dv[axis]);
        else
          s[dir] = -interface_location(-s[dir], 0.0, fn[dir], p0);
      }
    }
#pragma unroll
    for (int dir = 0; dir < 2 * D; ++dir) s_near[(int64_t)dir * N + n] = max2(s[dir], zdt);
  }
  status[n] = st;
}

// Six blocks per SM (at most 40 registers; a few hundred bytes of a thread's state spill to L1): once the pattern
// word and the exponent arithmetic had taken most of the FP64 work off the pipe, the kernel waited on its loads, and
// more resident warps hide them better (per launch on 13.7M nodes, all axes at once: 2 blocks 3.46 ms, 3 blocks
// 2.75, 4 blocks 2.33, 5 blocks 2.20, 6 blocks 2.21; one axis at a time, fewer values live: 5 blocks 2.18, 6 blocks
// 2.16). The second-derivative sweep runs at eight blocks (32 registers: 0.79 ms at five, 0.71 at six, 0.67 at
// eight) and the advection stage at six (20 steps on 122M nodes: 866 ms at five, 848 at six) for the same reason.
template <int D, int ORDER_SPACE, bool AVG>
__global__ void __launch_bounds__(TPB, 6) k_reinit_stage64(DTab64<D> T, const uint16_t* __restrict__ status, const double* __restrict__ s_near,
                                                        const double* __restrict__ phi0, const double* __restrict__ phin,
                                                        const double* __restrict__ dd, double* out, const double* avg_with,
                                                        int64_t first, int64_t last) {
  const int64_t n = first + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t N = T.N;
  if (n >= last) return;
  const uint16_t st = status[n];
  double r;
  if (st & ST_ANCHORED) {
    r = 0.0;
  } else if (st & ST_OUTSIDE) {
    r = phi0[n];
  } else {
    const double p0 = phi0[n];
    const double f0 = phin[n];
    double Dv[D];
#pragma unroll
    for (int a = 0; a < D; ++a) Dv[a] = dd[(int64_t)a * N + n];
    const NodeWord nw = node_word<D>(T, n);
    const bool near = (st & ST_NEAR) != 0;
    const uint8_t wl = T.wall[n];
    // sgn = (p0 > 0 ? 1 : -1): the prep step stored p0 > 0 as ST_POSITIVE; sgn * g is +-g exactly, so the
    // upwind tests are sign tests of g
    const bool pos = (st & ST_POSITIVE) != 0;
    // one axis at a time (the same operations on the same values as all axes at once, and the sum and the
    // minimum accumulated in the same order), so that only one axis's values are live
    double h = 0.0, dt = 0.0;
#pragma unroll
    for (int a = 0; a < D; ++a) {
      double fm = quad_nb64<D>(T, 2 * a, n, phin, Dv, nw), fp = quad_nb64<D>(T, 2 * a + 1, n, phin, Dv, nw);
      double sm, sp;
      if (near) {
        sm = s_near[(int64_t)(2 * a) * N + n];
        sp = s_near[(int64_t)(2 * a + 1) * N + n];
        if (st & (1u << (ST_CUT_SHIFT + 2 * a))) fm = 0.0;
        if (st & (1u << (ST_CUT_SHIFT + 2 * a + 1))) fp = 0.0;
      } else {
        sm = T.d[(int64_t)(2 * a) * N + n];
        sp = T.d[(int64_t)(2 * a + 1) * N + n];
      }
      double x0 = 0.0, xm_nb = 0.0, xp_nb = 0.0;
      if (ORDER_SPACE > 1) {
        x0 = Dv[a];
        xm_nb = lin64w<D>(T, 2 * a, n, dd + (int64_t)a * N, nw);
        xp_nb = lin64w<D>(T, 2 * a + 1, n, dd + (int64_t)a * N, nw);
      }
      if (wl & (1u << (2 * a))) {
        sm = sp;
        fm = fp;
        x0 = xm_nb = xp_nb = 0.0;
      }
      if (wl & (1u << (2 * a + 1))) {
        sp = sm;
        fp = fm;
        x0 = xm_nb = xp_nb = 0.0;
      }
      double gp = qdiv(fp - f0, sp);
      double gm = qdiv(f0 - fm, sm);
      if (ORDER_SPACE > 1) {
        const double xm = minmod_x(xm_nb, x0);
        gm = gm + scale2(sm, -1) * xm;
        const double xp = minmod_x(xp_nb, x0);
        gp = gp - scale2(sp, -1) * xp;
      }
      dt = a == 0 ? min2x(sm, sp) : min3x(dt, sm, sp);
      if (pos ? positive(gp) : negative(gp)) gp = 0.0;  // sgn * gp > 0
      if (pos ? negative(gm) : positive(gm)) gm = 0.0;  // sgn * gm < 0
      const double ha = max2x(gp * gp, gm * gm);
      h = a == 0 ? ha : h + ha;
    }
    dt = D == 3 ? div3(dt) : qdiv(dt, (double)D);
    r = f0 - times_sign(dt, pos) * (sqrt(h) - 1.);
    if (product_negative(p0, r)) r = neg1(r);
  }
  if (AVG) r = scale2(avg_with[n] + r, -1);
  out[n] = r;
}

template <int D, bool AVG>
__global__ void __launch_bounds__(TPB, 6) k_advect_stage64(DTab64<D> T, const double* __restrict__ phin, const double* __restrict__ ddq,
                                                        const double* __restrict__ ddm, const double* __restrict__ vn, double dt,
                                                        double* out, const double* avg_with, int64_t first, int64_t last) {
  const int64_t n = first + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t N = T.N;
  if (n >= last) return;
  const double f0 = phin[n];
  double Dq[D];
#pragma unroll
  for (int a = 0; a < D; ++a) Dq[a] = ddq[(int64_t)a * N + n];
  double fnb[2 * D], s[2 * D], xx0[D], xxnb[2 * D];
  const NodeWord nw = node_word<D>(T, n);
#pragma unroll
  for (int dir = 0; dir < 2 * D; ++dir) {
    fnb[dir] = quad_nb64<D>(T, dir, n, phin, Dq, nw);
    s[dir] = T.d[(int64_t)dir * N + n];
  }
#pragma unroll
  for (int a = 0; a < D; ++a) {
    xx0[a] = ddm[(int64_t)a * N + n];
    xxnb[2 * a] = lin64w<D>(T, 2 * a, n, ddm + (int64_t)a * N, nw);
    xxnb[2 * a + 1] = lin64w<D>(T, 2 * a + 1, n, ddm + (int64_t)a * N, nw);
  }
  const uint8_t wl = T.wall[n];
#pragma unroll
  for (int a = 0; a < D; ++a) {
    if (wl & (1u << (2 * a))) {
      s[2 * a] = s[2 * a + 1];
      fnb[2 * a] = fnb[2 * a + 1];
      xx0[a] = xxnb[2 * a] = xxnb[2 * a + 1] = 0.0;
    }
    if (wl & (1u << (2 * a + 1))) {
      s[2 * a + 1] = s[2 * a];
      fnb[2 * a + 1] = fnb[2 * a];
      xx0[a] = xxnb[2 * a] = xxnb[2 * a + 1] = 0.0;
    }
  }
  double gp[D], gm[D];
#pragma unroll
  for (int a = 0; a < D; ++a) {
    gp[a] = qdiv(fnb[2 * a + 1] - f0, s[2 * a + 1]);
    gm[a] = qdiv(f0 - fnb[2 * a], s[2 * a]);
  }
#pragma unroll
  for (int a = 0; a < D; ++a) {
    const double xm = minmod_x(xxnb[2 * a], xx0[a]);
    gm[a] = gm[a] + scale2(s[2 * a], -1) * xm;
    const double xp = minmod_x(xxnb[2 * a + 1], xx0[a]);
    gp[a] = gp[a] - scale2(s[2 * a + 1], -1) * xp;
  }
  const double v = vn[n];
  // sgn = (v > 0 ? 1 : -1); sgn * g is +-g exactly, so the upwind tests are sign tests of g
  const bool pos = positive(v);
#pragma unroll
  for (int a = 0; a < D; ++a) {
    if (pos ? positive(gp[a]) : negative(gp[a])) gp[a] = 0.0;  // sgn * gp > 0
    if (pos ? negative(gm[a]) : positive(gm[a])) gm[a] = 0.0;  // sgn * gm < 0
  }
  double h = (gp[0] * gp[0] + gm[0] * gm[0]) + (gp[1] * gp[1] + gm[1] * gm[1]);
  if (D == 3) h = h + (gp[2 % D] * gp[2 % D] + gm[2 % D] * gm[2 % D]);
  double r = f0 - dt * v * (sqrt(h));
  if (AVG) r = scale2(avg_with[n] + r, -1);
  out[n] = r;
}

__global__ void k_copy64(const double* __restrict__ a, double* __restrict__ b, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = a[i];
}

// dt = min over nodes of 0.8*|s_min/vn| (min is exact in any order). Values are non-negative, so
// their IEEE bit patterns order like unsigned integers and an atomicMin on the bits is exact.
__global__ void k_min_cfl(const double* __restrict__ smin, const double* __restrict__ vn, int64_t n, unsigned long long* out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double v = 1.7976931348623157e308;
  if (i < n) v = 0.8 * fabs(smin[i] / vn[i]);
  for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
  if ((threadIdx.x & 31) == 0) atomicMin(out, (unsigned long long)__double_as_longlong(v));
}

// d_a f at node n: central_derivative of the linearly interpolated neighbours along a
// (src/my_p4est_quad_neighbor_nodes_of_node.h:193-199), minus the tangential second-derivative
// corrections that apply (correct_naive_first_derivatives, .cpp:575-640)
template <int D>
__device__ __forceinline__ double grad_comp64(const DTab64<D>& T, const DGrad& G, int64_t n, const double* __restrict__ f,
                                              const double* __restrict__ fdd, int a, int32_t r) {
  const int64_t N = T.N;
  const double f0 = f[n];
  const double fm = lin64<D>(T, 2 * a, n, f), fp = lin64<D>(T, 2 * a + 1, n, f);
  const double dm = T.d[(int64_t)(2 * a) * N + n], dp = T.d[(int64_t)(2 * a + 1) * N + n];
  double g = qdiv(qdiv((fp - f0) * dm, dp) + qdiv((f0 - fm) * dp, dm), dp + dm);
  if (r >= 0) {
    const uint8_t mask = G.gmask[r];
#pragma unroll
    for (int j = 0; j < D - 1; ++j) {
      const int b = (j == 0) ? (a == 0 ? 1 : 0) : (a == 2 ? 1 : 2);
      if ((mask >> (a * (D - 1) + j)) & 1) g -= fdd[(int64_t)b * N + n] * G.grec[(int64_t)r * (D * (D - 1)) + a * (D - 1) + j];
    }
  }
  return g;
}

template <int D>
__global__ void __launch_bounds__(TPB) k_grad64(DTab64<D> T, DGrad G, const double* __restrict__ f, const double* __restrict__ fdd,
                                                double* __restrict__ out, int which) {
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= T.N) return;
  const int32_t r = G.gidx[n];
#pragma unroll
  for (int a = 0; a < D; ++a)
    if ((which >> a) & 1) out[(int64_t)a * T.N + n] = grad_comp64<D>(T, G, n, f, fdd, a, r);
}

template <int D>
__global__ void __launch_bounds__(TPB) k_normalize64(double* __restrict__ g, int64_t N) {
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  double s = g[n] * g[n] + g[N + n] * g[N + n];
  if (D == 3) s = s + g[2 * N + n] * g[2 * N + n];
  const double abs = sqrt(s);
#pragma unroll
  for (int a = 0; a < D; ++a) g[(int64_t)a * N + n] = abs < EPS ? 0.0 : g[(int64_t)a * N + n] / abs;
}

template <int D>
__global__ void __launch_bounds__(TPB) k_div64(DTab64<D> T, DGrad G, const double* __restrict__ nrm, const double* __restrict__ ndd,
                                               double* __restrict__ kappa) {
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t N = T.N;
  if (n >= N) return;
  const int32_t r = G.gidx[n];
  double k = grad_comp64<D>(T, G, n, nrm, ndd, 0, r) + grad_comp64<D>(T, G, n, nrm + N, ndd + (int64_t)D * N, 1, r);
  if (D == 3) k = k + grad_comp64<D>(T, G, n, nrm + 2 * N, ndd + (int64_t)2 * D * N, 2, r);
  kappa[n] = k;
}

template <int D>
__global__ void __launch_bounds__(TPB) k_kappa64(DTab64<D> T, DGrad G, const double* __restrict__ g, const double* __restrict__ phidd,
                                                 const double* __restrict__ gxdd, const double* __restrict__ gydd,
                                                 double* __restrict__ kappa) {
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t N = T.N;
  if (n >= N) return;
  const double dx = g[n], dy = g[N + n], dz = D == 3 ? g[2 * N + n] : 0.0;
  double mag = 0.0;
  mag += dx * dx;
  mag += dy * dy;
  if (D == 3) mag += dz * dz;
  mag = sqrt(mag);
  if (!(mag > EPS)) {
    kappa[n] = 0.0;
    return;
  }
  const int32_t r = G.gidx[n];
  const double d0 = phidd[n], d1 = phidd[N + n];
  const double dxy = grad_comp64<D>(T, G, n, g, gxdd, 1, r);
  if (D == 3) {
    const double d2 = phidd[2 * N + n];
    const double dxz = grad_comp64<D>(T, G, n, g, gxdd, 2, r);
    const double dyz = grad_comp64<D>(T, G, n, g + N, gydd, 2, r);
    kappa[n] = ((d1 + d2) * (dx * dx) + (d0 + d2) * (dy * dy) + (d0 + d1) * (dz * dz) - 2.0 * (dx * dy * dxy + dx * dz * dxz + dy * dz * dyz)) /
               (mag * mag * mag);
  } else {
    kappa[n] = ((d1) * (dx * dx) + (d0) * (dy * dy) - 2.0 * (dx * dy * dxy)) / (mag * mag * mag);
  }
}

// ---- extend_Over_Interface_TVD (src/my_p4est_level_set.cpp:969-1764) ------------------------------
// is_stencil_in_negative_domain (src/my_p4est_quad_neighbor_nodes_of_node.h:2492-2530): the node and
// every face node with a nonzero interpolation weight below -EPS
template <int D>
__device__ __forceinline__ bool stencil_negative64(const DTab64<D>& T, int64_t n, const double* __restrict__ f) {
  constexpr int NS = 2 * D * Dim<D>::HALF;
  if (!(f[n] < -EPS)) return false;
#pragma unroll
  for (int sl = 0; sl < NS; ++sl) {
    const int32_t j = T.nbr[(int64_t)sl * T.N + n];
    if (j >= 0 && !(f[j] < -EPS)) return false;
  }
  return true;
}
template <int D>
__device__ __forceinline__ bool stencil_negative_flag(const DTab64<D>& T, int64_t n, const int8_t* __restrict__ b) {
  constexpr int NS = 2 * D * Dim<D>::HALF;
  if (!(b[n] < 0)) return false;
#pragma unroll
  for (int sl = 0; sl < NS; ++sl) {
    const int32_t j = T.nbr[(int64_t)sl * T.N + n];
    if (j >= 0 && !(b[j] < 0)) return false;
  }
  return true;
}

template <int D>
__device__ __forceinline__ double ext_dt(const DTab64<D>& T, int64_t n) {
  const int64_t N = T.N;
  auto d = [&](int dir) { return fabs(T.d[(int64_t)dir * N + n]); };
  const double m = D == 3 ? min2(min3(d(0), d(2), d(4)), min3(d(1), d(3), d(5))) : min2(min2(d(0), d(2)), min2(d(1), d(3)));
  return m / double(D);
}

template <int D>
__global__ void __launch_bounds__(TPB) k_ext_init1(DTab64<D> T, DGrad G, const double* __restrict__ phi, const double* __restrict__ mask,
                                                   const double* __restrict__ q, const double* __restrict__ qdd, const double* __restrict__ nrm,
                                                   double band_use, int guess, double* __restrict__ qx, double* __restrict__ qn,
                                                   int8_t* __restrict__ bqn) {
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t N = T.N;
  if (n >= N) return;
  if (phi[n] > band_use && !stencil_negative64<D>(T, n, mask)) {
    // no value can be computed here: the caller's guess (use_nonzero_guess: n . grad q; a given q_n: its
    // value), else zero
    bqn[n] = 1;
    if (guess & EXT_GUESS_GRADIENT) {
      const int32_t r = G.gidx[n];
      double s = nrm[n] * grad_comp64<D>(T, G, n, q, qdd, 0, r) + nrm[N + n] * grad_comp64<D>(T, G, n, q, qdd, 1, r);
      if (D == 3) s = s + nrm[2 * N + n] * grad_comp64<D>(T, G, n, q, qdd, D == 3 ? 2 : 0, r);
      qn[n] = s;
    } else if (!(guess & EXT_GUESS_KEEP)) {
      qn[n] = 0;
    }
#pragma unroll
    for (int a = 0; a < D; ++a) qx[(int64_t)a * N + n] = 0;
    return;
  }
  if (phi[n] > band_use) {
    const int32_t r = G.gidx[n];
    double g[3];
#pragma unroll
    for (int a = 0; a < D; ++a) {
      g[a] = grad_comp64<D>(T, G, n, q, qdd, a, r);
      qx[(int64_t)a * N + n] = g[a];
    }
    double s = nrm[n] * g[0] + nrm[N + n] * g[1];
    if (D == 3) s = s + nrm[2 * N + n] * g[2];
    qn[n] = s;
    bqn[n] = -1;
  } else {
    bqn[n] = -1;
    qn[n] = 0;
#pragma unroll
    for (int a = 0; a < D; ++a) qx[(int64_t)a * N + n] = 0;
  }
}

template <int D>
__global__ void __launch_bounds__(TPB) k_ext_init2(DTab64<D> T, DGrad G, const double* __restrict__ phi, const double* __restrict__ mask,
                                                   const double* __restrict__ q, const double* __restrict__ qdd, const double* __restrict__ nrm,
                                                   const double* __restrict__ nrmdd, const double* __restrict__ qx,
                                                   const double* __restrict__ qxdd, const int8_t* __restrict__ bqn,
                                                   const int32_t* __restrict__ cnb, double band_use, int guess, const double* __restrict__ qn,
                                                   const double* __restrict__ qndd, double* __restrict__ qnn, int8_t* __restrict__ bqnn) {
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t N = T.N;
  if (n >= N) return;
  if (!(phi[n] > band_use)) {
    bqnn[n] = -1;
    qnn[n] = 0;
    return;
  }
  const int32_t r = G.gidx[n];
  if (!stencil_negative64<D>(T, n, mask)) {
    bqnn[n] = 1;
    if (guess & EXT_GUESS_GRADIENT) {
      const int64_t N_ = N;
      double s = nrm[n] * grad_comp64<D>(T, G, n, qn, qndd, 0, r) + nrm[N_ + n] * grad_comp64<D>(T, G, n, qn, qndd, 1, r);
      if (D == 3) s = s + nrm[2 * N_ + n] * grad_comp64<D>(T, G, n, qn, qndd, D == 3 ? 2 : 0, r);
      qnn[n] = s;
    } else if (!(guess & EXT_GUESS_KEEP)) {
      qnn[n] = 0;
    }
    return;
  }
  const int64_t DN = (int64_t)D * N;
  double Qxy = 0, Qyz = 0, Qzx = 0;
  bool ok = false;
  if (stencil_negative_flag<D>(T, n, bqn)) {
    ok = true;
    Qxy = scale2(grad_comp64<D>(T, G, n, qx + N, qxdd + DN, 0, r) + grad_comp64<D>(T, G, n, qx, qxdd, 1, r), -1);
    if (D == 3) {
      Qyz = scale2(grad_comp64<D>(T, G, n, qx + 2 * N, qxdd + 2 * DN, 1, r) + grad_comp64<D>(T, G, n, qx + N, qxdd + DN, 2, r), -1);
      Qzx = scale2(grad_comp64<D>(T, G, n, qx, qxdd, 2, r) + grad_comp64<D>(T, G, n, qx + 2 * N, qxdd + 2 * DN, 0, r), -1);
    }
  } else {
    constexpr int K = D == 3 ? 12 : 4;
    int32_t nb[K];
    bool exist = true;
#pragma unroll
    for (int k = 0; k < K; ++k) {
      nb[k] = cnb[(int64_t)k * N + n];
      exist = exist && nb[k] >= 0;
    }
    if (exist) {
      bool neg = true;
#pragma unroll
      for (int k = 0; k < K; ++k) neg = neg && mask[nb[k]] < 0;
      if (neg) {
        const double dx = T.d[n] + T.d[N + n], dy = T.d[2 * N + n] + T.d[3 * N + n];
        const int mm0 = D == 3 ? 8 : 0, pm0 = D == 3 ? 9 : 1, mp0 = D == 3 ? 10 : 2, pp0 = D == 3 ? 11 : 3;
        Qxy = qdiv(qdiv(q[nb[pp0]] + q[nb[mm0]] - q[nb[mp0]] - q[nb[pm0]], dx), dy);
        if (D == 3) {
          const double dz = T.d[4 * N + n] + T.d[5 * N + n];
          Qyz = qdiv(qdiv(q[nb[7]] + q[nb[4]] - q[nb[6]] - q[nb[5]], dy), dz);
          Qzx = qdiv(qdiv(q[nb[3]] + q[nb[0]] - q[nb[1]] - q[nb[2]], dz), dx);
        }
        ok = true;
      }
    }
  }
  if (!ok) {
    bqnn[n] = 1;
    if (!(guess & EXT_GUESS_KEEP)) qnn[n] = 0;  // left as it was: zero, or the caller's q_nn
    return;
  }
  bqnn[n] = -1;
  // dxx_central etc. of q: central second differences of the quadratically corrected neighbours
  // (x_ngbd_with_quadratic_interpolation, src/my_p4est_quad_neighbor_nodes_of_node.cpp:365-390)
  double Dq[D], Qaa[D];
#pragma unroll
  for (int a = 0; a < D; ++a) Dq[a] = qdd[(int64_t)a * N + n];
#pragma unroll
  for (int a = 0; a < D; ++a) {
    const double fp = quad_nb64<D>(T, 2 * a + 1, n, q, Dq), fm = quad_nb64<D>(T, 2 * a, n, q, Dq);
    const double dp = T.d[(int64_t)(2 * a + 1) * N + n], dm = T.d[(int64_t)(2 * a) * N + n];
    Qaa[a] = qdiv(scale2(qdiv(fp - q[n], dp) + qdiv(fm - q[n], dm), 1), dp + dm);
  }
  const double Qx = qx[n], Qy = qx[N + n];
  const double Nx = nrm[n], Ny = nrm[N + n];
  const double Nxx = grad_comp64<D>(T, G, n, nrm, nrmdd, 0, r), Nyx = grad_comp64<D>(T, G, n, nrm + N, nrmdd + DN, 0, r);
  const double Nxy = grad_comp64<D>(T, G, n, nrm, nrmdd, 1, r), Nyy = grad_comp64<D>(T, G, n, nrm + N, nrmdd + DN, 1, r);
  if (D == 3) {
    const double Qz = qx[2 * N + n], Nz = nrm[2 * N + n];
    const double Nzx = grad_comp64<D>(T, G, n, nrm + 2 * N, nrmdd + 2 * DN, 0, r);
    const double Nzy = grad_comp64<D>(T, G, n, nrm + 2 * N, nrmdd + 2 * DN, 1, r);
    const double Nxz = grad_comp64<D>(T, G, n, nrm, nrmdd, 2, r), Nyz = grad_comp64<D>(T, G, n, nrm + N, nrmdd + DN, 2, r);
    const double Nzz = grad_comp64<D>(T, G, n, nrm + 2 * N, nrmdd + 2 * DN, 2, r);
    qnn[n] = Nx * (Nx * Qaa[0] + 2. * Ny * Qxy + Qx * Nxx + Qy * Nyx + Qz * Nzx) +
             Ny * (Ny * Qaa[1] + 2. * Nz * Qyz + Qx * Nxy + Qy * Nyy + Qz * Nzy) +
             Nz * (Nz * Qaa[D == 3 ? 2 : 0] + 2. * Nx * Qzx + Qx * Nxz + Qy * Nyz + Qz * Nzz);
  } else {
    qnn[n] = Nx * (Nx * Qaa[0] + 2. * Ny * Qxy + Qx * Nxx + Qy * Nyx) + Ny * (Ny * Qaa[1] + Qx * Nxy + Qy * Nyy);
  }
}

template <int D, bool SRC>
__global__ void __launch_bounds__(TPB) k_ext_march(DTab64<D> T, const double* __restrict__ v, double* __restrict__ tmp,
                                                   const int8_t* __restrict__ b, const double* __restrict__ phi,
                                                   const double* __restrict__ nrm, const double* __restrict__ src, double band_extend) {
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t N = T.N;
  if (n >= N) return;
  if (!(b[n] > 0 && phi[n] < band_extend)) return;
  const double dt = ext_dt<D>(T, n);
  double g[3];
#pragma unroll
  for (int a = 0; a < D; ++a)
    g[a] = nrm[(int64_t)a * N + n] > 0 ? qdiv(v[n] - lin64<D>(T, 2 * a, n, v), T.d[(int64_t)(2 * a) * N + n])
                                        : qdiv(lin64<D>(T, 2 * a + 1, n, v) - v[n], T.d[(int64_t)(2 * a + 1) * N + n]);
  double s = nrm[n] * g[0] + nrm[N + n] * g[1];
  if (D == 3) s = s + nrm[2 * N + n] * g[2];
  tmp[n] = SRC ? v[n] - dt * (s - src[n]) : v[n] - dt * s;
}

template <int D, int ORDER>
__global__ void __launch_bounds__(TPB) k_ext_q(DTab64<D> T, const double* __restrict__ q, double* __restrict__ tmp,
                                               const double* __restrict__ qdd, const double* __restrict__ phi, const double* __restrict__ mask,
                                               const double* __restrict__ nrm, const double* __restrict__ qn, double band_extend) {
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t N = T.N;
  if (n >= N) return;
  if (!(mask[n] > -EPS && phi[n] < band_extend)) return;
  const double dt = ext_dt<D>(T, n);
  double g[3];
#pragma unroll
  for (int a = 0; a < D; ++a)
    g[a] = nrm[(int64_t)a * N + n] > 0 ? qdiv(q[n] - lin64<D>(T, 2 * a, n, q), T.d[(int64_t)(2 * a) * N + n])
                                        : qdiv(lin64<D>(T, 2 * a + 1, n, q) - q[n], T.d[(int64_t)(2 * a + 1) * N + n]);
  if (ORDER == 2) {
#pragma unroll
    for (int a = 0; a < D; ++a) {
      const double* qaa = qdd + (int64_t)a * N;
      const double c = qaa[n];
      double qm = lin64<D>(T, 2 * a, n, qaa), qp = lin64<D>(T, 2 * a + 1, n, qaa);
      qm = c * qm < 0 ? 0 : (fabs(c) < fabs(qm) ? c : qm);
      qp = c * qp < 0 ? 0 : (fabs(c) < fabs(qp) ? c : qp);
      if (nrm[(int64_t)a * N + n] < 0)
        g[a] -= scale2(T.d[(int64_t)(2 * a + 1) * N + n], -1) * qp;
      else
        g[a] += scale2(T.d[(int64_t)(2 * a) * N + n], -1) * qm;
    }
  }
  double s = nrm[n] * g[0] + nrm[N + n] * g[1];
  if (D == 3) s = s + nrm[2 * N + n] * g[2];
  const double change = dt * (s - (ORDER >= 1 ? qn[n] : 0));
  tmp[n] = q[n] - change;
}

// ---- extend_from_interface_to_whole_domain_TVD_one_iteration (src/my_p4est_level_set.cpp:3181-3323) --------
// One TVD-RK2 stage for one field: Godunov upwinding along sgn(phi) grad(phi)/|grad(phi)| with
// second-order one-sided differences (minmod of the quadratically interpolated second derivatives),
// the neighbour across the interface replaced by the interface value at the subcell distance
// (qi_nb, s_nb, cross from the set-up kernel), Neumann walls. qdd: D x N second derivatives of q;
// qdd2: D x D x N second derivatives of each of them. AVG: out = 0.5 (out + stage), the RK average.
template <int D, bool AVG>
__global__ void __launch_bounds__(TPB) k_efi_stage64(DTab64<D> T, const double* __restrict__ phi, const double* __restrict__ grad,
                                                     const double* __restrict__ q, const double* __restrict__ qdd,
                                                     const double* __restrict__ qdd2, const double* __restrict__ qi_nb,
                                                     const double* __restrict__ s_nb, const uint8_t* __restrict__ cross, double zdt,
                                                     double* __restrict__ out) {
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t N = T.N;
  if (n >= N) return;
  double res;
  if (fabs(phi[n]) < zdt) {
    res = q[n];
  } else {
    double Dq[D];
#pragma unroll
    for (int a = 0; a < D; ++a) Dq[a] = qdd[(int64_t)a * N + n];
    const double q0 = q[n];
    const uint8_t cr = cross[n];
    double qn[2 * D], s[2 * D];
#pragma unroll
    for (int dir = 0; dir < 2 * D; ++dir) {
      s[dir] = s_nb[(int64_t)dir * N + n];
      qn[dir] = (cr >> dir) & 1 ? qi_nb[(int64_t)dir * N + n] : quad_nb64<D>(T, dir, n, q, Dq);
    }
    double d0[D], dm[D], dp[D];
#pragma unroll
    for (int a = 0; a < D; ++a) {
      const double* qaa = qdd + (int64_t)a * N;
      double Da[D];
#pragma unroll
      for (int b = 0; b < D; ++b) Da[b] = qdd2[(int64_t)(a * D + b) * N + n];
      d0[a] = qaa[n];
      dm[a] = quad_nb64<D>(T, 2 * a, n, qaa, Da);
      dp[a] = quad_nb64<D>(T, 2 * a + 1, n, qaa, Da);
    }
    const uint8_t wl = T.wall[n];
#pragma unroll
    for (int a = 0; a < D; ++a) {
      if (wl & (1u << (2 * a))) {
        s[2 * a] = s[2 * a + 1];
        qn[2 * a] = qn[2 * a + 1];
        d0[a] = dm[a] = dp[a] = 0.0;
      } else if (wl & (1u << (2 * a + 1))) {
        s[2 * a + 1] = s[2 * a];
        qn[2 * a + 1] = qn[2 * a];
        d0[a] = dm[a] = dp[a] = 0.0;
      }
    }
    double dt = min2(s[0], s[1]);
    dt = min3(dt, s[2], s[3]);
    if (D == 3) dt = min3(dt, s[D == 3 ? 4 : 0], s[D == 3 ? 5 : 0]);
    dt = qdiv(dt, (double)D);
    const double gx = grad[n], gy = grad[N + n], gz = D == 3 ? grad[(D == 3 ? 2 : 0) * N + n] : 0.0;
    const double mag = D == 3 ? sqrt(gx * gx + gy * gy + gz * gz) : sqrt(gx * gx + gy * gy);
    const double sg = phi[n] < 0.0 ? -1.0 : +1.0;
    const double nv[3] = {mag > EPS ? sg * gx / mag : 0.0, mag > EPS ? sg * gy / mag : 0.0, mag > EPS ? sg * gz / mag : 0.0};
    double t[3];
#pragma unroll
    for (int a = 0; a < D; ++a) {
      const double qm = qdiv(q0 - qn[2 * a], s[2 * a]) + scale2(s[2 * a], -1) * minmod(dm[a], d0[a]);
      const double qp = qdiv(qn[2 * a + 1] - q0, s[2 * a + 1]) - scale2(s[2 * a + 1], -1) * minmod(dp[a], d0[a]);
      t[a] = nv[a] * (nv[a] > 0.0 ? qm : qp);
    }
    res = q0 - dt * (D == 3 ? (t[0] + t[1] + t[D == 3 ? 2 : 0]) : (t[0] + t[1]));
  }
  if (AVG)
    out[n] = scale2(out[n] + res, -1);
  else
    out[n] = res;
}

// Band L-infinity check in FP64: max |a - b| over the nodes with |b| < band (b the reference field),
// with the number of band nodes and a NaN flag. Warp shuffles, then one shared-memory pass per block,
// then one atomic per block; non-negative doubles order like their bit patterns, so atomicMax on the
// bits is exact and the result does not depend on the reduction order.
__global__ void __launch_bounds__(TPB) k_band_linf64(const double* __restrict__ a, const double* __restrict__ b, double band, int64_t n,
                                                     unsigned long long* __restrict__ out) {
  __shared__ double s_max[TPB / 32];
  __shared__ unsigned long long s_cnt[TPB / 32];
  __shared__ int s_nan[TPB / 32];
  double m = 0.0;
  unsigned long long cnt = 0;
  int nan = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double r = b[i];
    if (fabs(r) < band) {
      const double e = fabs(a[i] - r);
      if (e != e) nan = 1;
      else m = fmax(m, e);
      ++cnt;
    } else if (r != r) {
      nan = 1;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    nan |= __shfl_xor_sync(0xffffffffu, nan, o);
  }
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) {
    s_max[w] = m;
    s_cnt[w] = cnt;
    s_nan[w] = nan;
  }
  __syncthreads();
  if (w == 0) {
    const int nw = blockDim.x >> 5;
    m = lane < nw ? s_max[lane] : 0.0;
    cnt = lane < nw ? s_cnt[lane] : 0ull;
    nan = lane < nw ? s_nan[lane] : 0;
    for (int o = 16; o > 0; o >>= 1) {
      m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
      cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
      nan |= __shfl_xor_sync(0xffffffffu, nan, o);
    }
    if (lane == 0) {
      atomicMax(out, (unsigned long long)__double_as_longlong(m));
      atomicAdd(out + 1, cnt);
      if (nan) atomicOr(out + 2, 1ull);
    }
  }
}

// Interface location along cut grid edges, in FP64: every node n and direction whose stencil slot holds
// a single node (a grid edge to a node at distance d) where the reference field b changes sign; the crossing
// lies at t_b = d b_n / (b_n - b_nb) from n (the linear root along the edge). Where a changes sign on the same
// edge, |t_a - t_b| enters the maximum; otherwise the edge counts as a sign mismatch. out: max bits, cut edges,
// mismatched edges (each edge is seen from both ends). Same reduction as k_band_linf64.
template <int D>
__global__ void __launch_bounds__(TPB) k_iface_err64(DTab64<D> T, const double* __restrict__ a, const double* __restrict__ b,
                                                     unsigned long long* __restrict__ out) {
  constexpr int H = Dim<D>::HALF;
  __shared__ double s_max[TPB / 32];
  __shared__ unsigned long long s_cnt[TPB / 32], s_mis[TPB / 32];
  const int64_t N = T.N;
  double m = 0.0;
  unsigned long long cnt = 0, mis = 0;
  for (int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; n < N; n += (int64_t)gridDim.x * blockDim.x) {
    const double b0 = b[n], a0 = a[n];
#pragma unroll
    for (int dir = 0; dir < 2 * D; ++dir) {
      const int64_t base = (int64_t)(dir * H) * N + n;
      bool single = true;
#pragma unroll
      for (int k = 1; k < H; ++k) single = single && T.nbr[base + k * N] < 0;
      const int32_t nb = T.nbr[base];
      if (!single || nb < 0 || nb == n) continue;
      const double b1 = b[nb];
      if (!(b0 * b1 < 0.0)) continue;
      ++cnt;
      const double a1 = a[nb];
      if (!(a0 * a1 < 0.0)) {
        ++mis;
        continue;
      }
      const double d = T.d[(int64_t)dir * N + n];
      const double tb = d * b0 / (b0 - b1), ta = d * a0 / (a0 - a1);
      m = fmax(m, fabs(ta - tb));
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    mis += __shfl_xor_sync(0xffffffffu, mis, o);
  }
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) {
    s_max[w] = m;
    s_cnt[w] = cnt;
    s_mis[w] = mis;
  }
  __syncthreads();
  if (w == 0) {
    const int nw = blockDim.x >> 5;
    m = lane < nw ? s_max[lane] : 0.0;
    cnt = lane < nw ? s_cnt[lane] : 0ull;
    mis = lane < nw ? s_mis[lane] : 0ull;
    for (int o = 16; o > 0; o >>= 1) {
      m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
      cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
      mis += __shfl_xor_sync(0xffffffffu, mis, o);
    }
    if (lane == 0) {
      atomicMax(out, (unsigned long long)__double_as_longlong(m));
      atomicAdd(out + 1, cnt);
      atomicAdd(out + 2, mis);
    }
  }
}

inline unsigned nblocks(int64_t n) { return (unsigned)((n + TPB - 1) / TPB); }

}  // namespace

template <int D>
void launch_grad64(const DTab64<D>& T, const DGrad& G, const double* f, const double* fdd, double* out, int which, cudaStream_t s) {
  if (T.N) k_grad64<D><<<nblocks(T.N), TPB, 0, s>>>(T, G, f, fdd, out, which);
}
template <int D>
void launch_normalize64(double* g, int64_t N, cudaStream_t s) {
  if (N) k_normalize64<D><<<nblocks(N), TPB, 0, s>>>(g, N);
}
template <int D>
void launch_div64(const DTab64<D>& T, const DGrad& G, const double* nrm, const double* ndd, double* kappa, cudaStream_t s) {
  if (T.N) k_div64<D><<<nblocks(T.N), TPB, 0, s>>>(T, G, nrm, ndd, kappa);
}
template <int D>
void launch_kappa64(const DTab64<D>& T, const DGrad& G, const double* g, const double* phidd, const double* gxdd, const double* gydd,
                    double* kappa, cudaStream_t s) {
  if (T.N) k_kappa64<D><<<nblocks(T.N), TPB, 0, s>>>(T, G, g, phidd, gxdd, gydd, kappa);
}

template <int D>
void launch_ext_init1(const DTab64<D>& T, const DGrad& G, const double* phi, const double* mask, const double* q, const double* qdd,
                      const double* nrm, double band_use, int guess, double* qx, double* qn, int8_t* bqn, cudaStream_t s) {
  if (T.N) k_ext_init1<D><<<nblocks(T.N), TPB, 0, s>>>(T, G, phi, mask, q, qdd, nrm, band_use, guess, qx, qn, bqn);
}
template <int D>
void launch_ext_init2(const DTab64<D>& T, const DGrad& G, const double* phi, const double* mask, const double* q, const double* qdd,
                      const double* nrm, const double* nrmdd, const double* qx, const double* qxdd, const int8_t* bqn, const int32_t* cnb,
                      double band_use, int guess, const double* qn, const double* qndd, double* qnn, int8_t* bqnn, cudaStream_t s) {
  if (T.N)
    k_ext_init2<D><<<nblocks(T.N), TPB, 0, s>>>(T, G, phi, mask, q, qdd, nrm, nrmdd, qx, qxdd, bqn, cnb, band_use, guess, qn, qndd, qnn, bqnn);
}
template <int D>
void launch_ext_march(const DTab64<D>& T, const double* v, double* tmp, const int8_t* b, const double* phi, const double* nrm,
                      const double* src, double band_extend, cudaStream_t s) {
  if (!T.N) return;
  if (src)
    k_ext_march<D, true><<<nblocks(T.N), TPB, 0, s>>>(T, v, tmp, b, phi, nrm, src, band_extend);
  else
    k_ext_march<D, false><<<nblocks(T.N), TPB, 0, s>>>(T, v, tmp, b, phi, nrm, src, band_extend);
}
template <int D>
void launch_ext_q(const DTab64<D>& T, const double* q, double* tmp, const double* qdd, const double* phi, const double* mask,
                  const double* nrm, const double* qn, int order, double band_extend, cudaStream_t s) {
  if (!T.N) return;
  if (order == 2)
    k_ext_q<D, 2><<<nblocks(T.N), TPB, 0, s>>>(T, q, tmp, qdd, phi, mask, nrm, qn, band_extend);
  else if (order == 1)
    k_ext_q<D, 1><<<nblocks(T.N), TPB, 0, s>>>(T, q, tmp, qdd, phi, mask, nrm, qn, band_extend);
  else
    k_ext_q<D, 0><<<nblocks(T.N), TPB, 0, s>>>(T, q, tmp, qdd, phi, mask, nrm, qn, band_extend);
}

template <int D>
void launch_efi_stage64(const DTab64<D>& T, const double* phi, const double* grad, const double* q, const double* qdd, const double* qdd2,
                        const double* qi_nb, const double* s_nb, const uint8_t* cross, double zdt, bool average, double* out,
                        cudaStream_t s) {
  if (!T.N) return;
  if (average)
    k_efi_stage64<D, true><<<nblocks(T.N), TPB, 0, s>>>(T, phi, grad, q, qdd, qdd2, qi_nb, s_nb, cross, zdt, out);
  else
    k_efi_stage64<D, false><<<nblocks(T.N), TPB, 0, s>>>(T, phi, grad, q, qdd, qdd2, qi_nb, s_nb, cross, zdt, out);
}

// reinitialize_2nd_order_with_mask (src/my_p4est_level_set.h:487-525): nodes whose mask is 0 are left out
// of the updates and keep their value, which is what ST_OUTSIDE gives (phi_np1 = phi_np2 = phi_0 = phi_n at
// those nodes). perm (device index -> node) is null for node-ordered status arrays.
__global__ void k_apply_mask(const double* __restrict__ mask, const int32_t* __restrict__ perm, uint16_t* __restrict__ status, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (mask[perm ? perm[i] : i] == 0.0) status[i] = ST_OUTSIDE;
}

void launch_apply_mask(const double* mask, const int32_t* perm, uint16_t* status, int64_t n, cudaStream_t s) {
  if (n) k_apply_mask<<<nblocks(n), TPB, 0, s>>>(mask, perm, status, n);
}

void launch_band_linf64(const double* a, const double* b, double band, int64_t n, unsigned long long* out3, cudaStream_t s) {
  cudaMemsetAsync(out3, 0, 3 * sizeof(unsigned long long), s);
  if (n == 0) return;
  const unsigned g = std::min<unsigned>(nblocks(n), (unsigned)device_sm_count() * 8u);
  k_band_linf64<<<g, TPB, 0, s>>>(a, b, band, n, out3);
}

template <int D>
void launch_iface_err64(const DTab64<D>& T, const double* a, const double* b, unsigned long long* out3, cudaStream_t s) {
  cudaMemsetAsync(out3, 0, 3 * sizeof(unsigned long long), s);
  if (T.N == 0) return;
  const unsigned g = std::min<unsigned>(nblocks(T.N), (unsigned)device_sm_count() * 8u);
  k_iface_err64<D><<<g, TPB, 0, s>>>(T, a, b, out3);
}

// Each sweep covers the nodes [first, first + count) (count < 0: every node from first on).
template <int D>
void launch_dd64(const DTab64<D>& T, const double* f, double* dd, cudaStream_t s, int64_t first, int64_t count) {
  const int64_t last = count < 0 ? T.N : first + count;
  if (last <= first) return;
  k_dd64<D><<<nblocks(last - first), TPB, 0, s>>>(T, f, dd, first, last);
}

template <int D>
void launch_reinit_prep64(const DTab64<D>& T, const double* phi0, const double* dd0, double zdt, double lim_lo, double lim_hi,
                          int order_space, uint16_t* status, double* s_near, cudaStream_t s, int64_t first, int64_t count) {
  const int64_t last = count < 0 ? T.N : first + count;
  if (last <= first) return;
  k_reinit_prep64<D><<<nblocks(last - first), TPB, 0, s>>>(T, phi0, dd0, zdt, lim_lo, lim_hi, order_space, status, s_near, first, last);
}

template <int D>
void launch_reinit_stage64(const DTab64<D>& T, int order_space, const uint16_t* status, const double* s_near, const double* phi0,
                           const double* phin, const double* dd, double* out, const double* avg_with, cudaStream_t s, int64_t first,
                           int64_t count) {
  const int64_t last = count < 0 ? T.N : first + count;
  if (last <= first) return;
  const unsigned g = nblocks(last - first);
  if (order_space > 1) {
    if (avg_with)
      k_reinit_stage64<D, 2, true><<<g, TPB, 0, s>>>(T, status, s_near, phi0, phin, dd, out, avg_with, first, last);
    else
      k_reinit_stage64<D, 2, false><<<g, TPB, 0, s>>>(T, status, s_near, phi0, phin, dd, out, avg_with, first, last);
  } else {
    if (avg_with)
      k_reinit_stage64<D, 1, true><<<g, TPB, 0, s>>>(T, status, s_near, phi0, phin, dd, out, avg_with, first, last);
    else
      k_reinit_stage64<D, 1, false><<<g, TPB, 0, s>>>(T, status, s_near, phi0, phin, dd, out, avg_with, first, last);
  }
}

template <int D>
void launch_advect_stage64(const DTab64<D>& T, const double* phin, const double* ddq, const double* ddm, const double* vn, double dt,
                           double* out, const double* avg_with, cudaStream_t s, int64_t first, int64_t count) {
  const int64_t last = count < 0 ? T.N : first + count;
  if (last <= first) return;
  if (avg_with)
    k_advect_stage64<D, true><<<nblocks(last - first), TPB, 0, s>>>(T, phin, ddq, ddm, vn, dt, out, avg_with, first, last);
  else
    k_advect_stage64<D, false><<<nblocks(last - first), TPB, 0, s>>>(T, phin, ddq, ddm, vn, dt, out, avg_with, first, last);
}

void launch_copy64(const double* src, double* dst, int64_t n, cudaStream_t s) {
  if (n == 0) return;
  k_copy64<<<nblocks(n), TPB, 0, s>>>(src, dst, n);
}

void launch_min_cfl(const double* smin, const double* vn, int64_t n, double* dt_out_dev, cudaStream_t s) {
  const double init = 1.7976931348623157e308;
  cudaMemcpyAsync(dt_out_dev, &init, sizeof(double), cudaMemcpyHostToDevice, s);
  if (n == 0) return;
  k_min_cfl<<<nblocks(n), TPB, 0, s>>>(smin, vn, n, (unsigned long long*)dt_out_dev);
}

// ---- FP64 tables in stencil-pattern order ---------------------------------------------------------------
// The FP64 sweeps run one thread per node; in the reference's node order a warp mixes nodes with one face node
// per direction and hanging ones (two or four, a division by a non-power-of-two d_m + d_p, a correction), and
// GB300's FP64 pipe pays every divergent branch for the whole warp. Sorting the nodes by their stencil pattern
// (face-node counts, correction, walls; node order within a pattern) gives warps one path. The tables are
// copied in that order with neighbour indices renumbered; the per-node arithmetic is unchanged, so results
// are bit for bit those of the node-ordered sweeps.
namespace {
template <int D>
__global__ void k_pattern_key64(DTab64<D> T, uint32_t* __restrict__ key, int32_t* __restrict__ idx) {
  constexpr int H = Dim<D>::HALF;
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= T.N) return;
  uint32_t k = 0;
#pragma unroll
  for (int dir = 0; dir < 2 * D; ++dir) {
    int cnt = 0;
#pragma unroll
    for (int j = 0; j < H; ++j) cnt += T.nbr[(int64_t)(dir * H + j) * T.N + n] >= 0 ? 1 : 0;
    k |= (uint32_t)(cnt > 0 ? cnt - 1 : 0) << (2 * dir);
  }
  if (T.cidx[n] >= 0) k |= 1u << 12;
  k |= (uint32_t)T.wall[n] << 13;
  key[n] = k;
  idx[n] = (int32_t)n;
}
// the pattern word of every node of tables in stencil-pattern order (DTab64::word)
template <int D>
__global__ void k_node_word64(DTab64<D> T, uint32_t* __restrict__ word) {
  constexpr int H = Dim<D>::HALF;
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= T.N) return;
  const int64_t N = T.N;
  uint32_t k = 0;
  for (int dir = 0; dir < 2 * D; ++dir) {
    int cnt = 0;
    for (int j = 0; j < H; ++j) cnt += T.nbr[(int64_t)(dir * H + j) * N + n] >= 0 ? 1 : 0;
    k |= (uint32_t)(cnt > 0 ? cnt - 1 : 0) << (2 * dir);
    bool single = T.nbr[(int64_t)(dir * H) * N + n] >= 0;
    for (int j = 1; j < H; ++j) single = single && T.nbr[(int64_t)(dir * H + j) * N + n] < 0;
    if (single) {
      const unsigned long long bw = bits_of(T.w[(int64_t)(dir * H) * N + n]);
      const int ew = (int)(bw >> 52);  // a positive weight: no sign bit
      if (bw == bits_of(T.nrm[(int64_t)dir * N + n]) && (bw & 0x000fffffffffffffull) == 0 && ew >= 623 && ew <= 1423)
        k |= 1u << (20 + dir);
    }
    bool nocorr;
    if (D == 2) nocorr = !nonzero(T.q[(int64_t)dir * N + n]);
    else nocorr = !nonzero(T.q[(int64_t)(2 * dir) * N + n]) && !nonzero(T.q[(int64_t)(2 * dir + 1) * N + n]);
    if (nocorr) k |= 1u << (26 + dir);
  }
  if (T.cidx[n] >= 0) k |= 1u << 12;
  k |= (uint32_t)T.wall[n] << 13;
  word[n] = k;
}

__global__ void k_inverse_perm(const int32_t* __restrict__ perm, int32_t* __restrict__ iperm, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) iperm[perm[i]] = (int32_t)i;
}
template <int D>
__global__ void k_permute_tab64(DTab64<D> T, const int32_t* __restrict__ perm, const int32_t* __restrict__ iperm, int32_t* __restrict__ nbr,
                                double* __restrict__ w, double* __restrict__ nrm, double* __restrict__ d, double* __restrict__ q,
                                int32_t* __restrict__ cidx, uint8_t* __restrict__ wall) {
  constexpr int H = Dim<D>::HALF;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t N = T.N;
  if (i >= N) return;
  const int64_t n = perm[i];
#pragma unroll
  for (int sl = 0; sl < 2 * D * H; ++sl) {
    const int32_t nb = T.nbr[(int64_t)sl * N + n];
    nbr[(int64_t)sl * N + i] = nb >= 0 ? iperm[nb] : -1;
    w[(int64_t)sl * N + i] = T.w[(int64_t)sl * N + n];
  }
#pragma unroll
  for (int dir = 0; dir < 2 * D; ++dir) {
    nrm[(int64_t)dir * N + i] = T.nrm[(int64_t)dir * N + n];
    d[(int64_t)dir * N + i] = T.d[(int64_t)dir * N + n];
  }
#pragma unroll
  for (int j = 0; j < 2 * D * (D - 1); ++j) q[(int64_t)j * N + i] = T.q[(int64_t)j * N + n];
  cidx[i] = T.cidx[n];
  wall[i] = T.wall[n];
}
__global__ void k_gather_perm64(const double* __restrict__ src, const int32_t* __restrict__ perm, double* __restrict__ dst, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = src[perm[i]];
}
__global__ void k_scatter_perm64(const double* __restrict__ src, const int32_t* __restrict__ perm, double* __restrict__ dst, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[perm[i]] = src[i];
}
}  // namespace

size_t sort64_temp_bytes(int64_t n) {
  size_t bytes = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, bytes, (const uint32_t*)nullptr, (uint32_t*)nullptr, (const int32_t*)nullptr, (int32_t*)nullptr,
                                  (int)n, 0, 19);
  return bytes;
}

template <int D>
cudaError_t launch_sort_tab64(const DTab64<D>& T, uint32_t* keys, uint32_t* keys_out, int32_t* idx, void* temp, size_t temp_bytes,
                              int32_t* perm, int32_t* iperm, const Tab64Out& out, cudaStream_t s) {
  const int64_t N = T.N;
  if (N == 0) return cudaSuccess;
  k_pattern_key64<D><<<nblocks(N), TPB, 0, s>>>(T, keys, idx);
  const cudaError_t e = cub::DeviceRadixSort::SortPairs(temp, temp_bytes, keys, keys_out, idx, perm, (int)N, 0, 19, s);
  if (e != cudaSuccess) return e;
  k_inverse_perm<<<nblocks(N), TPB, 0, s>>>(perm, iperm, N);
  k_permute_tab64<D><<<nblocks(N), TPB, 0, s>>>(T, perm, iperm, out.nbr, out.w, out.nrm, out.d, out.q, out.cidx, out.wall);
  return cudaGetLastError();
}

template <int D>
void launch_node_word64(const DTab64<D>& T, uint32_t* word, cudaStream_t s) {
  if (T.N) k_node_word64<D><<<nblocks(T.N), TPB, 0, s>>>(T, word);
}

void launch_gather_perm64(const double* src, const int32_t* perm, double* dst, int64_t n, cudaStream_t s) {
  if (n) k_gather_perm64<<<nblocks(n), TPB, 0, s>>>(src, perm, dst, n);
}
void launch_scatter_perm64(const double* src, const int32_t* perm, double* dst, int64_t n, cudaStream_t s) {
  if (n) k_scatter_perm64<<<nblocks(n), TPB, 0, s>>>(src, perm, dst, n);
}

#define LSG_INST(D)                                                                                                          \
  template void launch_node_word64<D>(const DTab64<D>&, uint32_t*, cudaStream_t);                                             \
  template cudaError_t launch_sort_tab64<D>(const DTab64<D>&, uint32_t*, uint32_t*, int32_t*, void*, size_t, int32_t*, int32_t*, \
                                            const Tab64Out&, cudaStream_t);                                                  \
  template void launch_dd64<D>(const DTab64<D>&, const double*, double*, cudaStream_t, int64_t, int64_t);                    \
  template void launch_iface_err64<D>(const DTab64<D>&, const double*, const double*, unsigned long long*, cudaStream_t);     \
  template void launch_reinit_prep64<D>(const DTab64<D>&, const double*, const double*, double, double, double, int, uint16_t*, \
                                        double*, cudaStream_t, int64_t, int64_t);                                            \
  template void launch_reinit_stage64<D>(const DTab64<D>&, int, const uint16_t*, const double*, const double*, const double*, \
                                         const double*, double*, const double*, cudaStream_t, int64_t, int64_t);             \
  template void launch_advect_stage64<D>(const DTab64<D>&, const double*, const double*, const double*, const double*, double,  \
                                         double*, const double*, cudaStream_t, int64_t, int64_t);                                              \
  template void launch_grad64<D>(const DTab64<D>&, const DGrad&, const double*, const double*, double*, int, cudaStream_t);      \
  template void launch_efi_stage64<D>(const DTab64<D>&, const double*, const double*, const double*, const double*, const double*,  \
                                      const double*, const double*, const uint8_t*, double, bool, double*, cudaStream_t);          \
  template void launch_normalize64<D>(double*, int64_t, cudaStream_t);                                                        \
  template void launch_div64<D>(const DTab64<D>&, const DGrad&, const double*, const double*, double*, cudaStream_t);            \
  template void launch_kappa64<D>(const DTab64<D>&, const DGrad&, const double*, const double*, const double*, const double*,    \
                                  double*, cudaStream_t);                                                                     \
  template void launch_ext_init1<D>(const DTab64<D>&, const DGrad&, const double*, const double*, const double*, const double*,  \
                                    const double*, double, int, double*, double*, int8_t*, cudaStream_t);                     \
  template void launch_ext_init2<D>(const DTab64<D>&, const DGrad&, const double*, const double*, const double*, const double*,  \
                                    const double*, const double*, const double*, const double*, const int8_t*, const int32_t*, \
                                    double, int, const double*, const double*, double*, int8_t*, cudaStream_t);              \
  template void launch_ext_march<D>(const DTab64<D>&, const double*, double*, const int8_t*, const double*, const double*,     \
                                    const double*, double, cudaStream_t);                                                     \
  template void launch_ext_q<D>(const DTab64<D>&, const double*, double*, const double*, const double*, const double*,         \
                                const double*, const double*, int, double, cudaStream_t);
LSG_INST(2)
LSG_INST(3)
#undef LSG_INST

}  // namespace lsg
