// Mixed-precision level-set kernels: the stencil, Godunov Hamiltonian and RK stages in FP32 with
// FP32 accumulation; the subcell interface distances (quadratic root through the sign change of
// phi_0) in FP64, computed once per call because they depend on phi_0 only.
//
// Work runs in the device node order of the mixed tables (tables32.cpp): regular nodes first, then
// irregular nodes grouped by stencil pattern. One thread per node; a warp is (up to one boundary
// warp) entirely regular or entirely irregular, and irregular warps mostly share one pattern.
// The arithmetic restates the same reference routines as the FP64 kernels (stencil64.cuh):
// laplace/correct_naive_second_derivatives, ngbd_with_quadratic_interpolation,
// reinitialize_one_iteration and advect_in_normal_direction_one_iteration, with geometric divisions
// folded into FP32 coefficients.
#include <algorithm>

#include "kernels.h"
#include "stencil64.cuh"
#include "tables.hpp"

namespace lsg {

namespace {

constexpr int TPB = 256;

__device__ __forceinline__ int tan_axis32(int axis, int j) { return j == 0 ? (axis == 0 ? 1 : 0) : (axis == 2 ? 1 : 2); }
__device__ __forceinline__ int face_count(uint32_t meta, int dir) { return (int)((meta >> (2 * dir)) & 3u) + 1; }

// Cell size tree_size * 2^-(base + code), by exponent arithmetic (sizes are normal floats).
__device__ __forceinline__ float level_size(float tsize, int base, uint32_t code) {
  return __int_as_float(__float_as_int(tsize) - ((base + (int)code) << 23));
}
// its reciprocal, exact: the reciprocal tree size with the exponent raised by the level
__device__ __forceinline__ float level_inv(float inv_tsize, int base, uint32_t code) {
  return __int_as_float(__float_as_int(inv_tsize) + ((base + (int)code) << 23));
}

template <int D>
struct Reg {  // regular-node view
  uint32_t codes;
  __device__ __forceinline__ float d(const DTab32<D>& T, int dir) const {
    return level_size(T.tsize[dir >> 1], T.base, (codes >> (4 * dir)) & 15u);
  }
};

template <int D>
__device__ __forceinline__ float lin_irr(const DTab32<D>& T, uint32_t meta, int dir, int64_t i, const float* __restrict__ f) {
  constexpr int H = Dim<D>::HALF;
  const int64_t nI = T.nI;
  const int64_t base = (int64_t)(dir * H) * nI + i;
  const int c = face_count(meta, dir);
  const int32_t i0 = __ldcs(T.i_nbr + base);
  if (c == 1) return __ldg(f + i0);
  float acc = __ldg(T.i_wf + base) * __ldg(f + i0);
#pragma unroll
  for (int k = 1; k < H; ++k)
    if (k < c) acc = fmaf(__ldg(T.i_wf + base + k * nI), __ldg(f + __ldcs(T.i_nbr + base + k * nI)), acc);
  return acc;
}

template <int D>
__device__ __forceinline__ void correct_irr(const DTab32<D>& T, uint32_t meta, int64_t i, float* Dv) {
  if (!(meta & (1u << 16))) return;
  const float* M = T.corr + (int64_t)D * D * __ldg(T.i_cidx + i);
  float o[D];
#pragma unroll
  for (int r = 0; r < D; ++r) {
    float acc = 0.0f;
#pragma unroll
    for (int c = 0; c < D; ++c) acc = fmaf(__ldg(M + D * r + c), Dv[c], acc);
    o[r] = acc;
  }
#pragma unroll
  for (int r = 0; r < D; ++r) Dv[r] = o[r];
}

// ((fp-f0)/dp + (fm-f0)/dm) * 2/(dp+dm)
__device__ __forceinline__ float central_dd(float fp, float f0, float fm, float dp, float dm) {
  return __fdividef(2.0f * fmaf(fp - f0, dm, (fm - f0) * dp), dp * dm * (dp + dm));
}

template <int D>
__global__ void __launch_bounds__(TPB) k_dd32(DTab32<D> T, const float* __restrict__ f, float* __restrict__ dd) {
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t N = T.N;
  if (n >= N) return;
  const float f0 = __ldg(f + n);
  float Dv[D];
  if (n < T.nR) {
    const Reg<D> R{__ldcs(T.r_meta + n)};
#pragma unroll
    for (int a = 0; a < D; ++a) {
      const float fm = __ldg(f + __ldcs(T.r_nbr + (int64_t)(2 * a) * T.nR + n));
      const float fp = __ldg(f + __ldcs(T.r_nbr + (int64_t)(2 * a + 1) * T.nR + n));
      Dv[a] = central_dd(fp, f0, fm, R.d(T, 2 * a + 1), R.d(T, 2 * a));
    }
  } else {
    const int64_t i = n - T.nR;
    const uint32_t meta = __ldg(T.i_meta + i);
#pragma unroll
    for (int a = 0; a < D; ++a) {
      const float fm = lin_irr<D>(T, meta, 2 * a, i, f);
      const float fp = lin_irr<D>(T, meta, 2 * a + 1, i, f);
      Dv[a] = central_dd(fp, f0, fm, __ldg(T.i_d + (int64_t)(2 * a + 1) * T.nI + i), __ldg(T.i_d + (int64_t)(2 * a) * T.nI + i));
    }
    correct_irr<D>(T, meta, i, Dv);
  }
#pragma unroll
  for (int a = 0; a < D; ++a) dd[(int64_t)a * N + n] = Dv[a];
}

// Godunov update shared by both groups (reinitialize_one_iteration after the neighbour values).
template <int D, int ORDER_SPACE>
__device__ __forceinline__ float reinit_update(float f0, const float* fnb, const float* s, const float* is, const float* xx0,
                                             const float* xxnb, bool pos) {
  const float sgn = pos ? 1.0f : -1.0f;
  float dt = fminf(s[0], s[1]);
#pragma unroll
  for (int dir = 2; dir < 2 * D; ++dir) dt = fminf(dt, s[dir]);
  dt *= (1.0f / D);
  float h = 0.0f;
#pragma unroll
  for (int a = 0; a < D; ++a) {
    float gp = (fnb[2 * a + 1] - f0) * is[2 * a + 1];
    float gm = (f0 - fnb[2 * a]) * is[2 * a];
    if (ORDER_SPACE > 1) {
      gm = fmaf(0.5f * s[2 * a], minmodf(xxnb[2 * a], xx0[a]), gm);
      gp = fmaf(-0.5f * s[2 * a + 1], minmodf(xxnb[2 * a + 1], xx0[a]), gp);
    }
    if (sgn * gp > 0.0f) gp = 0.0f;
    if (sgn * gm < 0.0f) gm = 0.0f;
    h += fmaxf(gp * gp, gm * gm);
  }
  float r = f0 - dt * sgn * (sqrtf(h) - 1.0f);
  if (pos ? (r < 0.0f) : (r > 0.0f)) r = -r;
  return r;
}

// advect_in_normal_direction_one_iteration's update after the neighbour values (src/my_p4est_level_set.cpp:559-654):
// one-sided slopes with the minmod terms, upwinding by the sign of vn, phi - dt vn sqrt(sum gp^2 + gm^2)
template <int D>
__device__ __forceinline__ float advect_update(float f0, const float* fnb, const float* s, const float* is, const float* xx0,
                                               const float* xxnb, float v, float dt) {
  const float sgn = v > 0.0f ? 1.0f : -1.0f;
  float h = 0.0f;
#pragma unroll
  for (int a = 0; a < D; ++a) {
    float gp = (fnb[2 * a + 1] - f0) * is[2 * a + 1];
    float gm = (f0 - fnb[2 * a]) * is[2 * a];
    gm = fmaf(0.5f * s[2 * a], minmodf(xxnb[2 * a], xx0[a]), gm);
    gp = fmaf(-0.5f * s[2 * a + 1], minmodf(xxnb[2 * a + 1], xx0[a]), gp);
    if (sgn * gp > 0.0f) gp = 0.0f;
    if (sgn * gm < 0.0f) gm = 0.0f;
    h += gp * gp + gm * gm;
  }
  return f0 - dt * v * sqrtf(h);
}

// ---- fused reinitialisation stage ----------------------------------------------------------------
// One stage of reinitialize_one_iteration per node without a separate second-derivative sweep: the
// second derivatives of the face nodes along their axis are recomputed from phi here (regular face
// nodes: central difference of two gathered values), or read from dd_irr for irregular face nodes
// (written by k_dd_x32 just before on the extended set).
// class record accessors (layout in tables.hpp)
template <int D>
struct Cls {
  const float* c;
  __device__ __forceinline__ uint32_t meta() const { return __float_as_uint(__ldg(c)); }
  __device__ __forceinline__ float d(int dir) const { return __ldg(c + 1 + dir); }
  __device__ __forceinline__ float wf(int dir, int k) const { return __ldg(c + 1 + 2 * D + dir * Dim<D>::HALF + k); }
  __device__ __forceinline__ float q(int dir, int j) const { return __ldg(c + 1 + 2 * D + 2 * D * Dim<D>::HALF + dir * (D - 1) + j); }
  __device__ __forceinline__ float corr(int r, int col) const {
    return __ldg(c + 1 + 2 * D + 2 * D * Dim<D>::HALF + 2 * D * (D - 1) + r * D + col);
  }
};

template <int D>
__device__ __forceinline__ Cls<D> cls_of(const DTab32<D>& T, int64_t i) {
  return Cls<D>{T.cls32 + (int64_t)__ldcs(T.i_cls + i) * cls_words<D>()};
}

// linear interpolation over the face nodes of an irregular node (class weights)
template <int D>
__device__ __forceinline__ float lin_cls(const DTab32<D>& T, const Cls<D>& C, uint32_t meta, int dir, int64_t i, const float* __restrict__ f) {
  constexpr int H = Dim<D>::HALF;
  const int64_t base = (int64_t)(dir * H) * T.nI + i;
  const int c = face_count(meta, dir);
  if (c == 1) return __ldg(f + __ldcs(T.i_nbr + base));
  float acc = 0.0f;
#pragma unroll
  for (int k = 0; k < H; ++k)
    if (k < c) acc = fmaf(C.wf(dir, k), __ldg(f + __ldcs(T.i_nbr + base + k * T.nI)), acc);
  return acc;
}

// the same with the first face node of the direction already loaded (j0); the remaining ones are read
// only when the face holds more than one node
template <int D>
__device__ __forceinline__ float lin_cls_h(const DTab32<D>& T, const Cls<D>& C, uint32_t meta, int dir, int64_t i, int32_t j0,
                                           const float* __restrict__ f) {
  constexpr int H = Dim<D>::HALF;
  const int c = face_count(meta, dir);
  if (c == 1) return __ldg(f + j0);
  const int64_t base = (int64_t)(dir * H) * T.nI + i;
  float acc = fmaf(C.wf(dir, 0), __ldg(f + j0), 0.0f);
#pragma unroll
  for (int k = 1; k < H; ++k)
    if (k < c) acc = fmaf(C.wf(dir, k), __ldg(f + __ldcs(T.i_nbr + base + k * T.nI)), acc);
  return acc;
}

// second derivatives on the extended set: irregular nodes (laplace with the class coefficients and
// the correction matrix) and the listed regular nodes (central differences). An irregular node issues
// its class id, the first face node of every direction and its own value together, so the class record
// and the gathers wait for one round trip instead of three.
template <int D>
__global__ void __launch_bounds__(TPB) k_dd_x32(DTab32<D> T, const float* __restrict__ f, float* __restrict__ ddx) {
  constexpr int H = Dim<D>::HALF;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t N = T.N;
  float Dv[D];
  int64_t n;
  if (t < T.nI) {
    const int64_t i = t;
    n = T.nR + i;
    const uint32_t ci = __ldcs(T.i_cls + i);
    int32_t j0[2 * D];
#pragma unroll
    for (int dir = 0; dir < 2 * D; ++dir) j0[dir] = __ldcs(T.i_nbr + (int64_t)(dir * H) * T.nI + i);
    const float f0 = __ldg(f + n);
    const Cls<D> C{T.cls32 + (int64_t)ci * cls_words<D>()};
    const uint32_t meta = C.meta();
#pragma unroll
    for (int a = 0; a < D; ++a)
      Dv[a] = central_dd(lin_cls_h<D>(T, C, meta, 2 * a + 1, i, j0[2 * a + 1], f), f0, lin_cls_h<D>(T, C, meta, 2 * a, i, j0[2 * a], f),
                         C.d(2 * a + 1), C.d(2 * a));
    if (meta & (1u << 16)) {
      float o[D];
#pragma unroll
      for (int r = 0; r < D; ++r) {
        float acc = 0.0f;
#pragma unroll
        for (int c = 0; c < D; ++c) acc = fmaf(C.corr(r, c), Dv[c], acc);
        o[r] = acc;
      }
#pragma unroll
      for (int r = 0; r < D; ++r) Dv[r] = o[r];
    }
  } else if (t < T.nI + T.nX) {
    n = T.x_first + (t - T.nI);
    const Reg<D> R{__ldcs(T.r_meta + n)};
    const float f0 = __ldg(f + n);
#pragma unroll
    for (int a = 0; a < D; ++a) {
      const float fm = __ldg(f + __ldcs(T.r_nbr + (int64_t)(2 * a) * T.nR + n));
      const float fp = __ldg(f + __ldcs(T.r_nbr + (int64_t)(2 * a + 1) * T.nR + n));
      Dv[a] = central_dd(fp, f0, fm, R.d(T, 2 * a + 1), R.d(T, 2 * a));
    }
  } else {
    return;
  }
#pragma unroll
  for (int a = 0; a < D; ++a) ddx[(int64_t)a * N + n] = Dv[a];
}

// Irregular nodes [first, last) (first = nR). The loads that depend on nothing but the node (status,
// class id, the first face node of every direction, its value and second derivatives) are issued together,
// so the class record and the gathers wait for one round trip instead of three.
template <int D, int ORDER_SPACE, bool AVG, bool ADV>
__global__ void __launch_bounds__(TPB) k_reinit_fused32(DTab32<D> T, const uint16_t* __restrict__ status,
                                                        const float* __restrict__ s_near, const float* __restrict__ phin,
                                                        const float* __restrict__ dd_irr, float* out, const float* avg_with,
                                                        int64_t first, int64_t last, const float* __restrict__ vn, float adv_dt) {
  constexpr int H = Dim<D>::HALF;
  const int64_t n = first + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t N = T.N;
  if (n >= last) return;
  const int64_t i = n - T.nR;
  const uint16_t st = ADV ? (uint16_t)0 : __ldcs(status + n);
  const float v = ADV ? __ldcs(vn + n) : 0.0f;
  const uint32_t ci = __ldcs(T.i_cls + i);
  int32_t j0[2 * D];
#pragma unroll
  for (int dir = 0; dir < 2 * D; ++dir) j0[dir] = __ldcs(T.i_nbr + (int64_t)(dir * H) * T.nI + i);
  const float f0 = __ldg(phin + n);
  float Dv[D];
#pragma unroll
  for (int a = 0; a < D; ++a) Dv[a] = __ldg(dd_irr + (int64_t)a * N + n);
  float r;
  if (st & ST_ANCHORED) {
    r = 0.0f;
  } else if (st & (ST_OUTSIDE | ST_FROZEN)) {
    r = f0;
  } else {
    float fnb[2 * D], s[2 * D], xxnb[2 * D];
    const Cls<D> C{T.cls32 + (int64_t)ci * cls_words<D>()};
    const uint32_t meta = C.meta();
    const uint32_t wl = meta >> 24;
#pragma unroll
    for (int dir = 0; dir < 2 * D; ++dir) {
      const int axis = dir >> 1;
      const int c = face_count(meta, dir);
      const int64_t base = (int64_t)(dir * H) * T.nI + i;
      s[dir] = C.d(dir);
      if (c == 1) {
        fnb[dir] = __ldg(phin + j0[dir]);
        if (ORDER_SPACE > 1) xxnb[dir] = __ldg(dd_irr + (int64_t)axis * N + j0[dir]);
      } else {
        float v = 0.0f, x = 0.0f;
#pragma unroll
        for (int k = 0; k < H; ++k) {
          if (k < c) {
            const int32_t j = k == 0 ? j0[dir] : __ldcs(T.i_nbr + base + k * T.nI);
            const float w = C.wf(dir, k);
            v = fmaf(w, __ldg(phin + j), v);
            if (ORDER_SPACE > 1) x = fmaf(w, __ldg(dd_irr + (int64_t)axis * N + j), x);
          }
        }
#pragma unroll
        for (int jj = 0; jj < D - 1; ++jj) v = fmaf(-C.q(dir, jj), Dv[tan_axis32(axis, jj)], v);
        fnb[dir] = v;
        xxnb[dir] = x;
      }
    }
#pragma unroll
    for (int a = 0; a < D; ++a) {
      if (wl & (1u << (2 * a))) {
        s[2 * a] = s[2 * a + 1];
        fnb[2 * a] = fnb[2 * a + 1];
        Dv[a] = xxnb[2 * a] = xxnb[2 * a + 1] = 0.0f;
      }
      if (wl & (1u << (2 * a + 1))) {
        s[2 * a + 1] = s[2 * a];
        fnb[2 * a + 1] = fnb[2 * a];
        Dv[a] = xxnb[2 * a] = xxnb[2 * a + 1] = 0.0f;
      }
    }
    if (!ADV && (st & ST_NEAR)) {
#pragma unroll
      for (int dir = 0; dir < 2 * D; ++dir) {
        s[dir] = __ldg(s_near + (int64_t)dir * N + n);
        if (st & (1u << (ST_CUT_SHIFT + dir))) fnb[dir] = 0.0f;
      }
#pragma unroll
      for (int a = 0; a < D; ++a) {
        if (wl & (1u << (2 * a))) {
          s[2 * a] = s[2 * a + 1];
          fnb[2 * a] = fnb[2 * a + 1];
        }
        if (wl & (1u << (2 * a + 1))) {
          s[2 * a + 1] = s[2 * a];
          fnb[2 * a + 1] = fnb[2 * a];
        }
      }
    }
    float is[2 * D];
#pragma unroll
    for (int dir = 0; dir < 2 * D; ++dir) is[dir] = __fdividef(1.0f, s[dir]);
    r = ADV ? advect_update<D>(f0, fnb, s, is, Dv, xxnb, v, adv_dt)
              : reinit_update<D, ORDER_SPACE>(f0, fnb, s, is, Dv, xxnb, (st & ST_POSITIVE) != 0);
  }
  if (AVG) r = 0.5f * (avg_with[n] + r);
  out[n] = r;
}

// Regular nodes, persistent and software-pipelined: while a node's gathers are in flight the
// thread already loads the next node's status, level codes, face-node and second-neighbour indices
// and value. A face node's second derivative along its axis is a central difference of
// (second neighbour, face node, this node) when the second neighbour is recorded; otherwise it is
// read from the extended second-derivative set (k_dd_x32).
template <int D, int ORDER_SPACE, bool AVG, bool ADV>
__global__ void __launch_bounds__(TPB) k_reinit_fused_reg32(DTab32<D> T, const uint16_t* __restrict__ status,
                                                            const float* __restrict__ s_near, const float* __restrict__ phin,
                                                            const float* __restrict__ dd_irr, float* out, const float* avg_with,
                                                            int first, int last, const float* __restrict__ vn, float adv_dt) {
  const int nR = (int)T.nR;
  const int stride = gridDim.x * blockDim.x;
  int n = first + blockIdx.x * blockDim.x + threadIdx.x;
  uint16_t p_st = 0;
  uint32_t p_codes = 0, p_far = 0;
  int32_t p_nb[2 * D], p_nb2[2 * D];
  float p_f0 = 0.0f, p_avg = 0.0f, p_vn = 0.0f;
  auto prefetch = [&](int m) {
    p_st = ADV ? (uint16_t)0 : __ldcs(status + m);
    if (ADV) p_vn = __ldcs(vn + m);
    p_codes = __ldcs(T.r_meta + m);
    p_far = __ldcs(T.r_meta2 + m);
    // the 4D stencil indices with D vector loads from the node-major copy
    int32_t w[4 * D];
#pragma unroll
    for (int k = 0; k < D; ++k) {
      const int4 q = __ldcs(T.u_pack + (int64_t)D * m + k);
      w[4 * k] = q.x;
      w[4 * k + 1] = q.y;
      w[4 * k + 2] = q.z;
      w[4 * k + 3] = q.w;
    }
#pragma unroll
    for (int dir = 0; dir < 2 * D; ++dir) {
      p_nb[dir] = w[dir];
      p_nb2[dir] = w[2 * D + dir];
    }
    p_f0 = __ldg(phin + m);
    if (AVG) p_avg = __ldcs(avg_with + m);
  };
  if (n < last) prefetch(n);
  for (; n < last; n += stride) {
    const uint16_t st = p_st;
    const uint32_t codes = p_codes, far = p_far;
    int32_t nb[2 * D], nb2[2 * D];
#pragma unroll
    for (int dir = 0; dir < 2 * D; ++dir) {
      nb[dir] = p_nb[dir];
      nb2[dir] = p_nb2[dir];
    }
    const float f0 = p_f0, avg = p_avg, v = p_vn;
    if (n + stride < last) prefetch(n + stride);
    float r;
    if (st & ST_ANCHORED) {
      r = 0.0f;
    } else if (st & (ST_OUTSIDE | ST_FROZEN)) {
      r = f0;
    } else {
      // one round of gathers: every face value and, per direction, the second neighbour's value or
      // (when the face node has none recorded) the face node's second derivative along the axis
      float Dv[D], fnb[2 * D], s[2 * D], is[2 * D], xxnb[2 * D], fx[2 * D];
#pragma unroll
      for (int dir = 0; dir < 2 * D; ++dir) {
        fnb[dir] = __ldg(phin + nb[dir]);
        if (ORDER_SPACE > 1) fx[dir] = __ldg(nb2[dir] >= 0 ? phin + nb2[dir] : dd_irr + (int64_t)(dir >> 1) * T.N + nb[dir]);
        s[dir] = level_size(T.tsize[dir >> 1], T.base, (codes >> (4 * dir)) & 15u);
        is[dir] = level_inv(T.inv_tsize[dir >> 1], T.base, (codes >> (4 * dir)) & 15u);
      }
#pragma unroll
      for (int a = 0; a < D; ++a) Dv[a] = central_dd(fnb[2 * a + 1], f0, fnb[2 * a], s[2 * a + 1], s[2 * a]);
      if (ORDER_SPACE > 1) {
#pragma unroll
        for (int dir = 0; dir < 2 * D; ++dir) {
          if (nb2[dir] >= 0) {
            const float dfar = level_size(T.tsize[dir >> 1], T.base, (far >> (4 * dir)) & 15u);
            // outer side of the face node: second neighbour; inner side: this node
            xxnb[dir] = (dir & 1) ? central_dd(fx[dir], fnb[dir], f0, dfar, s[dir]) : central_dd(f0, fnb[dir], fx[dir], s[dir], dfar);
          } else {
            xxnb[dir] = fx[dir];
          }
        }
      }
      if (!ADV && (st & ST_NEAR)) {
#pragma unroll
        for (int dir = 0; dir < 2 * D; ++dir) {
          s[dir] = __ldg(s_near + (int64_t)dir * T.N + n);
          is[dir] = __fdividef(1.0f, s[dir]);
          if (st & (1u << (ST_CUT_SHIFT + dir))) fnb[dir] = 0.0f;
        }
      }
      r = ADV ? advect_update<D>(f0, fnb, s, is, Dv, xxnb, v, adv_dt)
              : reinit_update<D, ORDER_SPACE>(f0, fnb, s, is, Dv, xxnb, (st & ST_POSITIVE) != 0);
    }
    if (AVG) r = 0.5f * (avg + r);
    out[n] = r;
  }
}

// Regular nodes with uniform stencils (second order in space): the node and its face nodes have the
// same spacing h_a along each axis, so every second derivative is (f_+ + f_- - 2 f_0)/h_a^2 and all
// reciprocals are exponent shifts. Persistent and software-pipelined: with DEPTH 1 a thread loads the
// next node's indices while the current node's face values are gathered; with DEPTH 2 it also gathers
// the next node's face values while the current node is computed (two nodes' gathers in flight).
// Interface-adjacent nodes take their subcell distances from s_near.
template <int D>
struct UniIdx {  // a node's own words and stencil indices
  int n;
  uint16_t st;
  uint32_t code;
  float f0, avg, vn;
  int32_t nb[2 * D], nb2[2 * D];
};
template <int D>
struct UniVal {  // the same node with its face and second-neighbour values gathered
  int n;
  uint16_t st;
  uint32_t code;
  float f0, avg, vn;
  float v[2 * D], v2[2 * D];
};

// ADV: the normal-advection stage (every node updated, upwinding by vn) instead of the reinitialisation stage
template <int D, bool AVG, bool ADV>
__device__ __forceinline__ void uni_load(const DTab32<D>& T, int nR, const uint16_t* __restrict__ status, const float* __restrict__ phin,
                                         const float* avg_with, const float* __restrict__ vn, int m, UniIdx<D>& I) {
  I.n = m;
  I.st = ADV ? (uint16_t)0 : __ldcs(status + m);
  I.vn = ADV ? __ldcs(vn + m) : 0.0f;
  I.code = __ldcs(T.r_meta + m) & 15u;
  // the 4D stencil indices with D vector loads from the node-major copy
  int32_t w[4 * D];
#pragma unroll
  for (int k = 0; k < D; ++k) {
    const int4 q = __ldcs(T.u_pack + (int64_t)D * m + k);
    w[4 * k] = q.x;
    w[4 * k + 1] = q.y;
    w[4 * k + 2] = q.z;
    w[4 * k + 3] = q.w;
  }
#pragma unroll
  for (int dir = 0; dir < 2 * D; ++dir) {
    I.nb[dir] = w[dir];
    I.nb2[dir] = w[2 * D + dir];
  }
  I.f0 = __ldg(phin + m);
  I.avg = AVG ? __ldcs(avg_with + m) : 0.0f;
}

template <int D>
__device__ __forceinline__ void uni_gather(const UniIdx<D>& I, const float* __restrict__ phin, UniVal<D>& V) {
  V.n = I.n;
  V.st = I.st;
  V.code = I.code;
  V.f0 = I.f0;
  V.avg = I.avg;
  V.vn = I.vn;
  const bool active = !(I.st & (ST_ANCHORED | ST_OUTSIDE | ST_FROZEN));
#pragma unroll
  for (int dir = 0; dir < 2 * D; ++dir) {
    V.v[dir] = active ? __ldg(phin + I.nb[dir]) : 0.0f;
    V.v2[dir] = active ? __ldg(phin + I.nb2[dir]) : 0.0f;
  }
}

template <int D, bool AVG, bool ADV>
__device__ __forceinline__ float uni_update(const DTab32<D>& T, const float* __restrict__ s_near, const UniVal<D>& V, float adv_dt) {
  const uint16_t st = V.st;
  const float f0 = V.f0;
  float r;
  if (st & ST_ANCHORED) {
    r = 0.0f;
  } else if (st & (ST_OUTSIDE | ST_FROZEN)) {
    r = f0;
  } else {
    const int lvl = T.base + (int)V.code;
    const bool near = !ADV && (st & ST_NEAR) != 0;
    const float sgn = ADV ? (V.vn > 0.0f ? 1.0f : -1.0f) : ((st & ST_POSITIVE) ? 1.0f : -1.0f);
    float smin = 3.0e38f, hsum = 0.0f;
#pragma unroll
    for (int a = 0; a < D; ++a) {
      const float h = __int_as_float(__float_as_int(T.tsize[a]) - (lvl << 23));
      const float ih = __int_as_float(__float_as_int(T.inv_tsize[a]) + (lvl << 23));
      const float ih2 = ih * ih;
      float fm = V.v[2 * a], fp = V.v[2 * a + 1];
      const float fmm = V.v2[2 * a], fpp = V.v2[2 * a + 1];
      const float xx0 = (fp + fm - 2.0f * f0) * ih2;
      const float mm = minmodf((f0 + fmm - 2.0f * fm) * ih2, xx0);
      const float mp = minmodf((fpp + f0 - 2.0f * fp) * ih2, xx0);
      // one expression for both cases: away from the interface the distances are h and their reciprocal ih;
      // an interface-adjacent node takes its subcell distances and the reciprocals of those, and a cut
      // direction's neighbour value is the interface's zero
      float sm = h, sp = h, im = ih, ip = ih;
      if (near) {
        sm = __ldg(s_near + (int64_t)(2 * a) * T.N + V.n);
        sp = __ldg(s_near + (int64_t)(2 * a + 1) * T.N + V.n);
        im = __fdividef(1.0f, sm);
        ip = __fdividef(1.0f, sp);
        if (st & (1u << (ST_CUT_SHIFT + 2 * a))) fm = 0.0f;
        if (st & (1u << (ST_CUT_SHIFT + 2 * a + 1))) fp = 0.0f;
      }
      float gm = fmaf(0.5f * sm, mm, (f0 - fm) * im);
      float gp = fmaf(-0.5f * sp, mp, (fp - f0) * ip);
      smin = fminf(smin, fminf(sm, sp));
      if (sgn * gp > 0.0f) gp = 0.0f;
      if (sgn * gm < 0.0f) gm = 0.0f;
      hsum += ADV ? gp * gp + gm * gm : fmaxf(gp * gp, gm * gm);
    }
    if (ADV) {
      r = f0 - adv_dt * V.vn * sqrtf(hsum);
    } else {
      r = f0 - smin * (1.0f / D) * sgn * (sqrtf(hsum) - 1.0f);
      if ((st & ST_POSITIVE) ? (r < 0.0f) : (r > 0.0f)) r = -r;
    }
  }
  if (AVG) r = 0.5f * (V.avg + r);
  return r;
}

// MINB > 1 caps the registers so that MINB blocks of TPB threads fit on an SM (6: 40 registers, a few of the
// node's words spill to L1): more of the uniform kernel's warps stay resident beside the side stream's kernels.
template <int D, bool AVG, int DEPTH, bool ADV, int MINB = 1>
__global__ void __launch_bounds__(TPB, MINB) k_reinit_uniform32(DTab32<D> T, const uint16_t* __restrict__ status,
                                                          const float* __restrict__ s_near, const float* __restrict__ phin,
                                                          float* out, const float* avg_with, const float* __restrict__ vn, float adv_dt) {
  const int nR = (int)T.nR, nU = (int)T.nU;
  const int stride = gridDim.x * blockDim.x;
  int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nU) return;
  UniIdx<D> I;
  uni_load<D, AVG, ADV>(T, nR, status, phin, avg_with, vn, n, I);
  if (DEPTH == 1) {
    for (; n < nU; n += stride) {
      UniVal<D> V;
      uni_gather<D>(I, phin, V);
      if (n + stride < nU) uni_load<D, AVG, ADV>(T, nR, status, phin, avg_with, vn, n + stride, I);
      out[V.n] = uni_update<D, AVG, ADV>(T, s_near, V, adv_dt);
    }
  } else {
    UniVal<D> V;
    uni_gather<D>(I, phin, V);
    if (n + stride < nU) uni_load<D, AVG, ADV>(T, nR, status, phin, avg_with, vn, n + stride, I);
    for (; n < nU; n += stride) {
      // gathers of the next node and index loads of the one after are issued before this node's update
      UniVal<D> Vn;
      const bool more = n + stride < nU;
      if (more) uni_gather<D>(I, phin, Vn);
      if (n + 2 * stride < nU) uni_load<D, AVG, ADV>(T, nR, status, phin, avg_with, vn, n + 2 * stride, I);
      out[V.n] = uni_update<D, AVG, ADV>(T, s_near, V, adv_dt);
      if (more) V = Vn;
    }
  }
}

// ---- uniform kernel with bulk-copied stencil words and a staged window of phi ---------------------
// The same update, with everything a tile of nodes reads moved into shared memory by bulk asynchronous
// copies (cp.async.bulk, completion counted on an mbarrier) STAGES tiles ahead of the tile being
// computed: the words each node streams from HBM (status, level code, the 4D face and second-neighbour
// indices, the RK partner) and the window phi[m0 - halo, m0 + tile + halo) of the Morton-contiguous
// tile [m0, m0 + tile). In Morton order most face and second neighbours of a tile's nodes lie in that
// window (about 79% of the references with halo 512 on the 3D flower grids), so those values come from
// shared memory; the rest are gathered from global memory. The node's own value is read from the
// window too.
//
// A CTA owns tiles blockIdx.x, blockIdx.x + gridDim.x, ... of blockDim.x nodes. Copies start on
// 16-byte boundaries: a table segment starting at element e0 is copied from e0 rounded down to 16
// bytes and read at the remainder; the window starts at a multiple of 4 elements and ends at most at
// N rounded down to a multiple of 4. A tile is copied only when its node range ends at least 8 nodes
// before the uniform group does, so every copied byte lies inside its array (a plane of the index
// tables holds nR >= nU entries, phi holds N >= nU); the last tiles load directly from global memory.
// Every wait on an mbarrier is bounded (wait_cycles SM clock cycles, about a second by default) and
// suspends the thread between polls (try_wait) instead of spinning; the CTA then decides together
// (__syncthreads_or, so no thread is left at a barrier the others skip) whether any thread gave up,
// and if so sets *err, lets the copies it issued land (bounded by the full limit) and stops.
__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile(
      "{\n\t.reg .b64 st;\n\t"
      "mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(smem_addr(bar)),
      "r"(bytes)
      : "memory");
}
// potentially blocking test of the phase: the thread may be suspended until the phase completes or a
// hardware time limit passes, so a waiting warp takes no issue slots from the warps doing work
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return done != 0;
}
// non-blocking test of the phase
__device__ __forceinline__ bool mbar_test_wait(uint64_t* bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return done != 0;
}
// false once `limit` SM cycles have passed without the phase completing: a non-blocking test first, then
// suspending polls, the clock checked before each of them
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, long long limit) {
  const long long t0 = clock64();
  if (mbar_test_wait(bar, parity)) return true;
  for (;;) {
    if (clock64() - t0 > limit) return false;
    if (mbar_try_wait(bar, parity)) return true;
  }
}
constexpr long long kFullWaitCycles = 1ll << 31;  // about a second at the SM clock
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_addr(dst)), "l"(src),
               "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}

// table segments of a tile: status (u16), level code word, 2D face-index planes, 2D second-neighbour
// planes, and the RK partner when averaging; then the phi window
template <int D, bool AVG>
struct UniBulk {
  static constexpr int NSEG = 2 + 4 * D + (AVG ? 1 : 0);
  // bytes of one segment's slot in a stage (tile + 8 elements, 16-byte multiple)
  static __host__ __device__ uint32_t slot_bytes(int tile, int es) { return (uint32_t)(((tile + 8) * es + 15) & ~15); }
  static __host__ __device__ uint32_t table_bytes(int tile) { return slot_bytes(tile, 2) + (NSEG - 1) * slot_bytes(tile, 4); }
  // the window holds at most tile + 2 halo + 4 values (halo a multiple of 4)
  static __host__ __device__ uint32_t window_bytes(int tile, int halo) { return (uint32_t)((tile + 2 * halo + 8) * 4); }
  static __host__ __device__ uint32_t stage_bytes(int tile, int halo) { return table_bytes(tile) + window_bytes(tile, halo); }
  // global array, element size and first element of segment g for the tile starting at node m0
  static __device__ __forceinline__ const char* seg(const DTab32<D>& T, const uint16_t* status, const float* avg_with, int g, int64_t m0,
                                                     int& es, int64_t& e0) {
    const int64_t nR = T.nR;
    es = g == 0 ? 2 : 4;
    if (g == 0) {
      e0 = m0;
      return (const char*)status;
    }
    if (g == 1) {
      e0 = m0;
      return (const char*)T.r_meta;
    }
    if (g < 2 + 2 * D) {
      e0 = (int64_t)(g - 2) * nR + m0;
      return (const char*)T.r_nbr;
    }
    if (g < 2 + 4 * D) {
      e0 = (int64_t)(g - 2 - 2 * D) * nR + m0;
      return (const char*)T.r_nbr2;
    }
    e0 = m0;
    return (const char*)avg_with;
  }
  static __device__ __forceinline__ uint32_t slot_offset(int tile, int g) { return g == 0 ? 0 : slot_bytes(tile, 2) + (g - 1) * slot_bytes(tile, 4); }
  // window [w0, w0 + len) of the tile at m0: w0 = max(m0 - halo, 0) rounded down to a multiple of 4;
  // the end m0 + tile + halo, at most nal (N rounded down to a multiple of 4), rounded up to a multiple of 4
  static __device__ __forceinline__ void window(int64_t m0, int tile, int halo, int64_t nal, int64_t& w0, int& len) {
    int64_t lo = m0 - halo;
    if (lo < 0) lo = 0;
    lo &= ~(int64_t)3;
    int64_t hi = m0 + tile + halo;
    if (hi > nal) hi = nal;
    w0 = lo;
    len = (int)(((hi + 3) & ~(int64_t)3) - lo);
  }
};

template <int D, bool AVG, int STAGES, int NPT>
__global__ void __launch_bounds__(TPB) k_reinit_uniform32_bulk(DTab32<D> T, const uint16_t* __restrict__ status,
                                                               const float* __restrict__ s_near, const float* __restrict__ phin,
                                                               float* out, const float* avg_with, int* err, long long wait_cycles, int halo) {
  using B = UniBulk<D, AVG>;
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) uint64_t full[STAGES];
  const int tile = NPT * blockDim.x;  // NPT nodes per thread and tile
  const int tid = threadIdx.x;
  const int64_t nU = T.nU;
  const int64_t nal = T.N & ~(int64_t)3;
  const int64_t ntiles = (nU + tile - 1) / tile;
  const uint32_t sb = B::stage_bytes(tile, halo);
  const uint32_t woff = B::table_bytes(tile);
  // tile k of this CTA is copied when it ends at least 8 nodes before the uniform group does
  auto tile_of = [&](int64_t k) { return (int64_t)blockIdx.x + k * (int64_t)gridDim.x; };
  auto bulk_ok = [&](int64_t t) { return (t + 1) * (int64_t)tile + 8 <= nU; };
  auto issue = [&](int64_t t, int s) {  // one thread: arm stage s and copy tile t into it
    const int64_t m0 = t * (int64_t)tile;
    uint32_t total = 0;
    uint32_t bytes[B::NSEG];
#pragma unroll
    for (int g = 0; g < B::NSEG; ++g) {
      int es;
      int64_t e0;
      B::seg(T, status, avg_with, g, m0, es, e0);
      const int ga = 16 / es;
      const int off = (int)(e0 & (ga - 1));
      bytes[g] = (uint32_t)(((off + tile + ga - 1) / ga) * ga * es);
      total += bytes[g];
    }
    int64_t w0;
    int wlen;
    B::window(m0, tile, halo, nal, w0, wlen);
    total += (uint32_t)wlen * 4u;
    mbar_arrive_expect_tx(&full[s], total);
#pragma unroll
    for (int g = 0; g < B::NSEG; ++g) {
      int es;
      int64_t e0;
      const char* base = B::seg(T, status, avg_with, g, m0, es, e0);
      const int ga = 16 / es;
      const int64_t a0 = e0 & ~(int64_t)(ga - 1);
      bulk_copy_g2s(smem + (size_t)s * sb + B::slot_offset(tile, g), base + a0 * es, bytes[g], &full[s]);
    }
    bulk_copy_g2s(smem + (size_t)s * sb + woff, phin + w0, (uint32_t)wlen * 4u, &full[s]);
  };
  if (tid == 0) {
    for (int s = 0; s < STAGES; ++s) mbar_init(&full[s], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (tid == 0)
    for (int s = 0; s < STAGES; ++s)
      if (tile_of(s) < ntiles && bulk_ok(tile_of(s))) issue(tile_of(s), s);
  const int nR = (int)T.nR;
  for (int64_t k = 0;; ++k) {
    const int64_t t = tile_of(k);
    if (t >= ntiles) break;
    const int s = (int)(k % STAGES);
    const int64_t m0 = t * (int64_t)tile;
    UniIdx<D> I[NPT];
    bool have[NPT];
    UniVal<D> V[NPT];
    if (bulk_ok(t)) {  // the same for every thread of the CTA
      const bool landed = mbar_wait_bounded(&full[s], (uint32_t)((k / STAGES) & 1), wait_cycles);
      if (__syncthreads_or(!landed)) {
        if (tid == 0) {
          atomicOr(err, 1);
          // let the copies this CTA issued land (bounded by the full limit) before it exits
          for (int64_t kk = k; kk < k + STAGES; ++kk)
            if (tile_of(kk) < ntiles && bulk_ok(tile_of(kk)))
              mbar_wait_bounded(&full[kk % STAGES], (uint32_t)((kk / STAGES) & 1), kFullWaitCycles);
        }
        return;
      }
      const unsigned char* st = smem + (size_t)s * sb;
      const float* win = reinterpret_cast<const float*>(st + woff);
      int64_t w0;
      int wlen;
      B::window(m0, tile, halo, nal, w0, wlen);
      const int wbase = (int)w0;
      auto word = [&](int g, int li) -> uint32_t {
        int es;
        int64_t e0;
        B::seg(T, status, avg_with, g, m0, es, e0);
        return reinterpret_cast<const uint32_t*>(st + B::slot_offset(tile, g))[(int)(e0 & 3) + li];
      };
      // a value from the window when the index falls inside it, else from global memory
      auto value = [&](int j) -> float {
        const unsigned r = (unsigned)(j - wbase);
        return r < (unsigned)wlen ? win[r] : __ldg(phin + j);
      };
#pragma unroll
      for (int j = 0; j < NPT; ++j) {
        const int li = tid + j * blockDim.x;
        const int m = (int)(m0 + li);
        V[j].n = m;
        V[j].st = reinterpret_cast<const uint16_t*>(st)[(int)(m0 & 7) + li];
        V[j].code = word(1, li) & 15u;
        V[j].f0 = win[m - wbase];
        V[j].avg = AVG ? __uint_as_float(word(2 + 4 * D, li)) : 0.0f;
        V[j].vn = 0.0f;
        const bool active = !(V[j].st & (ST_ANCHORED | ST_OUTSIDE | ST_FROZEN));
#pragma unroll
        for (int dir = 0; dir < 2 * D; ++dir) {
          V[j].v[dir] = active ? value((int32_t)word(2 + dir, li)) : 0.0f;
          V[j].v2[dir] = active ? value((int32_t)word(2 + 2 * D + dir, li)) : 0.0f;
        }
        have[j] = true;
      }
    } else {
#pragma unroll
      for (int j = 0; j < NPT; ++j) {
        const int64_t m = m0 + tid + j * blockDim.x;
        have[j] = m < nU;
        if (have[j]) uni_load<D, AVG, false>(T, nR, status, phin, avg_with, nullptr, (int)m, I[j]);
      }
#pragma unroll
      for (int j = 0; j < NPT; ++j)
        if (have[j]) uni_gather<D>(I[j], phin, V[j]);
    }
#pragma unroll
    for (int j = 0; j < NPT; ++j)
      if (have[j]) out[V[j].n] = uni_update<D, AVG, false>(T, s_near, V[j], 0.0f);
    __syncthreads();  // every thread is done with stage s
    if (tid == 0) {
      const int64_t tn = tile_of(k + STAGES);
      if (tn < ntiles && bulk_ok(tn)) {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // the reads above come before the copy's writes
        issue(tn, s);
      }
    }
  }
}

template <int D, bool AVG>
__global__ void __launch_bounds__(TPB) k_advect_stage32(DTab32<D> T, const float* __restrict__ phin, const float* __restrict__ ddq,
                                                        const float* __restrict__ ddm, const float* __restrict__ vn, float dt,
                                                        float* out, const float* avg_with) {
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t N = T.N;
  if (n >= N) return;
  const float f0 = __ldg(phin + n);
  float xx0[D], fnb[2 * D], s[2 * D], xxnb[2 * D];
#pragma unroll
  for (int a = 0; a < D; ++a) xx0[a] = __ldg(ddm + (int64_t)a * N + n);
  if (n < T.nR) {
    const Reg<D> R{__ldcs(T.r_meta + n)};
#pragma unroll
    for (int dir = 0; dir < 2 * D; ++dir) {
      const int32_t nb = __ldcs(T.r_nbr + (int64_t)dir * T.nR + n);
      fnb[dir] = __ldg(phin + nb);
      xxnb[dir] = __ldg(ddm + (int64_t)(dir >> 1) * N + nb);
      s[dir] = R.d(T, dir);
    }
  } else {
    const int64_t i = n - T.nR;
    const uint32_t meta = __ldg(T.i_meta + i);
    float Dq[D];
#pragma unroll
    for (int a = 0; a < D; ++a) Dq[a] = __ldg(ddq + (int64_t)a * N + n);
#pragma unroll
    for (int dir = 0; dir < 2 * D; ++dir) {
      float v = lin_irr<D>(T, meta, dir, i, phin);
      if (face_count(meta, dir) > 1) {
#pragma unroll
        for (int j = 0; j < D - 1; ++j) v = fmaf(-__ldg(T.i_q + (int64_t)(dir * (D - 1) + j) * T.nI + i), Dq[tan_axis32(dir >> 1, j)], v);
      }
      fnb[dir] = v;
      xxnb[dir] = lin_irr<D>(T, meta, dir, i, ddm + (int64_t)(dir >> 1) * N);
      s[dir] = __ldg(T.i_d + (int64_t)dir * T.nI + i);
    }
    const uint32_t wl = meta >> 24;
#pragma unroll
    for (int a = 0; a < D; ++a) {
      if (wl & (1u << (2 * a))) {
        s[2 * a] = s[2 * a + 1];
        fnb[2 * a] = fnb[2 * a + 1];
        xx0[a] = xxnb[2 * a] = xxnb[2 * a + 1] = 0.0f;
      }
      if (wl & (1u << (2 * a + 1))) {
        s[2 * a + 1] = s[2 * a];
        fnb[2 * a + 1] = fnb[2 * a];
        xx0[a] = xxnb[2 * a] = xxnb[2 * a + 1] = 0.0f;
      }
    }
  }
  const float v = __ldg(vn + n);
  const float sgn = v > 0.0f ? 1.0f : -1.0f;
  float h = 0.0f;
#pragma unroll
  for (int a = 0; a < D; ++a) {
    float gp = __fdividef(fnb[2 * a + 1] - f0, s[2 * a + 1]);
    float gm = __fdividef(f0 - fnb[2 * a], s[2 * a]);
    gm = fmaf(0.5f * s[2 * a], minmodf(xxnb[2 * a], xx0[a]), gm);
    gp = fmaf(-0.5f * s[2 * a + 1], minmodf(xxnb[2 * a + 1], xx0[a]), gp);
    if (sgn * gp > 0.0f) gp = 0.0f;
    if (sgn * gm < 0.0f) gm = 0.0f;
    h += gp * gp + gm * gm;
  }
  float r = f0 - dt * v * sqrtf(h);
  if (AVG) r = 0.5f * (avg_with[n] + r);
  out[n] = r;
}

// ---- FP64 subcell step (device order) ------------------------------------------------------------
// Accurate FP64 arithmetic without the reference's division order: reciprocals by Newton iteration,
// normalised weights and correction matrices precomputed in FP64.
__device__ __forceinline__ double rcp64(double x) {
  // a power of two (the product of uniform cell sizes) has an exact reciprocal: its exponent negated
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned ex = (unsigned)(b >> 52) & 0x7ffu;
  if ((b & 0x000fffffffffffffull) == 0 && ex - 1u < 2045u)
    return __longlong_as_double((long long)((b & 0x8000000000000000ull) | ((unsigned long long)(2046u - ex) << 52)));
  const double ax = fabs(x);
  if (!(ax > 1e-30 && ax < 1e30)) return 1.0 / x;
  double r = (double)__frcp_rn((float)x);
  double e = fma(-x, r, 1.0);
  r = fma(r, e, r);
  e = fma(-x, r, 1.0);
  return fma(r, e, r);
}

using st64::product_negative;

__device__ __forceinline__ double level_size64(double tsize, int base, uint32_t code) {
  return __longlong_as_double(__double_as_longlong(tsize) - ((long long)(base + (int)code) << 52));
}

__device__ __forceinline__ double central_dd64(double fp, double f0, double fm, double dp, double dm) {
  return st64::scale2(fma(fp - f0, dm, (fm - f0) * dp), 1) * rcp64(dp * dm * (dp + dm));
}

template <int D>
__device__ __forceinline__ double lin_irr64(const DTab32<D>& T, uint32_t meta, int dir, int64_t i, const double* __restrict__ f) {
  constexpr int H = Dim<D>::HALF;
  const int64_t nI = T.nI;
  const int64_t base = (int64_t)(dir * H) * nI + i;
  const int c = face_count(meta, dir);
  if (c == 1) return f[T.i_nbr[base]];
  double acc = 0.0;
#pragma unroll
  for (int k = 0; k < H; ++k)
    if (k < c) acc = fma(T.i_wf64[base + k * nI], f[T.i_nbr[base + k * nI]], acc);
  return acc;
}

// FP64 second derivatives of an irregular node (laplace + cross-term correction)
template <int D>
__device__ void laplace_irr64(const DTab32<D>& T, int64_t i, const double* __restrict__ f, double f0, double* Dv) {
  const uint32_t meta = T.i_meta[i];
#pragma unroll
  for (int a = 0; a < D; ++a) {
    const double fm = lin_irr64<D>(T, meta, 2 * a, i, f);
    const double fp = lin_irr64<D>(T, meta, 2 * a + 1, i, f);
    Dv[a] = central_dd64(fp, f0, fm, T.i_d64[(int64_t)(2 * a + 1) * T.nI + i], T.i_d64[(int64_t)(2 * a) * T.nI + i]);
  }
  if (meta & (1u << 16)) {
    const double* M = T.corr64 + (int64_t)D * D * T.i_cidx[i];
    double o[D];
#pragma unroll
    for (int r = 0; r < D; ++r) {
      double acc = 0.0;
#pragma unroll
      for (int c = 0; c < D; ++c) acc = fma(M[D * r + c], Dv[c], acc);
      o[r] = acc;
    }
#pragma unroll
    for (int r = 0; r < D; ++r) Dv[r] = o[r];
  }
}

// second derivative along `axis` of node j (device order)
template <int D>
__device__ __forceinline__ double dd_axis64(const DTab32<D>& T, int64_t j, int axis, const double* __restrict__ phi0,
                                            const double* __restrict__ dd0_irr) {
  if (j >= T.nR) return dd0_irr[(int64_t)axis * T.nI + (j - T.nR)];
  const uint32_t codes = T.r_meta[j];
  const double dm = level_size64(T.tsize64[axis], T.base, (codes >> (8 * axis)) & 15u);
  const double dp = level_size64(T.tsize64[axis], T.base, (codes >> (8 * axis + 4)) & 15u);
  const double fm = phi0[T.r_nbr[(int64_t)(2 * axis) * T.nR + j]];
  const double fp = phi0[T.r_nbr[(int64_t)(2 * axis + 1) * T.nR + j]];
  return central_dd64(fp, phi0[j], fm, dp, dm);
}

__global__ void k_gather64(const double* __restrict__ src, const int32_t* __restrict__ perm, double* __restrict__ dst, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = src[perm[i]];
}

template <int D>
__global__ void __launch_bounds__(TPB) k_dd0_irr(DTab32<D> T, const double* __restrict__ phi0, double* __restrict__ dd0_irr) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= T.nI) return;
  double Dv[D];
  laplace_irr64<D>(T, i, phi0, phi0[T.nR + i], Dv);
#pragma unroll
  for (int a = 0; a < D; ++a) dd0_irr[(int64_t)a * T.nI + i] = Dv[a];
}

// phi_0's quadratic neighbour in direction dir (ngbd_with_quadratic_interpolation), FP64
template <int D>
__device__ __forceinline__ double quad_nb_m64(const DTab32<D>& T, int64_t n, int dir, const double* __restrict__ phi0,
                                              const double* __restrict__ dd0_irr) {
  if (n < T.nR) return phi0[T.r_nbr[(int64_t)dir * T.nR + n]];
  const int64_t i = n - T.nR;
  const uint32_t meta = T.i_meta[i];
  double v = lin_irr64<D>(T, meta, dir, i, phi0);
  if (face_count(meta, dir) > 1) {
#pragma unroll
    for (int j = 0; j < D - 1; ++j)
      v = fma(-T.i_q64[(int64_t)(dir * (D - 1) + j) * T.nI + i], dd0_irr[(int64_t)tan_axis32(dir >> 1, j) * T.nI + i], v);
  }
  return v;
}

// pass 1 (every node): anchoring, limits, sign and the sign test against each of phi_0's quadratic
// neighbours; the cut directions go into the status word and interface-adjacent nodes are appended to a
// list.
template <int D>
__global__ void __launch_bounds__(TPB) k_prep_classify(DTab32<D> T, const double* __restrict__ phi0, const double* __restrict__ dd0_irr,
                                                       double zdt, double lim_lo, double lim_hi, uint16_t* __restrict__ status,
                                                       int32_t* __restrict__ near_list, unsigned* __restrict__ near_count) {
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  bool near = false;
  if (n < T.N) {
    const double p0 = phi0[n];
    uint16_t st;
    if (fabs(p0) < zdt) {
      st = ST_ANCHORED;
    } else if (!(lim_lo < p0 && p0 < lim_hi)) {
      st = ST_OUTSIDE;
    } else {
      st = (p0 > 0.0) ? ST_POSITIVE : 0;
      uint32_t cut = 0;
#pragma unroll
      for (int dir = 0; dir < 2 * D; ++dir)
        if (product_negative(p0, quad_nb_m64<D>(T, n, dir, phi0, dd0_irr))) cut |= 1u << dir;
      if (cut) {
        near = true;
        st |= (uint16_t)(ST_NEAR | (cut << ST_CUT_SHIFT));
      }
    }
    status[n] = st;
  }
  const unsigned mask = __ballot_sync(0xffffffffu, near);
  if (mask) {
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(mask) - 1;
    unsigned base = 0;
    if (lane == leader) base = atomicAdd(near_count, (unsigned)__popc(mask));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (near) near_list[base + __popc(mask & ((1u << lane) - 1))] = (int32_t)n;
  }
}

// grid distance of node n (device order) in direction dir: its level's cell size, or the table distance
template <int D>
__device__ __forceinline__ double grid_distance64(const DTab32<D>& T, int64_t n, int dir) {
  if (n < T.nR) return level_size64(T.tsize64[dir >> 1], T.base, (T.r_meta[n] >> (4 * dir)) & 15u);
  return T.i_d64[(int64_t)dir * T.nI + (n - T.nR)];
}

// subcell distance of node n in the cut direction dir (src/my_p4est_level_set.cpp:133-211)
template <int D>
__device__ double subcell_distance64(const DTab32<D>& T, const double* __restrict__ phi0, const double* __restrict__ dd0_irr,
                                     int order_space, int64_t n, int dir) {
  constexpr int H = Dim<D>::HALF;
  const int axis = dir >> 1;
  const double p0 = phi0[n];
  const double s = grid_distance64<D>(T, n, dir);
  const double fn = quad_nb_m64<D>(T, n, dir, phi0, dd0_irr);
  double xx0 = 0.0, xx_nb = 0.0;
  if (order_space > 1) {
    xx0 = dd_axis64<D>(T, n, axis, phi0, dd0_irr);
    // f_<dir>_linear of phi_0's second derivative along axis
    if (n < T.nR) {
      xx_nb = dd_axis64<D>(T, T.r_nbr[(int64_t)dir * T.nR + n], axis, phi0, dd0_irr);
    } else {
      const int64_t i = n - T.nR;
      const int c = face_count(T.i_meta[i], dir);
      const int64_t base = (int64_t)(dir * H) * T.nI + i;
      if (c == 1) {
        xx_nb = dd_axis64<D>(T, T.i_nbr[base], axis, phi0, dd0_irr);
      } else {
        for (int kk = 0; kk < c; ++kk)
          xx_nb = fma(T.i_wf64[base + kk * T.nI], dd_axis64<D>(T, T.i_nbr[base + kk * T.nI], axis, phi0, dd0_irr), xx_nb);
      }
    }
  }
  if (dir & 1)
    return order_space > 1 ? st64::interface_location_2nd(0.0, s, p0, fn, xx0, xx_nb) : st64::interface_location(0.0, s, p0, fn);
  return order_space > 1 ? -st64::interface_location_2nd(-s, 0.0, fn, p0, xx_nb, xx0) : -st64::interface_location(-s, 0.0, fn, p0);
}

// pass 2 (interface-adjacent nodes): subcell distances. A warp takes 32 listed nodes, writes the grid
// distance of every direction that is not cut, and deals the warp's cut (node, direction) pairs out to
// its lanes, so each lane computes only cut directions and only the second derivatives along their axis
// (a node has one or two cut directions of its 2D).
template <int D>
__global__ void __launch_bounds__(TPB) k_prep_subcell(DTab32<D> T, const double* __restrict__ phi0, const double* __restrict__ dd0_irr,
                                                      double zdt, int order_space, const int32_t* __restrict__ near_list,
                                                      const unsigned* __restrict__ near_count, const uint16_t* __restrict__ status,
                                                      float* __restrict__ s_near) {
  constexpr unsigned FULL = 0xffffffffu;
  const int64_t N = T.N;
  const unsigned cnt = *near_count;
  const int lane = threadIdx.x & 31;
  const unsigned warp = (unsigned)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const unsigned nwarps = (unsigned)((gridDim.x * blockDim.x) >> 5);
  for (unsigned base = warp * 32u; base < cnt; base += nwarps * 32u) {  // the same trip count for every lane of the warp
    const unsigned k = base + (unsigned)lane;
    const bool valid = k < cnt;
    const int n = valid ? near_list[k] : 0;
    const uint32_t cut = valid ? ((uint32_t)status[n] >> ST_CUT_SHIFT) & ((1u << (2 * D)) - 1u) : 0u;
    if (valid) {
#pragma unroll
      for (int dir = 0; dir < 2 * D; ++dir)
        if (!((cut >> dir) & 1u)) s_near[(int64_t)dir * N + n] = (float)max2(grid_distance64<D>(T, n, dir), zdt);
    }
    // inclusive prefix sum of the lanes' cut counts
    const unsigned c = (unsigned)__popc(cut);
    unsigned incl = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned v = __shfl_up_sync(FULL, incl, o);
      if (lane >= o) incl += v;
    }
    const unsigned total = __shfl_sync(FULL, incl, 31);
    for (unsigned t0 = 0; t0 < total; t0 += 32u) {  // warp-uniform
      const unsigned t = t0 + (unsigned)lane;
      // owner: the lowest lane whose inclusive count exceeds t
      int pos = 0;
#pragma unroll
      for (int step = 16; step > 0; step >>= 1) {
        const unsigned v = __shfl_sync(FULL, incl, pos + step - 1);
        if (v <= t) pos += step;
      }
      const unsigned o_incl = __shfl_sync(FULL, incl, pos);
      const uint32_t o_cut = __shfl_sync(FULL, cut, pos);
      const int o_n = __shfl_sync(FULL, n, pos);
      if (t < total) {
        // the j-th cut direction of the owner, j counted from its first item
        int j = (int)(t - (o_incl - (unsigned)__popc(o_cut)));
        int dir = 0;
#pragma unroll
        for (int d = 0; d < 2 * D; ++d)
          if ((o_cut >> d) & 1u) {
            if (j == 0) dir = d;
            --j;
          }
        const double sd = subcell_distance64<D>(T, phi0, dd0_irr, order_space, o_n, dir);
        s_near[(int64_t)dir * N + o_n] = (float)max2(sd, zdt);
      }
    }
  }
}

__global__ void k_gather_f32(const double* __restrict__ src, const int32_t* __restrict__ perm, float* __restrict__ dst, int64_t n,
                             int64_t src_stride, int64_t dst_stride, int blocks) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t p = perm[i];
  for (int b = 0; b < blocks; ++b) dst[b * dst_stride + i] = (float)src[b * src_stride + p];
}
__global__ void k_scatter_f64(const float* __restrict__ src, const int32_t* __restrict__ perm, const uint16_t* __restrict__ status,
                              const uint16_t* __restrict__ lim, double* __restrict__ dst, int64_t n, int64_t src_stride,
                              int64_t dst_stride, int blocks) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (status && (status[i] & ST_OUTSIDE)) return;
  if (lim && lim[i] == 0) return;  // a grid of a batch run for zero iterations keeps its values
  const int64_t p = perm[i];
  for (int b = 0; b < blocks; ++b) dst[b * dst_stride + p] = (double)src[b * src_stride + i];
}

inline unsigned nblocks(int64_t n) { return (unsigned)((n + TPB - 1) / TPB); }

}  // namespace

template <int D>
void launch_dd32(const DTab32<D>& T, const float* f, float* dd, cudaStream_t s) {
  if (T.N == 0) return;
  k_dd32<D><<<nblocks(T.N), TPB, 0, s>>>(T, f, dd);
}

template <int D>
void launch_reinit_prep_mixed(const DTab32<D>& T, const int32_t* perm, const double* phi0, double zdt, double lim_lo, double lim_hi,
                              int order_space, double* phi0_dev, double* dd0_irr, uint16_t* status, float* s_near, int32_t* near_list,
                              unsigned* near_count, cudaStream_t s) {
  if (T.N == 0) return;
  cudaMemsetAsync(near_count, 0, sizeof(unsigned), s);
  k_gather64<<<nblocks(T.N), TPB, 0, s>>>(phi0, perm, phi0_dev, T.N);
  if (T.nI) k_dd0_irr<D><<<nblocks(T.nI), TPB, 0, s>>>(T, phi0_dev, dd0_irr);
  k_prep_classify<D><<<nblocks(T.N), TPB, 0, s>>>(T, phi0_dev, dd0_irr, zdt, lim_lo, lim_hi, status, near_list, near_count);
  k_prep_subcell<D><<<(unsigned)device_sm_count() * 8u, TPB, 0, s>>>(T, phi0_dev, dd0_irr, zdt, order_space, near_list, near_count, status, s_near);
}


template <int D>
void launch_dd_x32(const DTab32<D>& T, const float* f, float* ddx, cudaStream_t s, int tpb) {
  const int64_t n = T.nI + T.nX;
  if (n) k_dd_x32<D><<<(unsigned)((n + tpb - 1) / tpb), tpb, 0, s>>>(T, f, ddx);
}

__global__ void k_freeze32(const uint16_t* __restrict__ lim, int it, uint16_t* __restrict__ status, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && lim[i] <= it) status[i] |= ST_FROZEN;
}

void launch_freeze32(const uint16_t* lim, int it, uint16_t* status, int64_t n, cudaStream_t s) {
  if (n) k_freeze32<<<nblocks(n), TPB, 0, s>>>(lim, it, status, n);
}

template <int D>
static int persistent_blocks(const void* kernel) {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, TPB, 0);
  return device_sm_count() * (per_sm > 0 ? per_sm : 1);
}

// the bulk copies read 16-byte aligned spans from the bases of these arrays
template <int D>
static bool uniform_bulk_ok(const DTab32<D>& T, const uint16_t* status, const float* phin, const float* avg_with) {
  auto al = [](const void* p) { return ((uintptr_t)p & 15) == 0; };
  return al(status) && al(phin) && al(avg_with) && al(T.r_meta) && al(T.r_nbr) && al(T.r_nbr2);
}

// the bulk-copy uniform kernel with STAGES tiles in flight: shared memory per CTA and the full-wave grid
// are set up again whenever the tile or the halo changes
template <int D, bool AVG, int STAGES>
static void bulk_launch(const DTab32<D>& T, const uint16_t* status, const float* s_near, const float* phin, float* out,
                        const float* avg_with, int* err, long long wait_cycles, int halo, int tpb, int blocks, unsigned max_grid,
                        cudaStream_t s) {
  using B = UniBulk<D, AVG>;
  const uint32_t smem = STAGES * B::stage_bytes(tpb, halo);
  auto kern = k_reinit_uniform32_bulk<D, AVG, STAGES, 1>;
  static uint32_t configured_smem = 0;
  static int configured_tpb = 0, per_sm = 0;
  if (configured_smem != smem || configured_tpb != tpb) {
    // a failure here makes the launch below fail, which the caller's cudaGetLastError reports
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, tpb, smem);
    configured_smem = smem;
    configured_tpb = tpb;
  }
  const int full = device_sm_count() * (per_sm > 0 ? per_sm : 1);
  const int gb = blocks > 0 ? std::min(blocks, full) : full;
  const unsigned g = std::min<unsigned>((unsigned)gb, max_grid);
  kern<<<g, tpb, smem, s>>>(T, status, s_near, phin, out, avg_with, err, wait_cycles, halo);
}

template <int D, int OS, bool AVG, bool ADV>
static void fused_launch(const DTab32<D>& T, int part, const uint16_t* status, const float* s_near, const float* phin, const float* ddx,
                         float* out, const float* avg_with, cudaStream_t s, const StageCfg& cfg, int* err, const float* vn, float adv_dt) {
  static int gb_reg = 0, gb_uni = 0, gb_uni2 = 0, gb_uni5 = 0;
  if (!gb_reg) gb_reg = persistent_blocks<D>((const void*)k_reinit_fused_reg32<D, OS, AVG, ADV>);
  if (!gb_uni) gb_uni = persistent_blocks<D>((const void*)k_reinit_uniform32<D, AVG, 1, ADV>);
  if (!gb_uni2) gb_uni2 = persistent_blocks<D>((const void*)k_reinit_uniform32<D, AVG, 2, ADV>);
  if (!gb_uni5) gb_uni5 = persistent_blocks<D>((const void*)k_reinit_uniform32<D, AVG, 1, ADV, 6>);
  const int tpb = (cfg.tpb > 0 && cfg.tpb <= TPB) ? cfg.tpb : TPB;
  // a persistent grid sized for TPB-thread blocks keeps the same thread count with smaller blocks
  const int scale = TPB / tpb;
  auto grid_of = [&](int64_t n) { return (unsigned)((n + tpb - 1) / tpb); };
  const int64_t uni_end = (OS > 1) ? T.nU : 0;  // the uniform kernel is second order in space only
  if (part == STAGE_PART_IRREGULAR && T.nI)
    k_reinit_fused32<D, OS, AVG, ADV><<<grid_of(T.nI), tpb, 0, s>>>(T, status, s_near, phin, ddx, out, avg_with, T.nR, T.N, vn, adv_dt);
  if (part == STAGE_PART_REGULAR && T.nR > uni_end) {
    const int gb = cfg.regular_blocks > 0 ? std::min(cfg.regular_blocks, gb_reg * scale) : gb_reg * scale;
    k_reinit_fused_reg32<D, OS, AVG, ADV><<<(unsigned)std::min<int64_t>(gb, grid_of(T.nR - uni_end)), tpb, 0, s>>>(
        T, status, s_near, phin, ddx, out, avg_with, (int)uni_end, (int)T.nR, vn, adv_dt);
  }
  // the bulk-copy uniform kernel serves the reinitialisation only; the advection stage uses the register pipeline
  if (!ADV && part == STAGE_PART_UNIFORM && uni_end > 0 && (cfg.depth == 3 || cfg.depth == 4) && uniform_bulk_ok(T, status, phin, avg_with) &&
      err) {
    const int halo = cfg.halo >= 0 ? (cfg.halo & ~3) : 512;
    const long long wc = cfg.wait_cycles > 0 ? cfg.wait_cycles : kFullWaitCycles;
    if (cfg.depth == 4)
      bulk_launch<D, AVG, 3>(T, status, s_near, phin, out, avg_with, err, wc, halo, tpb, cfg.uniform_blocks, grid_of(uni_end), s);
    else
      bulk_launch<D, AVG, 2>(T, status, s_near, phin, out, avg_with, err, wc, halo, tpb, cfg.uniform_blocks, grid_of(uni_end), s);
  } else if (part == STAGE_PART_UNIFORM && uni_end > 0) {
    const int full = (cfg.depth == 2 ? gb_uni2 : cfg.depth == 5 ? gb_uni5 : gb_uni) * scale;
    const int gb = cfg.uniform_blocks > 0 ? std::min(cfg.uniform_blocks, full) : full;
    const unsigned g = (unsigned)std::min<int64_t>(gb, grid_of(uni_end));
    if (cfg.depth == 2)
      k_reinit_uniform32<D, AVG, 2, ADV><<<g, tpb, 0, s>>>(T, status, s_near, phin, out, avg_with, vn, adv_dt);
    else if (cfg.depth == 5)
      k_reinit_uniform32<D, AVG, 1, ADV, 6><<<g, tpb, 0, s>>>(T, status, s_near, phin, out, avg_with, vn, adv_dt);
    else
      k_reinit_uniform32<D, AVG, 1, ADV><<<g, tpb, 0, s>>>(T, status, s_near, phin, out, avg_with, vn, adv_dt);
  }
}

template <int D>
void launch_reinit_part32(const DTab32<D>& T, int part, int order_space, const uint16_t* status, const float* s_near,
                          const float* phin, const float* ddx, float* out, const float* avg_with, cudaStream_t s, const StageCfg& cfg,
                          int* err, const float* adv_vn, float adv_dt) {
  if (T.N == 0) return;
  if (adv_vn) {  // the normal-advection stage: second order in space, every node updated
    if (avg_with) fused_launch<D, 2, true, true>(T, part, status, s_near, phin, ddx, out, avg_with, s, cfg, err, adv_vn, adv_dt);
    else fused_launch<D, 2, false, true>(T, part, status, s_near, phin, ddx, out, avg_with, s, cfg, err, adv_vn, adv_dt);
  } else if (order_space > 1) {
    if (avg_with) fused_launch<D, 2, true, false>(T, part, status, s_near, phin, ddx, out, avg_with, s, cfg, err, nullptr, 0.0f);
    else fused_launch<D, 2, false, false>(T, part, status, s_near, phin, ddx, out, avg_with, s, cfg, err, nullptr, 0.0f);
  } else {
    if (avg_with) fused_launch<D, 1, true, false>(T, part, status, s_near, phin, ddx, out, avg_with, s, cfg, err, nullptr, 0.0f);
    else fused_launch<D, 1, false, false>(T, part, status, s_near, phin, ddx, out, avg_with, s, cfg, err, nullptr, 0.0f);
  }
}

template <int D>
void launch_advect_stage32(const DTab32<D>& T, const float* phin, const float* ddq, const float* ddm, const float* vn, float dt,
                           float* out, const float* avg_with, cudaStream_t s) {
  if (T.N == 0) return;
  if (avg_with)
    k_advect_stage32<D, true><<<nblocks(T.N), TPB, 0, s>>>(T, phin, ddq, ddm, vn, dt, out, avg_with);
  else
    k_advect_stage32<D, false><<<nblocks(T.N), TPB, 0, s>>>(T, phin, ddq, ddm, vn, dt, out, avg_with);
}

template <int D>
__global__ void k_pack_uniform32(DTab32<D> T, int4* __restrict__ out) {
  const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= T.nR) return;
  int32_t w[4 * D];
  for (int dir = 0; dir < 2 * D; ++dir) {
    w[dir] = T.r_nbr[dir * T.nR + m];
    w[2 * D + dir] = T.r_nbr2[dir * T.nR + m];
  }
  for (int k = 0; k < D; ++k) out[(int64_t)D * m + k] = make_int4(w[4 * k], w[4 * k + 1], w[4 * k + 2], w[4 * k + 3]);
}

template <int D>
void launch_pack_uniform32(const DTab32<D>& T, int4* out, cudaStream_t s) {
  if (T.nR > 0) k_pack_uniform32<D><<<nblocks(T.nR), TPB, 0, s>>>(T, out);
}

void launch_gather_f32(const double* src, const int32_t* perm, float* dst, int64_t n, int64_t src_stride, int64_t dst_stride,
                       int blocks, cudaStream_t s) {
  if (n) k_gather_f32<<<nblocks(n), TPB, 0, s>>>(src, perm, dst, n, src_stride, dst_stride, blocks);
}
void launch_scatter_f64(const float* src, const int32_t* perm, const uint16_t* status, double* dst, int64_t n, int64_t src_stride,
                        int64_t dst_stride, int blocks, cudaStream_t s, const uint16_t* lim) {
  if (n) k_scatter_f64<<<nblocks(n), TPB, 0, s>>>(src, perm, status, lim, dst, n, src_stride, dst_stride, blocks);
}

#define LSG_INST(D)                                                                                                             \
  template void launch_dd32<D>(const DTab32<D>&, const float*, float*, cudaStream_t);                                           \
  template void launch_reinit_prep_mixed<D>(const DTab32<D>&, const int32_t*, const double*, double, double, double, int,       \
                                            double*, double*, uint16_t*, float*, int32_t*, unsigned*, cudaStream_t);            \
  template void launch_advect_stage32<D>(const DTab32<D>&, const float*, const float*, const float*, const float*, float, float*, \
                                         const float*, cudaStream_t);                                                           \
  template void launch_dd_x32<D>(const DTab32<D>&, const float*, float*, cudaStream_t, int);                                  \
  template void launch_reinit_part32<D>(const DTab32<D>&, int, int, const uint16_t*, const float*, const float*, const float*,  \
                                        float*, const float*, cudaStream_t, const StageCfg&, int*, const float*, float);        \
  template void launch_pack_uniform32<D>(const DTab32<D>&, int4*, cudaStream_t);
LSG_INST(2)
LSG_INST(3)
#undef LSG_INST

}  // namespace lsg
