// Mixed-precision level-set kernels: the stencil, Godunov Hamiltonian and RK stages in FP32 with
// FP32 accumulation; the subcell interface distances (quadratic root through the sign change of
// phi_0) in FP64, computed once per call because they depend on phi_0 only.
//
// The arithmetic follows the same reference routines as the FP64 kernels (see stencil64.cuh and
// kernels_fp64.cu) with every geometric division folded into precomputed FP32 coefficients.
#include "kernels.h"
#include "stencil64.cuh"
#include "tables.hpp"

namespace lsg {

namespace {

constexpr int TPB = 256;

__device__ __forceinline__ int tan_axis32(int axis, int j) { return j == 0 ? (axis == 0 ? 1 : 0) : (axis == 2 ? 1 : 2); }

__device__ __forceinline__ int face_count(uint32_t meta, int dir) { return (int)((meta >> (2 * dir)) & 3u) + 1; }

// Linear interpolation over the face nodes of direction dir (weights normalised; a single face node
// has weight exactly 1).
template <int D>
__device__ __forceinline__ float lin32(const DTab32<D>& T, uint32_t meta, int dir, int64_t n, const float* __restrict__ f) {
  constexpr int H = Dim<D>::HALF;
  const int64_t N = T.N;
  const int64_t base = (int64_t)(dir * H) * N + n;
  const int c = face_count(meta, dir);
  const int32_t i0 = __ldg(T.nbr + base);
  if (c == 1) return __ldg(f + i0);
  float acc = __ldg(T.wf + base) * __ldg(f + i0);
#pragma unroll
  for (int k = 1; k < H; ++k)
    if (k < c) acc = fmaf(__ldg(T.wf + base + k * N), __ldg(f + __ldg(T.nbr + base + k * N)), acc);
  return acc;
}

template <int D>
__device__ __forceinline__ void laplace32(const DTab32<D>& T, uint32_t meta, int64_t n, const float* __restrict__ f, float* Dv) {
  const int64_t N = T.N;
  const float f0 = __ldg(f + n);
#pragma unroll
  for (int a = 0; a < D; ++a) {
    const float fm = lin32<D>(T, meta, 2 * a, n, f);
    const float fp = lin32<D>(T, meta, 2 * a + 1, n, f);
    const float dm = __ldg(T.d + (int64_t)(2 * a) * N + n), dp = __ldg(T.d + (int64_t)(2 * a + 1) * N + n);
    // ((fp-f0)/dp + (fm-f0)/dm) * 2/(dp+dm)
    Dv[a] = __fdividef(2.0f * fmaf(fp - f0, dm, (fm - f0) * dp), dp * dm * (dp + dm));
  }
  if (meta & (1u << 16)) {
    const float* M = T.corr + (int64_t)D * D * __ldg(T.cidx + n);
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
}

template <int D>
__device__ __forceinline__ float quad_nb32(const DTab32<D>& T, uint32_t meta, int dir, int64_t n, const float* __restrict__ f,
                                           const float* Dv) {
  float v = lin32<D>(T, meta, dir, n, f);
  if (face_count(meta, dir) > 1) {
    const int64_t N = T.N;
    const int axis = dir >> 1;
#pragma unroll
    for (int j = 0; j < D - 1; ++j) v = fmaf(-__ldg(T.q + (int64_t)(dir * (D - 1) + j) * N + n), Dv[tan_axis32(axis, j)], v);
  }
  return v;
}

template <int D>
__global__ void __launch_bounds__(TPB) k_dd32(DTab32<D> T, const float* __restrict__ f, float* __restrict__ dd) {
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= T.N) return;
  const uint32_t meta = __ldg(T.meta + n);
  float Dv[D];
  laplace32<D>(T, meta, n, f, Dv);
#pragma unroll
  for (int a = 0; a < D; ++a) dd[(int64_t)a * T.N + n] = Dv[a];
}

// FP64 second derivative along `axis`, linearly interpolated to the face of direction dir
// (f_<dir>_linear of phi_0's second derivatives, computed here from phi_0 itself).
template <int D>
__device__ double lin_dd64(const DTab64<D>& T, int dir, int axis, int64_t n, const double* __restrict__ f) {
  constexpr int H = Dim<D>::HALF;
  const int64_t N = T.N;
  const int64_t base = (int64_t)(dir * H) * N + n;
  double acc = 0.0;
#pragma unroll
  for (int k = 0; k < H; ++k) {
    const int32_t ik = T.nbr[base + k * N];
    if (ik < 0) continue;
    double Dj[D];
    st64::laplace64<D>(T, ik, f, Dj);
    acc = acc + Dj[axis] * T.w[base + k * N];
  }
  return acc / T.nrm[(int64_t)dir * N + n];
}

// Everything reinitialize_one_iteration derives from phi_0 alone, in FP64 (see k_reinit_prep64).
template <int D>
__global__ void __launch_bounds__(TPB) k_reinit_prep_mixed(DTab64<D> T, const uint32_t* __restrict__ meta32,
                                                           const double* __restrict__ phi0, double zdt, double lim_lo,
                                                           double lim_hi, int order_space, uint16_t* __restrict__ status,
                                                           float* __restrict__ s_near) {
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t N = T.N;
  if (n >= N) return;
  const double p0 = phi0[n];
  if (fabs(p0) < zdt) {
    status[n] = ST_ANCHORED;
    return;
  }
  if (!(lim_lo < p0 && p0 < lim_hi)) {
    status[n] = ST_OUTSIDE;
    return;
  }
  const uint32_t meta = meta32[n];
  bool hanging = false;
#pragma unroll
  for (int dir = 0; dir < 2 * D; ++dir) hanging = hanging || face_count(meta, dir) > 1;
  double Dv[D];
  bool have_dv = false;
  if (hanging) {
    st64::laplace64<D>(T, n, phi0, Dv);
    have_dv = true;
  }
  double fn[2 * D];
  bool near = false;
#pragma unroll
  for (int dir = 0; dir < 2 * D; ++dir) {
    if (face_count(meta, dir) == 1)
      fn[dir] = phi0[T.nbr[(int64_t)(dir * Dim<D>::HALF) * N + n]];
    else
      fn[dir] = st64::quad_nb64<D>(T, dir, n, phi0, Dv);
    near = near || (p0 * fn[dir] < 0.0);
  }
  uint16_t st = (p0 > 0.0) ? ST_POSITIVE : 0;
  if (near) {
    st |= ST_NEAR;
    if (!have_dv) st64::laplace64<D>(T, n, phi0, Dv);
    double s[2 * D];
#pragma unroll
    for (int dir = 0; dir < 2 * D; ++dir) s[dir] = T.d[(int64_t)dir * N + n];
#pragma unroll
    for (int dir = 0; dir < 2 * D; ++dir) {
      if (!(p0 * fn[dir] < 0.0)) continue;
      st |= (uint16_t)(1u << (ST_CUT_SHIFT + dir));
      const int axis = dir >> 1;
      if (dir & 1) {
        if (order_space > 1)
          s[dir] = st64::interface_location_2nd(0.0, s[dir], p0, fn[dir], Dv[axis], lin_dd64<D>(T, dir, axis, n, phi0));
        else
          s[dir] = st64::interface_location(0.0, s[dir], p0, fn[dir]);
      } else {
        if (order_space > 1)
          s[dir] = -st64::interface_location_2nd(-s[dir], 0.0, fn[dir], p0, lin_dd64<D>(T, dir, axis, n, phi0), Dv[axis]);
        else
          s[dir] = -st64::interface_location(-s[dir], 0.0, fn[dir], p0);
      }
    }
#pragma unroll
    for (int dir = 0; dir < 2 * D; ++dir) s_near[(int64_t)dir * N + n] = (float)max2(s[dir], zdt);
  }
  status[n] = st;
}

template <int D, int ORDER_SPACE, bool AVG>
__global__ void __launch_bounds__(TPB) k_reinit_stage32(DTab32<D> T, const uint16_t* __restrict__ status,
                                                        const float* __restrict__ s_near, const float* __restrict__ phin,
                                                        const float* __restrict__ dd, float* out, const float* avg_with) {
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t N = T.N;
  if (n >= N) return;
  const uint16_t st = status[n];
  float r;
  if (st & ST_ANCHORED) {
    r = 0.0f;
  } else if (st & ST_OUTSIDE) {
    r = phin[n];
  } else {
    const uint32_t meta = __ldg(T.meta + n);
    const float f0 = __ldg(phin + n);
    float Dv[D];
#pragma unroll
    for (int a = 0; a < D; ++a) Dv[a] = __ldg(dd + (int64_t)a * N + n);
    float fnb[2 * D], s[2 * D], xx0[D], xxnb[2 * D];
#pragma unroll
    for (int dir = 0; dir < 2 * D; ++dir) fnb[dir] = quad_nb32<D>(T, meta, dir, n, phin, Dv);
    if (st & ST_NEAR) {
#pragma unroll
      for (int dir = 0; dir < 2 * D; ++dir) {
        s[dir] = __ldg(s_near + (int64_t)dir * N + n);
        if (st & (1u << (ST_CUT_SHIFT + dir))) fnb[dir] = 0.0f;
      }
    } else {
#pragma unroll
      for (int dir = 0; dir < 2 * D; ++dir) s[dir] = __ldg(T.d + (int64_t)dir * N + n);
    }
    if (ORDER_SPACE > 1) {
#pragma unroll
      for (int a = 0; a < D; ++a) {
        xx0[a] = Dv[a];
        xxnb[2 * a] = lin32<D>(T, meta, 2 * a, n, dd + (int64_t)a * N);
        xxnb[2 * a + 1] = lin32<D>(T, meta, 2 * a + 1, n, dd + (int64_t)a * N);
      }
    }
    const uint32_t wl = meta >> 24;
#pragma unroll
    for (int a = 0; a < D; ++a) {
      if (wl & (1u << (2 * a))) {
        s[2 * a] = s[2 * a + 1];
        fnb[2 * a] = fnb[2 * a + 1];
        if (ORDER_SPACE > 1) xx0[a] = xxnb[2 * a] = xxnb[2 * a + 1] = 0.0f;
      }
      if (wl & (1u << (2 * a + 1))) {
        s[2 * a + 1] = s[2 * a];
        fnb[2 * a + 1] = fnb[2 * a];
        if (ORDER_SPACE > 1) xx0[a] = xxnb[2 * a] = xxnb[2 * a + 1] = 0.0f;
      }
    }
    float gp[D], gm[D];
#pragma unroll
    for (int a = 0; a < D; ++a) {
      gp[a] = __fdividef(fnb[2 * a + 1] - f0, s[2 * a + 1]);
      gm[a] = __fdividef(f0 - fnb[2 * a], s[2 * a]);
      if (ORDER_SPACE > 1) {
        gm[a] = fmaf(0.5f * s[2 * a], minmodf(xxnb[2 * a], xx0[a]), gm[a]);
        gp[a] = fmaf(-0.5f * s[2 * a + 1], minmodf(xxnb[2 * a + 1], xx0[a]), gp[a]);
      }
    }
    const bool pos = (st & ST_POSITIVE) != 0;
    const float sgn = pos ? 1.0f : -1.0f;
    float dt = fminf(s[0], s[1]);
#pragma unroll
    for (int dir = 2; dir < 2 * D; ++dir) dt = fminf(dt, s[dir]);
    dt *= (1.0f / D);
    float h = 0.0f;
#pragma unroll
    for (int a = 0; a < D; ++a) {
      if (sgn * gp[a] > 0.0f) gp[a] = 0.0f;
      if (sgn * gm[a] < 0.0f) gm[a] = 0.0f;
      h += fmaxf(gp[a] * gp[a], gm[a] * gm[a]);
    }
    r = f0 - dt * sgn * (sqrtf(h) - 1.0f);
    if (pos ? (r < 0.0f) : (r > 0.0f)) r = -r;
  }
  if (AVG) r = 0.5f * (avg_with[n] + r);
  out[n] = r;
}

template <int D, bool AVG>
__global__ void __launch_bounds__(TPB) k_advect_stage32(DTab32<D> T, const float* __restrict__ phin, const float* __restrict__ ddq,
                                                        const float* __restrict__ ddm, const float* __restrict__ vn, float dt,
                                                        float* out, const float* avg_with) {
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t N = T.N;
  if (n >= N) return;
  const uint32_t meta = __ldg(T.meta + n);
  const float f0 = __ldg(phin + n);
  float Dq[D];
#pragma unroll
  for (int a = 0; a < D; ++a) Dq[a] = __ldg(ddq + (int64_t)a * N + n);
  float fnb[2 * D], s[2 * D], xx0[D], xxnb[2 * D];
#pragma unroll
  for (int dir = 0; dir < 2 * D; ++dir) {
    fnb[dir] = quad_nb32<D>(T, meta, dir, n, phin, Dq);
    s[dir] = __ldg(T.d + (int64_t)dir * N + n);
  }
#pragma unroll
  for (int a = 0; a < D; ++a) {
    xx0[a] = __ldg(ddm + (int64_t)a * N + n);
    xxnb[2 * a] = lin32<D>(T, meta, 2 * a, n, ddm + (int64_t)a * N);
    xxnb[2 * a + 1] = lin32<D>(T, meta, 2 * a + 1, n, ddm + (int64_t)a * N);
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

__global__ void k_f64_to_f32(const double* __restrict__ a, float* __restrict__ b, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = (float)a[i];
}
__global__ void k_f32_to_f64(const float* __restrict__ a, double* __restrict__ b, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = (double)a[i];
}
// Back to FP64 except where the reinitialisation leaves phi_0 untouched (outside the limits).
__global__ void k_f32_to_f64_status(const float* __restrict__ a, const uint16_t* __restrict__ st, double* __restrict__ b, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && !(st[i] & ST_OUTSIDE)) b[i] = (double)a[i];
}

inline unsigned nblocks(int64_t n) { return (unsigned)((n + TPB - 1) / TPB); }

}  // namespace

template <int D>
void launch_dd32(const DTab32<D>& T, const float* f, float* dd, cudaStream_t s) {
  if (T.N == 0) return;
  k_dd32<D><<<nblocks(T.N), TPB, 0, s>>>(T, f, dd);
}

template <int D>
void launch_reinit_prep_mixed(const DTab64<D>& T, const uint32_t* meta32, const double* phi0, double zdt, double lim_lo,
                              double lim_hi, int order_space, uint16_t* status, float* s_near, cudaStream_t s) {
  if (T.N == 0) return;
  k_reinit_prep_mixed<D><<<nblocks(T.N), TPB, 0, s>>>(T, meta32, phi0, zdt, lim_lo, lim_hi, order_space, status, s_near);
}

template <int D>
void launch_reinit_stage32(const DTab32<D>& T, int order_space, const uint16_t* status, const float* s_near, const float* phin,
                           const float* dd, float* out, const float* avg_with, cudaStream_t s) {
  if (T.N == 0) return;
  const unsigned g = nblocks(T.N);
  if (order_space > 1) {
    if (avg_with)
      k_reinit_stage32<D, 2, true><<<g, TPB, 0, s>>>(T, status, s_near, phin, dd, out, avg_with);
    else
      k_reinit_stage32<D, 2, false><<<g, TPB, 0, s>>>(T, status, s_near, phin, dd, out, avg_with);
  } else {
    if (avg_with)
      k_reinit_stage32<D, 1, true><<<g, TPB, 0, s>>>(T, status, s_near, phin, dd, out, avg_with);
    else
      k_reinit_stage32<D, 1, false><<<g, TPB, 0, s>>>(T, status, s_near, phin, dd, out, avg_with);
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

void launch_f64_to_f32(const double* src, float* dst, int64_t n, cudaStream_t s) {
  if (n) k_f64_to_f32<<<nblocks(n), TPB, 0, s>>>(src, dst, n);
}
void launch_f32_to_f64(const float* src, double* dst, int64_t n, cudaStream_t s) {
  if (n) k_f32_to_f64<<<nblocks(n), TPB, 0, s>>>(src, dst, n);
}
void launch_f32_to_f64_status(const float* src, const uint16_t* status, double* dst, int64_t n, cudaStream_t s) {
  if (n) k_f32_to_f64_status<<<nblocks(n), TPB, 0, s>>>(src, status, dst, n);
}

#define LSG_INST(D)                                                                                                             \
  template void launch_dd32<D>(const DTab32<D>&, const float*, float*, cudaStream_t);                                           \
  template void launch_reinit_prep_mixed<D>(const DTab64<D>&, const uint32_t*, const double*, double, double, double, int,      \
                                            uint16_t*, float*, cudaStream_t);                                                   \
  template void launch_reinit_stage32<D>(const DTab32<D>&, int, const uint16_t*, const float*, const float*, const float*,      \
                                         float*, const float*, cudaStream_t);                                                   \
  template void launch_advect_stage32<D>(const DTab32<D>&, const float*, const float*, const float*, const float*, float, float*, \
                                         const float*, cudaStream_t);
LSG_INST(2)
LSG_INST(3)
#undef LSG_INST

}  // namespace lsg
