// Node interpolation and the semi-Lagrangian departure-point step, FP64 (compiled with
// -fmad=false so every expression rounds as the reference's double arithmetic does).
//
//   point location     my_p4est_hierarchy_t::find_smallest_quadrant_containing_point and
//                      find_quadrant_containing_point (src/my_p4est_hierarchy.cpp:264-567), single
//                      process, non-periodic brick
//   clipping           clip_in_domain (src/my_p4est_utils.h:2177-2187)
//   weights            get_local_interpolation_weights (src/my_p4est_utils.cpp:367-408)
//   kernels            linear, quadratic, quadratic_non_oscillatory, _continuous_v1, _continuous_v2
//                      (src/my_p4est_utils.cpp:410-576)
//   per-point driver   my_p4est_interpolation_nodes_t::interpolate (src/my_p4est_interpolation_nodes.cpp:107-288)
//   backtrace          my_p4est_semi_lagrangian_t::advect_from_n_to_np1 (src/my_p4est_semi_lagrangian.cpp:108-223)
//   interface values   extend_from_interface_to_whole_domain_TVD, set-up part (src/my_p4est_level_set.cpp:3325-3633)
//
// One thread per point. The reference walks a cell tree from the root; here the leaf holding a
// logical point is found from a coarse-cell table plus a binary search over the sorted leaf keys
// (the same leaf: a leaf [x0, x0+h) holds the real coordinate s exactly when it holds floor(s)).
#include "kernels.h"
#include "stencil64.cuh"

namespace lsg {
namespace {

constexpr int TPB = 256;
constexpr double PI_D = 3.1415926535897932384626433832795;  // src/casl_math.h:15

inline int64_t nblocks(int64_t n) { return (n + TPB - 1) / TPB; }

template <int D>
__device__ __forceinline__ void clip_in_domain(const DLoc<D>& L, double* x) {
#pragma unroll
  for (int a = 0; a < D; ++a)
    if (x[a] < L.xyz_min[a] || x[a] > L.xyz_max[a]) x[a] = max2(L.xyz_min[a], min2(L.xyz_max[a], x[a]));
}

// leaf of tree tt containing the integer logical point X
template <int D>
__device__ __forceinline__ int32_t find_leaf(const DLoc<D>& L, int tt, const int32_t* X) {
  int32_t c[3] = {0, 0, 0};
#pragma unroll
  for (int a = 0; a < D; ++a) c[a] = X[a] >> (Dim<D>::MAXLEVEL - L.L0);
  const int64_t idx = (int64_t)tt * L.ncoarse + (int64_t)morton<D>(c);
  int32_t lo = __ldg(L.ctab + idx), hi = __ldg(L.ctab + idx + 1);
  const uint64_t key = ((uint64_t)tt << tree_shift<D>()) | morton<D>(X);
  while (lo < hi) {
    const int32_t mid = (lo + hi + 1) >> 1;
    if (__ldg(L.key + mid) <= key)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

// find_smallest_quadrant_containing_point for a point already clipped into the domain; -1 only if a
// probe left the brick, which clipping rules out.
template <int D>
__device__ int32_t locate(const DLoc<D>& L, const double* xyz) {
  const double ROOT = (double)Dim<D>::ROOT_LEN;
  const double qeps = (double)1 / ROOT;
  const double threshold = 0.01 * (double)1;
  double c[3] = {0, 0, 0};
  int tr[3] = {0, 0, 0};
  bool face[3] = {false, false, false};
#pragma unroll
  for (int a = 0; a < D; ++a) {
    double xs = xyz[a] - L.xyz_min[a];
    xs = st64::qdiv(xs, L.tree_dim[a]);
    xs = max2(qeps, min2(xs, L.n[a] - qeps));
    tr[a] = (int)floor(xs);
    c[a] = (xs - tr[a]) * ROOT;
    face[a] = (fabs(c[a] - floor(c[a])) < threshold || fabs(ceil(c[a]) - c[a]) < threshold);
  }
  int32_t best = -1;
  int best_level = -1;
  for (int i = (face[0] ? -1 : 0); i < 2; i += 2)
    for (int j = (face[1] ? -1 : 0); j < 2; j += 2)
      for (int k = (D == 3 && face[2] ? -1 : 0); k < (D == 3 ? 2 : 1); k += 2) {
        const int off[3] = {i, j, k};
        int t[3] = {tr[0], tr[1], tr[2]};
        int32_t X[3] = {0, 0, 0};
        bool inside = true;
#pragma unroll
        for (int a = 0; a < D; ++a) {
          double s = (off[a] == 0 ? c[a] : c[a] + off[a] * threshold);
          if (s < 0 || s >= ROOT) {
            const int slide = (int)floor(s / ROOT);
            s -= ((double)slide) * ROOT;
            t[a] = tr[a] + slide;
          }
          inside = inside && t[a] >= 0 && t[a] < L.n[a] && s >= 0 && s < ROOT;
          X[a] = (int32_t)floor(s);
        }
        if (!inside) continue;
        const int tt = __ldg(L.ijk_to_tree + ((int64_t)L.n[0] * L.n[1] * (D == 3 ? t[2] : 0) + (int64_t)L.n[0] * t[1] + t[0]));
        const int32_t q = find_leaf<D>(L, tt, X);
        const int lvl = __ldg(L.level + q);
        if (lvl > best_level) {
          best_level = lvl;
          best = q;
        }
      }
  return best;
}

// get_local_interpolation_weights at the point xg (as given, not clipped)
template <int D>
__device__ __forceinline__ void local_weights(const DLoc<D>& L, int32_t q, const double* xg, double* lw, double* sdw) {
  const uint64_t key = __ldg(L.key + q);
  const int tree = (int)(key >> tree_shift<D>());
  int32_t X[3] = {0, 0, 0};
  unmorton<D>(key & ((uint64_t(1) << tree_shift<D>()) - 1), X);
  const int lvl = __ldg(L.level + q);
  const double qh = st64::qdiv((double)(Dim<D>::ROOT_LEN >> lvl), (double)Dim<D>::ROOT_LEN);
  double d0[3], d1[3];
#pragma unroll
  for (int a = 0; a < D; ++a) {
    const double tmin = __ldg(L.tmin + 3 * tree + a), tmax = __ldg(L.tmax + 3 * tree + a);
    const double qmin = st64::qdiv((double)X[a], (double)Dim<D>::ROOT_LEN);
    double x = st64::qdiv(xg[a] - tmin, tmax - tmin);
    x = st64::qdiv(x - qmin, qh);
    d0[a] = 1.0 - x;
    d1[a] = x;
    const double h = (tmax - tmin) * qh;
    sdw[a] = h * h * d0[a] * d1[a];
  }
#pragma unroll
  for (int c = 0; c < Dim<D>::CHILDREN; ++c) {
    const double wx = (c & 1) ? d1[0] : d0[0];
    const double wy = ((c >> 1) & 1) ? d1[1] : d0[1];
    if (D == 3) {
      const double wz = ((c >> 2) & 1) ? d1[2] : d0[2];
      lw[c] = wx * wy * wz;
    } else {
      lw[c] = wx * wy;
    }
  }
}

template <int D, int M>
__device__ __forceinline__ double interpolate_local(const double* lw, const double* sdw, const double* f, const double (*fdd)[3]) {
  constexpr int CH = Dim<D>::CHILDREN;
  double r = 0.0;
  if (M == 0) {
#pragma unroll
    for (int j = 0; j < CH; ++j) r += +f[j] * lw[j];
    return r;
  }
  double dd[3] = {0, 0, 0};
  if (M == 1) {
#pragma unroll
    for (int j = 0; j < CH; ++j) {
#pragma unroll
      for (int i = 0; i < D; ++i) dd[i] = ((j == 0) ? 0.0 : dd[i]) + fdd[j][i] * lw[j];
      r += f[j] * lw[j];
    }
  } else if (M == 2) {
#pragma unroll
    for (int j = 0; j < CH; ++j) {
#pragma unroll
      for (int i = 0; i < D; ++i) dd[i] = (j == 0 ? fdd[j][i] : minmod(dd[i], fdd[j][i]));
      r += f[j] * lw[j];
    }
  } else if (M == 3) {
#pragma unroll
    for (int i = 0; i < D; ++i) {
      dd[i] = 0.0;
#pragma unroll
      for (int jm = 0; jm < CH; ++jm) {
        if ((jm >> i) & 1) continue;
        const int jp = jm | (1 << i);
        dd[i] += minmod(fdd[jm][i], fdd[jp][i]) * (lw[jm] + lw[jp]);
      }
    }
#pragma unroll
    for (int j = 0; j < CH; ++j) r += f[j] * lw[j];
  } else {
#pragma unroll
    for (int i = 0; i < D; ++i) {
      double m = 0, p = 0;
#pragma unroll
      for (int jm = 0; jm < CH; ++jm) {
        if ((jm >> i) & 1) continue;
        const int jp = jm | (1 << i);
        m += fdd[jm][i] * (lw[jm] + lw[jp]);
        p += fdd[jp][i] * (lw[jm] + lw[jp]);
      }
      dd[i] = minmod(m, p);
    }
#pragma unroll
    for (int j = 0; j < CH; ++j) r += f[j] * lw[j];
  }
  if (D == 3)
    r -= st64::scale2(sdw[0] * dd[0] + sdw[1] * dd[1] + sdw[2] * dd[2], -1);
  else
    r -= st64::scale2(sdw[0] * dd[0] + sdw[1] * dd[1], -1);
  return r;
}

// locate + weights + gather + interpolate nf fields at the point x (weights at x, location at clip(x))
template <int D, int M>
__device__ __forceinline__ void interpolate_at(const DLoc<D>& L, const double* x, int nf, const double* __restrict__ F,
                                               const double* __restrict__ Fdd, int64_t np, int64_t p, double* __restrict__ out) {
  constexpr int CH = Dim<D>::CHILDREN;
  double xc[3] = {0, 0, 0};
#pragma unroll
  for (int a = 0; a < D; ++a) xc[a] = x[a];
  clip_in_domain<D>(L, xc);
  const int32_t q = locate<D>(L, xc);
  if (q < 0) {
    for (int k = 0; k < nf; ++k) out[(int64_t)k * np + p] = __longlong_as_double(0x7ff8000000000000ll);
    return;
  }
  double lw[CH], sdw[3];
  local_weights<D>(L, q, x, lw, sdw);
  int32_t nd[CH];
#pragma unroll
  for (int j = 0; j < CH; ++j) nd[j] = __ldg(L.local_nodes + (int64_t)q * CH + j);
  const int64_t N = L.N;
  for (int k = 0; k < nf; ++k) {
    double f[CH], fdd[CH][3];
#pragma unroll
    for (int j = 0; j < CH; ++j) {
      f[j] = __ldg(F + (int64_t)k * N + nd[j]);
#pragma unroll
      for (int a = 0; a < D; ++a) fdd[j][a] = (M == 0 ? 0.0 : __ldg(Fdd + ((int64_t)k * D + a) * N + nd[j]));
    }
    out[(int64_t)k * np + p] = interpolate_local<D, M>(lw, sdw, f, fdd);
  }
}

template <int D, int M>
__global__ void __launch_bounds__(TPB) k_interp64(DLoc<D> L, const double* __restrict__ xyz, int64_t np, const double* __restrict__ shift,
                                                  double coef, int nf, const double* __restrict__ F, const double* __restrict__ Fdd,
                                                  double* __restrict__ out) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= np) return;
  double x[3] = {0, 0, 0};
#pragma unroll
  for (int a = 0; a < D; ++a) x[a] = xyz[p * D + a];
  if (shift) {
#pragma unroll
    for (int a = 0; a < D; ++a) x[a] -= coef * shift[(int64_t)a * np + p];
    clip_in_domain<D>(L, x);
  }
  interpolate_at<D, M>(L, x, nf, F, Fdd, np, p, out);
}

// single-vortex velocity (examples/level_set_advection/main_2d.cpp:116-181) scaled by s; sin(pi x) and
// cos(pi x) come from one sincospi per axis and sin(2 pi x) = 2 sin(pi x) cos(pi x), which halves the FP64
// transcendental work of the reference's six sines (same field to a few ulps)
template <int D>
__device__ __forceinline__ void vortex(const double* x, double s, double* v) {
  double sn[3], cs[3], s2[3];
#pragma unroll
  for (int a = 0; a < D; ++a) {
    sincospi(x[a], &sn[a], &cs[a]);
    s2[a] = 2.0 * sn[a] * cs[a];
  }
  if (D == 3) {
    v[0] = 2.0 * (sn[0] * sn[0]) * s2[1] * s2[2] * s;
    v[1] = -(sn[1] * sn[1]) * s2[0] * s2[2] * s;
    v[2] = -(sn[2] * sn[2]) * s2[0] * s2[1] * s;
  } else {
    v[0] = -(sn[0] * sn[0]) * s2[1] * s;
    v[1] = (sn[1] * sn[1]) * s2[0] * s;
  }
}

template <int D, int M>
__global__ void __launch_bounds__(TPB) k_sl_vortex64(DLoc<D> L, const double* __restrict__ xyz, int64_t np, double dt, double vscale,
                                                     const double* __restrict__ phi, const double* __restrict__ phi_dd,
                                                     double* __restrict__ out) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= np) return;
  double x[3] = {0, 0, 0}, xs[3] = {0, 0, 0}, xd[3] = {0, 0, 0}, v[3];
#pragma unroll
  for (int a = 0; a < D; ++a) x[a] = xyz[p * D + a];
  vortex<D>(x, vscale, v);
#pragma unroll
  for (int a = 0; a < D; ++a) xs[a] = x[a] - st64::scale2(dt, -1) * v[a];
  clip_in_domain<D>(L, xs);
  vortex<D>(xs, vscale, v);
#pragma unroll
  for (int a = 0; a < D; ++a) xd[a] = x[a] - dt * v[a];
  clip_in_domain<D>(L, xd);
  interpolate_at<D, M>(L, xd, 1, phi, phi_dd, np, p, out);
}

// Last round of the two-velocity semi-Lagrangian step (src/my_p4est_semi_lagrangian.cpp:296-314): with
// v_n(x*) and v_nm1(x*) from the previous rounds, v* = ca v_n(x*) - cb v_nm1(x*) (ca = 1 + dt_n/(2 dt_nm1),
// cb = dt_n/(2 dt_nm1), formed by the caller in the reference's order), x_d = x - dt_n v* clipped into the
// domain, and phi_n interpolated at x_d.
template <int D, int M>
__global__ void __launch_bounds__(TPB) k_sl2_phi64(DLoc<D> L, const double* __restrict__ xyz, int64_t np,
                                                   const double* __restrict__ vn_star, const double* __restrict__ vnm1_star, double ca,
                                                   double cb, double dt_n, const double* __restrict__ phi,
                                                   const double* __restrict__ phi_dd, double* __restrict__ out) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= np) return;
  double x[3] = {0, 0, 0};
#pragma unroll
  for (int a = 0; a < D; ++a) {
    const double vs = ca * vn_star[(int64_t)a * np + p] - cb * vnm1_star[(int64_t)a * np + p];
    x[a] = xyz[p * D + a] - dt_n * vs;
  }
  clip_in_domain<D>(L, x);
  interpolate_at<D, M>(L, x, 1, phi, phi_dd, np, p, out);
}

template <int D>
__global__ void __launch_bounds__(TPB) k_locate64(DLoc<D> L, const double* __restrict__ xyz, int64_t np, int32_t* __restrict__ leaf) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= np) return;
  double x[3] = {0, 0, 0};
#pragma unroll
  for (int a = 0; a < D; ++a) x[a] = xyz[p * D + a];
  clip_in_domain<D>(L, x);
  leaf[p] = locate<D>(L, x);
}

// smoothstep(N, x) with its pascalTriangle coefficients (src/my_p4est_utils.cpp:3350-3370)
__device__ double pascal_triangle(int a, int b) {
  double result = 1.;
  for (int i = 0; i < b; ++i) result *= double(a - i) / double(i + 1);
  return result;
}
__device__ double smoothstep(int N, double x) {
  if (x <= 0) return 0;
  if (x >= 1) return 1;
  double result = 0;
  for (int n = 0; n <= N; ++n) result += pascal_triangle(-N - 1, n) * pascal_triangle(2 * N + 1, N - n) * pow(x, (double)(N + n + 1));
  return result;
}

// Set-up of extend_from_interface_to_whole_domain_TVD for one field, one thread per node: the start
// value of q, and along each of the 2D grid directions whose quadratically interpolated phi neighbour
// has the other sign, the subcell distance to the interface (second-order location, at least EPS) and
// qi interpolated there with method M (times 1 - smoothstep(1, (mask - band_zero)/band_smooth) when a
// mask is given, the mask interpolated linearly); elsewhere qi at the node and the grid distance.
// M < 0: the interface values come from the caller's cf function instead (filled in afterwards), q
// starts at zero everywhere and the crossing entries of qi_nb are left at zero.
template <int D, int M>
__global__ void __launch_bounds__(TPB) k_efi_init64(DTab64<D> T, DLoc<D> L, const double* __restrict__ xyz, const double* __restrict__ phi,
                                                    const double* __restrict__ pdd, const double* __restrict__ qi,
                                                    const double* __restrict__ qidd, const double* __restrict__ mask, double dl,
                                                    double band_zero, double band_smooth, double* __restrict__ q,
                                                    double* __restrict__ qi_nb, double* __restrict__ s_nb, uint8_t* __restrict__ cross) {
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t N = T.N;
  if (n >= N) return;
  const double p0 = phi[n];
  if (M < 0)
    q[n] = 0.0;
  else
    q[n] = (mask ? max2(mask[n], fabs(p0)) : fabs(p0)) < 1.5 * dl ? qi[n] : 0;
  double Dp[D];
#pragma unroll
  for (int a = 0; a < D; ++a) Dp[a] = pdd[(int64_t)a * N + n];
  uint8_t bits = 0;
  for (int dir = 0; dir < 2 * D; ++dir) {
    const int a = dir >> 1;
    const double pn = st64::quad_nb64<D>(T, dir, n, phi, Dp);
    const double dd = T.d[(int64_t)dir * N + n];
    if (p0 * pn < 0.0) {
      double dist = st64::interface_location_2nd(0, dd, p0, pn, Dp[a], st64::lin64<D>(T, dir, n, pdd + (int64_t)a * N));
      dist = max2(dist, EPS);
      double v = 0.0;
      if constexpr (M >= 0) {
        double x[3] = {0, 0, 0};
#pragma unroll
        for (int b = 0; b < D; ++b) x[b] = xyz[n * D + b];
        x[a] = (dir & 1) ? x[a] + dist : x[a] - dist;
        interpolate_at<D, M>(L, x, 1, qi, qidd, 1, 0, &v);
        if (mask) {
          double m;
          interpolate_at<D, 0>(L, x, 1, mask, nullptr, 1, 0, &m);
          v *= 1. - smoothstep(1, (m - band_zero) / band_smooth);
        }
      }
      qi_nb[(int64_t)dir * N + n] = v;
      s_nb[(int64_t)dir * N + n] = dist;
      bits |= (uint8_t)(1u << dir);
    } else {
      qi_nb[(int64_t)dir * N + n] = qi[n];
      s_nb[(int64_t)dir * N + n] = dd;
    }
  }
  cross[n] = bits;
}

__global__ void __launch_bounds__(TPB) k_gather_idx64(const double* __restrict__ src, const int64_t* __restrict__ idx, int64_t m,
                                                      double* __restrict__ dst) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < m) dst[i] = src[idx[i]];
}
__global__ void __launch_bounds__(TPB) k_scatter_idx64(const double* __restrict__ src, const int64_t* __restrict__ idx, int64_t m,
                                                       double* __restrict__ dst) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < m) dst[idx[i]] = src[i];
}

}  // namespace

void launch_gather_idx64(const double* src, const int64_t* idx, int64_t m, double* dst, cudaStream_t s) {
  if (m) k_gather_idx64<<<nblocks(m), TPB, 0, s>>>(src, idx, m, dst);
}
void launch_scatter_idx64(const double* src, const int64_t* idx, int64_t m, double* dst, cudaStream_t s) {
  if (m) k_scatter_idx64<<<nblocks(m), TPB, 0, s>>>(src, idx, m, dst);
}

template <int D>
void launch_efi_init64(const DTab64<D>& T, const DLoc<D>& L, int method, const double* xyz, const double* phi, const double* pdd,
                       const double* qi, const double* qidd, const double* mask, double dl, double band_zero, double band_smooth,
                       double* q, double* qi_nb, double* s_nb, uint8_t* cross, cudaStream_t s) {
  if (T.N == 0) return;
  const int64_t g = nblocks(T.N);
#define LSG_EFI(M) k_efi_init64<D, M><<<g, TPB, 0, s>>>(T, L, xyz, phi, pdd, qi, qidd, mask, dl, band_zero, band_smooth, q, qi_nb, s_nb, cross)
  switch (method) {
    case -1: LSG_EFI(-1); break;
    case 0: LSG_EFI(0); break;
    case 1: LSG_EFI(1); break;
    case 2: LSG_EFI(2); break;
    case 3: LSG_EFI(3); break;
    default: LSG_EFI(4); break;
  }
#undef LSG_EFI
}

template <int D>
void launch_interp64(const DLoc<D>& L, int method, const double* xyz, int64_t np, const double* shift, double coef, int nf,
                     const double* F, const double* Fdd, double* out, cudaStream_t s) {
  if (np == 0) return;
  const int64_t g = nblocks(np);
  switch (method) {
    case 0: k_interp64<D, 0><<<g, TPB, 0, s>>>(L, xyz, np, shift, coef, nf, F, Fdd, out); break;
    case 1: k_interp64<D, 1><<<g, TPB, 0, s>>>(L, xyz, np, shift, coef, nf, F, Fdd, out); break;
    case 2: k_interp64<D, 2><<<g, TPB, 0, s>>>(L, xyz, np, shift, coef, nf, F, Fdd, out); break;
    case 3: k_interp64<D, 3><<<g, TPB, 0, s>>>(L, xyz, np, shift, coef, nf, F, Fdd, out); break;
    default: k_interp64<D, 4><<<g, TPB, 0, s>>>(L, xyz, np, shift, coef, nf, F, Fdd, out); break;
  }
}

template <int D>
void launch_sl_vortex64(const DLoc<D>& L, int method, const double* xyz, int64_t np, double dt, double vscale, const double* phi,
                        const double* phi_dd, double* out, cudaStream_t s) {
  if (np == 0) return;
  const int64_t g = nblocks(np);
  switch (method) {
    case 0: k_sl_vortex64<D, 0><<<g, TPB, 0, s>>>(L, xyz, np, dt, vscale, phi, phi_dd, out); break;
    case 1: k_sl_vortex64<D, 1><<<g, TPB, 0, s>>>(L, xyz, np, dt, vscale, phi, phi_dd, out); break;
    case 2: k_sl_vortex64<D, 2><<<g, TPB, 0, s>>>(L, xyz, np, dt, vscale, phi, phi_dd, out); break;
    case 3: k_sl_vortex64<D, 3><<<g, TPB, 0, s>>>(L, xyz, np, dt, vscale, phi, phi_dd, out); break;
    default: k_sl_vortex64<D, 4><<<g, TPB, 0, s>>>(L, xyz, np, dt, vscale, phi, phi_dd, out); break;
  }
}

template <int D>
void launch_sl2_phi64(const DLoc<D>& L, int method, const double* xyz, int64_t np, const double* vn_star, const double* vnm1_star,
                      double ca, double cb, double dt_n, const double* phi, const double* phi_dd, double* out, cudaStream_t s) {
  if (np == 0) return;
  const int64_t g = nblocks(np);
  switch (method) {
    case 0: k_sl2_phi64<D, 0><<<g, TPB, 0, s>>>(L, xyz, np, vn_star, vnm1_star, ca, cb, dt_n, phi, phi_dd, out); break;
    case 1: k_sl2_phi64<D, 1><<<g, TPB, 0, s>>>(L, xyz, np, vn_star, vnm1_star, ca, cb, dt_n, phi, phi_dd, out); break;
    case 2: k_sl2_phi64<D, 2><<<g, TPB, 0, s>>>(L, xyz, np, vn_star, vnm1_star, ca, cb, dt_n, phi, phi_dd, out); break;
    case 3: k_sl2_phi64<D, 3><<<g, TPB, 0, s>>>(L, xyz, np, vn_star, vnm1_star, ca, cb, dt_n, phi, phi_dd, out); break;
    default: k_sl2_phi64<D, 4><<<g, TPB, 0, s>>>(L, xyz, np, vn_star, vnm1_star, ca, cb, dt_n, phi, phi_dd, out); break;
  }
}

template <int D>
void launch_locate64(const DLoc<D>& L, const double* xyz, int64_t np, int32_t* leaf, cudaStream_t s) {
  if (np == 0) return;
  k_locate64<D><<<nblocks(np), TPB, 0, s>>>(L, xyz, np, leaf);
}

#define LSG_INST(D)                                                                                                              \
  template void launch_interp64<D>(const DLoc<D>&, int, const double*, int64_t, const double*, double, int, const double*,     \
                                   const double*, double*, cudaStream_t);                                                      \
  template void launch_sl_vortex64<D>(const DLoc<D>&, int, const double*, int64_t, double, double, const double*, const double*, \
                                      double*, cudaStream_t);                                                                  \
  template void launch_locate64<D>(const DLoc<D>&, const double*, int64_t, int32_t*, cudaStream_t);                              \
  template void launch_sl2_phi64<D>(const DLoc<D>&, int, const double*, int64_t, const double*, const double*, double, double,   \
                                    double, const double*, const double*, double*, cudaStream_t);                               \
  template void launch_efi_init64<D>(const DTab64<D>&, const DLoc<D>&, int, const double*, const double*, const double*,        \
                                     const double*, const double*, const double*, double, double, double, double*, double*,     \
                                     double*, uint8_t*, cudaStream_t);
LSG_INST(2)
LSG_INST(3)
#undef LSG_INST

}  // namespace lsg
