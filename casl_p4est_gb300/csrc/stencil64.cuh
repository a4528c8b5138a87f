// FP64 stencil helpers shared by the FP64 kernels and the FP64 subcell step of the mixed path.
// Each function restates one reference routine with the reference's expression order; the FP64
// translation unit is compiled with -fmad=false, which makes its results bit-identical to the
// reference's double arithmetic.
//   lin64            interpolate_linearly          src/my_p4est_quad_neighbor_nodes_of_node.h:290-306
//   correct64        correct_naive_second_derivatives  src/my_p4est_quad_neighbor_nodes_of_node.cpp:44-298
//   laplace64        laplace                       .h:615-635 (central_second_derivative .h:214-220)
//   quad_nb64        ngbd_with_quadratic_interpolation .h:1514-1545
//   interface_location[_2nd]                       src/casl_math.cpp:55-97
#pragma once
#include "kernels.h"
#include "tables.hpp"

namespace lsg {
namespace st64 {

// Comparisons of doubles decided on their bit patterns where that gives the IEEE answer for every input (other
// inputs take the FP64 comparison). GB300 issues FP64 instructions, compares included, at 2 per SM cycle and
// integer ones at 64, so these keep the FP64 pipe for arithmetic.
constexpr unsigned long long kMag = 0x7fffffffffffffffull, kInf = 0x7ff0000000000000ull;
__device__ __forceinline__ unsigned long long bits_of(double v) { return (unsigned long long)__double_as_longlong(v); }
// The FP64 fallbacks of the helpers below are functions that are never inlined: inlined, the compiler may evaluate
// a fallback on every lane and select its result (if-conversion), which puts its FP64 instructions on the pipe for
// inputs that never need them. A call is taken only by the lanes whose inputs need it.
static __device__ __noinline__ bool less_fp64(double a, double b) { return a < b; }
static __device__ __noinline__ bool product_negative_fp64(double a, double b) { return a * b < 0.0; }
static __device__ __noinline__ double mul_fp64(double a, double b) { return __dmul_rn(a, b); }
static __device__ __noinline__ double minmod_fp64(double a, double b) { return minmod(a, b); }
// +0 .. +inf (no sign bit, not NaN): for these the integer order of the bit patterns is the numeric order
__device__ __forceinline__ bool nonneg_num(unsigned long long b) { return b <= kInf; }
__device__ __forceinline__ bool is_zero(double v) { return (bits_of(v) & kMag) < bits_of(EPS); }  // fabs(v) < EPS, check_if_zero .h:186
__device__ __forceinline__ bool nonzero(double v) { return (bits_of(v) << 1) != 0; }             // v != 0.0 (NaN included)
__device__ __forceinline__ bool positive(double v) { return bits_of(v) - 1ull < kInf; }          // v > 0.0
__device__ __forceinline__ bool negative(double v) {                                              // v < 0.0
  const unsigned long long b = bits_of(v);
  return (b >> 63) && (b & kMag) - 1ull < kInf;
}
// max2 (src/casl_math.h: b < a ? a : b) and min2 / min3 (a < b ? ...), the same result for every input
__device__ __forceinline__ bool less64(double a, double b) {
  const unsigned long long ia = bits_of(a), ib = bits_of(b);
  if (nonneg_num(ia) && nonneg_num(ib)) return ia < ib;
  return less_fp64(a, b);
}
__device__ __forceinline__ double max2x(double a, double b) { return less64(b, a) ? a : b; }
__device__ __forceinline__ double min2x(double a, double b) { return less64(a, b) ? a : b; }
__device__ __forceinline__ double min3x(double a, double b, double c) { return less64(a, b) ? min2x(a, c) : min2x(b, c); }
// MINMOD (src/casl_math.h:80-88: a b <= 0 ? 0 : (|a| < |b| ? a : b)). Both finite with opposite signs: the
// product is <= 0. Same signs, both normal and ea + eb >= 972: |a b| >= 2^(ea+eb-2046) >= 2^-1074, so the
// product is > 0 and the magnitudes order as their bit patterns. Anything else is decided in FP64.
__device__ __forceinline__ double minmod_x(double a, double b) {
  const unsigned long long ia = bits_of(a), ib = bits_of(b);
  const unsigned ea = (unsigned)(ia >> 52) & 0x7ffu, eb = (unsigned)(ib >> 52) & 0x7ffu;
  if (ea != 0x7ffu && eb != 0x7ffu) {
    if ((ia ^ ib) >> 63) return 0.0;
    if (ea > 0 && eb > 0 && ea + eb >= 972u) return (ia & kMag) < (ib & kMag) ? a : b;
  }
  return minmod_fp64(a, b);
}
// a * b < 0.0 with IEEE double semantics, decided from the bit patterns where that is exact: opposite
// sign bits, both finite and normal, and exponents large enough that the product cannot round to
// zero (|a b| >= 2^(ea+eb-2046) >= 2^-1074); same signs without NaN give a b >= 0; every other case takes
// the FP64 product.
__device__ __forceinline__ bool product_negative(double a, double b) {
  const long long ia = __double_as_longlong(a), ib = __double_as_longlong(b);
  if ((ia ^ ib) >= 0) {
    if (((ia >> 52) & 0x7ff) != 0x7ff && ((ib >> 52) & 0x7ff) != 0x7ff) return false;  // same signs, no NaN: a b >= 0
    return product_negative_fp64(a, b);
  }
  const int ea = (int)((ia >> 52) & 0x7ff), eb = (int)((ib >> 52) & 0x7ff);
  if (ea > 0 && eb > 0 && ea < 0x7ff && eb < 0x7ff && ea + eb >= 972) return true;
  return product_negative_fp64(a, b);
}

// x / y, bit for bit. When y is a normal power of two whose reciprocal 1/y is normal too (octree cell
// sizes and their sums of equal halves are, for power-of-two tree sizes), x * (1/y) is exactly the real
// number x / y, and IEEE multiplication and division round that same number the same way (subnormal,
// infinite and zero results included), so one multiplication replaces the division sequence; GB300
// issues FP64 at 2 operations per SM cycle, where a division takes about ten. Any other y is divided.
// When x and the quotient are normal numbers the quotient is exact, and it is x's bit pattern with the exponent
// field moved by e - 1023 and the sign bit of y added: integer work, no FP64 instruction at all.
__device__ __forceinline__ double qdiv(double x, double y) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(y);
  const unsigned e = (unsigned)(b >> 52) & 0x7ffu;  // biased exponent
  if ((b & 0x000fffffffffffffull) == 0 && e - 1u < 2045u) {  // mantissa zero, e in [1, 2045]: 1/y = 2^(1023 - (e - 1023))
    const unsigned long long bx = bits_of(x) ^ (b & 0x8000000000000000ull);
    const int ex = (int)((bx >> 52) & 0x7ffu), r = ex + 1023 - (int)e;
    if (ex >= 1 && ex <= 2046 && r >= 1 && r <= 2046)
      return __longlong_as_double((long long)(bx - ((unsigned long long)e << 52) + (1023ull << 52)));
    return mul_fp64(x, __longlong_as_double((long long)((b & 0x8000000000000000ull) | ((unsigned long long)(2046u - e) << 52))));
  }
  return x / y;
}

// x * 2^k (k in [-1022, 1023]), bit for bit: when x and the product are normal the product is exact and is x with
// k added to its exponent field (integer work); zeros, subnormals, infinities, NaN and products outside the normal
// range take the FP64 multiplication by 2^k. scale2(x, -1) is 0.5 * x and scale2(x, 1) is x * 2.
__device__ __forceinline__ double scale2(double x, int k) {
  const unsigned long long b = bits_of(x);
  const int e = (int)((b >> 52) & 0x7ffu), r = e + k;
  if (e >= 1 && e <= 2046 && r >= 1 && r <= 2046) return __longlong_as_double((long long)(b + ((unsigned long long)(long long)k << 52)));
  return mul_fp64(x, __longlong_as_double((long long)(1023 + k) << 52));
}

// x * -1.0 bit for bit: the sign bit flipped; a NaN is multiplied
__device__ __forceinline__ double neg1(double x) {
  const unsigned long long b = bits_of(x);
  if ((b & kMag) > kInf) return mul_fp64(x, -1.0);
  return __longlong_as_double((long long)(b ^ 0x8000000000000000ull));
}
// x * (pos ? 1.0 : -1.0) bit for bit
__device__ __forceinline__ double times_sign(double x, bool pos) {
  const unsigned long long b = bits_of(x);
  if ((b & kMag) > kInf) return mul_fp64(x, pos ? 1.0 : -1.0);
  return pos ? x : __longlong_as_double((long long)(b ^ 0x8000000000000000ull));
}

// x / 3 (the local pseudo-time step min(s) / P4EST_DIM of a 3D node), bit for bit. When x = +-2^k with x and
// x/3 in the normal range, RN(x/3) = x * RN(1/3): scaling by a power of two commutes with rounding, so one
// multiplication by the double nearest 1/3 (0x3FD5555555555555) replaces the division; any other x is divided.
__device__ __forceinline__ double div3(double x) {
  const unsigned long long b = bits_of(x);
  const unsigned e = (unsigned)(b >> 52) & 0x7ffu;
  if ((b & 0x000fffffffffffffull) == 0 && e > 2u && e < 2047u) return __dmul_rn(x, __longlong_as_double(0x3FD5555555555555ll));
  return x / 3.0;
}

// (f w) / nrm with one face node and nrm == w == 2^k, bit for bit: it is f itself whenever f w is a normal
// number (then f w and the division by 2^k are exact). The test is integer work on the bit patterns; a face
// node that coincides with the neighbour position (every regular direction on power-of-two trees) then costs
// no FP64 operation. Any other case takes the reference's arithmetic.
__device__ __forceinline__ bool unit_weight_exact(double f, double w, double nrm) {
  const unsigned long long bw = bits_of(w), bf = bits_of(f);
  const int ew = (int)(bw >> 52);  // w > 0: no sign bit
  const int ef = (int)((bf >> 52) & 0x7ffu);
  const int e = ef + ew - 1023;  // biased exponent of f w
  return bw == bits_of(nrm) && (bw & 0x000fffffffffffffull) == 0 && ew >= 1 && ew <= 2045 && ef >= 1 && ef <= 2046 && e >= 1 &&
         e <= 2046;
}

template <int D>
__device__ __forceinline__ double lin64(const DTab64<D>& T, int dir, int64_t n, const double* __restrict__ f) {
  constexpr int H = Dim<D>::HALF;
  const int64_t N = T.N;
  const int64_t base = (int64_t)(dir * H) * N + n;
  const double f0 = f[T.nbr[base]], w0 = T.w[base], nrm = T.nrm[(int64_t)dir * N + n];
  int32_t ik[H];
  bool single = true;
#pragma unroll
  for (int k = 1; k < H; ++k) {
    ik[k] = T.nbr[base + k * N];
    single = single && ik[k] < 0;
  }
  if (single && unit_weight_exact(f0, w0, nrm)) return f0;
  double acc = f0 * w0;
#pragma unroll
  for (int k = 1; k < H; ++k)
    if (ik[k] >= 0) acc = acc + f[ik[k]] * T.w[base + k * N];
  return qdiv(acc, nrm);
}

// The node's pattern word (DTab64::word) when the tables carry one: which faces have one face node of unit
// weight and which need no tangential correction, so those faces load one index and one value instead of the
// H indices, the weight, the norm and the two correction factors.
struct NodeWord {
  uint32_t w;
  bool known;
};
template <int D>
__device__ __forceinline__ NodeWord node_word(const DTab64<D>& T, int64_t n) {
  return NodeWord{T.word ? __ldg(T.word + n) : 0u, T.word != nullptr};
}
// lin64 with the pattern word: a single face node of unit weight gives its value itself when that value's exponent
// keeps f w normal for every weight in [2^-400, 2^400] (|f| in [2^-622, 2^622]); anything else takes lin64
template <int D>
__device__ __forceinline__ double lin64w(const DTab64<D>& T, int dir, int64_t n, const double* __restrict__ f, NodeWord nw) {
  constexpr int H = Dim<D>::HALF;
  if (nw.known && ((nw.w >> (2 * dir)) & 3u) == 0 && ((nw.w >> (20 + dir)) & 1u)) {
    const double f0 = f[T.nbr[(int64_t)(dir * H) * T.N + n]];
    const int ef = (int)((bits_of(f0) >> 52) & 0x7ffu);
    if (ef >= 401 && ef <= 1645) return f0;
  }
  return lin64<D>(T, dir, n, f);
}

// correct_naive_second_derivatives (src/my_p4est_quad_neighbor_nodes_of_node.cpp:44-298), all branches.
template <int D>
__device__ void correct64(const double* __restrict__ m, double* Dv) {
  if (D == 2) {
    const double m12 = m[CM12], m21 = m[CM21];
    if (is_zero(m12)) {
      if (!is_zero(m21)) Dv[1] = Dv[1] - m21 * Dv[0];
    } else if (is_zero(m21)) {
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
  double& Dxx = Dv[0];
  double& Dyy = Dv[1];
  double& Dzz = Dv[2 % D];
  if (is_zero(m12) && is_zero(m13)) {
    if (is_zero(m23)) {
      const bool m21nz = !is_zero(m21), m31nz = !is_zero(m31), m32nz = !is_zero(m32);
      if (m21nz) Dyy = Dyy - m21 * Dxx;
      if (m31nz) Dzz = Dzz - m31 * Dxx;
      if (m32nz) Dzz = Dzz - m32 * Dyy;
    } else if (is_zero(m32)) {
      const bool m21nz = !is_zero(m21), m31nz = !is_zero(m31);
      if (m31nz) Dzz = Dzz - m31 * Dxx;
      Dyy = Dyy - m23 * Dzz;
      if (m21nz) Dyy = Dyy - m21 * Dxx;
    } else {
      const double idet = 1.0 / (1.0 - m23 * m32);
      const bool m21z = is_zero(m21), m31z = is_zero(m31);
      const double nDyy = Dyy, nDzz = Dzz;
      Dyy = ((m21z ? nDyy : (nDyy - m21 * Dxx)) - m23 * (m31z ? nDzz : (nDzz - m31 * Dxx))) * idet;
      Dzz = ((m31z ? nDzz : (nDzz - m31 * Dxx)) - m32 * (m21z ? nDyy : (nDyy - m21 * Dxx))) * idet;
    }
  } else if (is_zero(m21) && is_zero(m23)) {
    if (is_zero(m13)) {
      const bool m12nz = !is_zero(m12), m31nz = !is_zero(m31), m32nz = !is_zero(m32);
      if (m12nz) Dxx = Dxx - m12 * Dyy;
      if (m31nz) Dzz = Dzz - m31 * Dxx;
      if (m32nz) Dzz = Dzz - m32 * Dyy;
    } else if (is_zero(m31)) {
      const bool m12nz = !is_zero(m12), m32nz = !is_zero(m32);
      if (m32nz) Dzz = Dzz - m32 * Dyy;
      Dxx = Dxx - m13 * Dzz;
      if (m12nz) Dxx = Dxx - m12 * Dyy;
    } else {
      const double idet = 1.0 / (1.0 - m13 * m31);
      const bool m12z = is_zero(m12), m32z = is_zero(m32);
      const double nDxx = Dxx, nDzz = Dzz;
      Dxx = ((m12z ? nDxx : (nDxx - m12 * Dyy)) - m13 * (m32z ? nDzz : (nDzz - m32 * Dyy))) * idet;
      Dzz = ((m32z ? nDzz : (nDzz - m32 * Dyy)) - m31 * (m12z ? nDxx : (nDxx - m12 * Dyy))) * idet;
    }
  } else if (is_zero(m31) && is_zero(m32)) {
    if (is_zero(m12)) {
      const bool m13nz = !is_zero(m13), m21nz = !is_zero(m21), m23nz = !is_zero(m23);
      if (m13nz) Dxx = Dxx - m13 * Dzz;
      if (m21nz) Dyy = Dyy - m21 * Dxx;
      if (m23nz) Dyy = Dyy - m23 * Dzz;
    } else if (is_zero(m21)) {
      const bool m13nz = !is_zero(m13), m23nz = !is_zero(m23);
      if (m23nz) Dyy = Dyy - m23 * Dzz;
      Dxx = Dxx - m12 * Dyy;
      if (m13nz) Dxx = Dxx - m13 * Dzz;
    } else {
      const double idet = 1.0 / (1.0 - m12 * m21);
      const bool m13z = is_zero(m13), m23z = is_zero(m23);
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

// laplace(): virtual neighbours by linear interpolation, naive central second derivatives
// ((fp-f0)/dp + (fm-f0)/dm)*2/(dp+dm), then the cross-term correction.
template <int D>
__device__ __forceinline__ void laplace64(const DTab64<D>& T, int64_t n, const double* __restrict__ f, double* Dv) {
  const int64_t N = T.N;
  const double f0 = f[n];
  const NodeWord nw = node_word<D>(T, n);
#pragma unroll
  for (int a = 0; a < D; ++a) {
    const double fm = lin64w<D>(T, 2 * a, n, f, nw);
    const double fp = lin64w<D>(T, 2 * a + 1, n, f, nw);
    const double dm = T.d[(int64_t)(2 * a) * N + n], dp = T.d[(int64_t)(2 * a + 1) * N + n];
    Dv[a] = qdiv(scale2(qdiv(fp - f0, dp) + qdiv(fm - f0, dm), 1), dp + dm);
  }
  if (nw.known && !((nw.w >> 12) & 1u)) return;  // no correction record
  const int32_t ci = T.cidx[n];
  if (ci >= 0) correct64<D>(T.crec + (int64_t)6 * ci, Dv);
}

// Tangential axes of the neighbour direction along `axis` (x: y,z; y: x,z; z: x,y).
__device__ __forceinline__ int tan_axis(int axis, int j) {
  return j == 0 ? (axis == 0 ? 1 : 0) : (axis == 2 ? 1 : 2);
}

// ngbd_with_quadratic_interpolation: f_dir -= (0.5 d_m0 d_p0 f_t1t1 [+ 0.5 d_0m d_0p f_t2t2]).
template <int D>
__device__ __forceinline__ double quad_nb64(const DTab64<D>& T, int dir, int64_t n, const double* __restrict__ f, const double* Dv,
                                           NodeWord nw = NodeWord{0u, false}) {
  const int64_t N = T.N;
  double v = lin64w<D>(T, dir, n, f, nw);
  if (nw.known && ((nw.w >> (26 + dir)) & 1u)) return v;  // both correction factors zero
  const int axis = dir >> 1;
  if (D == 2) {
    const double q0 = T.q[(int64_t)dir * N + n];
    if (nonzero(q0)) v = v - q0 * Dv[tan_axis(axis, 0)];
  } else {
    const double q0 = T.q[(int64_t)(2 * dir) * N + n], q1 = T.q[(int64_t)(2 * dir + 1) * N + n];
    if (nonzero(q0) || nonzero(q1)) v = v - (q0 * Dv[tan_axis(axis, 0)] + q1 * Dv[tan_axis(axis, 1 % (D - 1))]);
  }
  return v;
}

__device__ __forceinline__ double interface_location(double a, double b, double fa, double fb) {
  return scale2(a + b + (a - b) * (fa + fb) / (fb - fa), -1);
}

__device__ inline double interface_location_2nd(double a, double b, double fa, double fb, double fxxa, double fxxb) {
  if (fabs(fa) < EPS) return a + EPS;
  if (fabs(fb) < EPS) return b - EPS;
  const double fxx = minmod(fxxa, fxxb);
  const double h = b - a;
  const double c2 = scale2(fxx, -1);
  const double c1 = qdiv(fb - fa, h);
  const double c0 = scale2(fb + fa, -1) - qdiv(h * h, 8.0) * fxx;
  double x;
  if (fabs(c2) < EPS)
    x = -c0 / c1;
  else {
    if (fb < 0)
      x = neg1(scale2(c0, 1)) / (c1 - sqrt(c1 * c1 - scale2(c2, 2) * c0));
    else
      x = neg1(scale2(c0, 1)) / (c1 + sqrt(c1 * c1 - scale2(c2, 2) * c0));
  }
  return x + scale2(a + b, -1);
}


}  // namespace st64
}  // namespace lsg
