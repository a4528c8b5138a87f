// Shared constants and scalar helpers for the host grid code and the CUDA kernels.
//
// Everything here restates small pieces of parCASL that the level-set path depends on:
//   EPS                     src/casl_math.h:23
//   MINMOD                  src/casl_math.h:80-88
//   two/three-argument MIN  src/casl_math.h:165-175 (the reference undefines the MIN/MAX macros
//                           in src/my_p4est_level_set.cpp:20-21 so the templates below are used)
//   p4est logical units     p4est: P4EST_MAXLEVEL = 30 (2D), P8EST_MAXLEVEL = 19 (3D);
//                           P4EST_ROOT_LEN = 2^MAXLEVEL, P4EST_QUADRANT_LEN(l) = 2^(MAXLEVEL-l)
#pragma once
#include <math.h>
#include <stdint.h>

#if defined(__CUDACC__)
#define LSG_HD __host__ __device__ __forceinline__
#else
#define LSG_HD inline
#endif

namespace lsg {

static constexpr double EPS = 1e-13;  // src/casl_math.h:23

template <int D>
struct Dim {
  static constexpr int MAXLEVEL = (D == 2 ? 30 : 19);
  static constexpr int QMAXLEVEL = MAXLEVEL - 1;
  static constexpr int32_t ROOT_LEN = int32_t(1) << MAXLEVEL;
  static constexpr int CHILDREN = 1 << D;
  static constexpr int FACES = 2 * D;
  static constexpr int HALF = 1 << (D - 1);  // corner nodes on one cell face
};

LSG_HD int32_t quadrant_len(int maxlevel, int level) { return int32_t(1) << (maxlevel - level); }

// src/casl_math.h:80-88
LSG_HD double minmod(double a, double b) {
  if (a * b <= 0) return 0;
  return (fabs(a) < fabs(b)) ? a : b;
}
LSG_HD float minmodf(float a, float b) {
  if (a * b <= 0.0f) return 0.0f;
  return (fabsf(a) < fabsf(b)) ? a : b;
}
// src/casl_math.h:165-186 (argument order matters only for NaN handling, kept as in the reference)
template <typename T>
LSG_HD T min2(T a, T b) { return a < b ? a : b; }
template <typename T>
LSG_HD T min3(T a, T b, T c) { return a < b ? min2(a, c) : min2(b, c); }
template <typename T>
LSG_HD T max2(T a, T b) { return b < a ? a : b; }
template <typename T>
LSG_HD T max3(T a, T b, T c) { return b < a ? max2(a, c) : max2(b, c); }

// Spread the low bits of v so that consecutive bits land D positions apart (Morton interleave).
LSG_HD uint64_t spread2(uint64_t v) {
  v &= 0xFFFFFFFFull;
  v = (v | (v << 16)) & 0x0000FFFF0000FFFFull;
  v = (v | (v << 8)) & 0x00FF00FF00FF00FFull;
  v = (v | (v << 4)) & 0x0F0F0F0F0F0F0F0Full;
  v = (v | (v << 2)) & 0x3333333333333333ull;
  v = (v | (v << 1)) & 0x5555555555555555ull;
  return v;
}
LSG_HD uint64_t spread3(uint64_t v) {
  v &= 0x1FFFFFull;
  v = (v | (v << 32)) & 0x1F00000000FFFFull;
  v = (v | (v << 16)) & 0x1F0000FF0000FFull;
  v = (v | (v << 8)) & 0x100F00F00F00F00Full;
  v = (v | (v << 4)) & 0x10C30C30C30C30C3ull;
  v = (v | (v << 2)) & 0x1249249249249249ull;
  return v;
}
// Inverse of spread2 / spread3: gather every D-th bit.
LSG_HD uint32_t compact2(uint64_t v) {
  v &= 0x5555555555555555ull;
  v = (v | (v >> 1)) & 0x3333333333333333ull;
  v = (v | (v >> 2)) & 0x0F0F0F0F0F0F0F0Full;
  v = (v | (v >> 4)) & 0x00FF00FF00FF00FFull;
  v = (v | (v >> 8)) & 0x0000FFFF0000FFFFull;
  v = (v | (v >> 16)) & 0x00000000FFFFFFFFull;
  return (uint32_t)v;
}
LSG_HD uint32_t compact3(uint64_t v) {
  v &= 0x1249249249249249ull;
  v = (v | (v >> 2)) & 0x10C30C30C30C30C3ull;
  v = (v | (v >> 4)) & 0x100F00F00F00F00Full;
  v = (v | (v >> 8)) & 0x1F0000FF0000FFull;
  v = (v | (v >> 16)) & 0x1F00000000FFFFull;
  v = (v | (v >> 32)) & 0x1FFFFFull;
  return (uint32_t)v;
}
// Morton index of logical coordinates (x fastest), p4est linear order within one tree.
template <int D>
LSG_HD uint64_t morton(const int32_t* xyz) {
  if (D == 2) return spread2((uint64_t)xyz[0]) | (spread2((uint64_t)xyz[1]) << 1);
  return spread3((uint64_t)xyz[0]) | (spread3((uint64_t)xyz[1]) << 1) | (spread3((uint64_t)xyz[2]) << 2);
}
template <int D>
LSG_HD void unmorton(uint64_t m, int32_t* xyz) {
  if (D == 2) {
    xyz[0] = (int32_t)compact2(m);
    xyz[1] = (int32_t)compact2(m >> 1);
  } else {
    xyz[0] = (int32_t)compact3(m);
    xyz[1] = (int32_t)compact3(m >> 1);
    xyz[2] = (int32_t)compact3(m >> 2);
  }
}
// Tree index goes above the Morton bits: (tree, morton) lexicographic order as p4est sorts
// quadrants and nodes (src/my_p4est_nodes.c:606-627).
template <int D>
LSG_HD int tree_shift() { return D * Dim<D>::MAXLEVEL; }
template <int D>
LSG_HD int max_trees_for_keys() { return 1 << (63 - D * Dim<D>::MAXLEVEL); }

}  // namespace lsg
