// Checks, on the GPU, that the FP64 helpers of stencil64.cuh give the same double as the plain FP64 operation they
// replace, for ordinary and edge-case operands: zeros, subnormals, the ends of the normal range, infinities, NaN,
// powers of two over the whole exponent range and random values. A NaN result is compared as "NaN" (its payload is
// not part of the claim). Built with -fmad=false, like the FP64 kernels. Prints "fp64 helpers ok" on success.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

#include "stencil64.cuh"

using namespace lsg;
using namespace lsg::st64;

enum { Q_DIV, Q_SCALE_M1, Q_SCALE_P1, Q_SCALE_P2, Q_NEG, Q_SIGN_P, Q_SIGN_N, Q_PNEG, Q_LESS, Q_MAX, Q_MIN, Q_MINMOD, Q_UNIT, Q_DIV3, NQ };
static const char* kNames[NQ] = {"qdiv", "scale2(-1)", "scale2(1)", "scale2(2)", "neg1", "times_sign(+)", "times_sign(-)",
                                 "product_negative", "less64", "max2x", "min2x", "minmod_x", "unit_weight_exact", "div3"};

__device__ bool same(double a, double b) {
  if (a != a && b != b) return true;  // both NaN
  return __double_as_longlong(a) == __double_as_longlong(b);
}

__global__ void k_check(const double* x, const double* y, int64_t n, unsigned long long* bad, long long* first_bad) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double a = x[i], b = y[i];
  bool ok[NQ];
  ok[Q_DIV] = same(qdiv(a, b), a / b);
  ok[Q_SCALE_M1] = same(scale2(a, -1), 0.5 * a);
  ok[Q_SCALE_P1] = same(scale2(a, 1), a * 2.0);
  ok[Q_SCALE_P2] = same(scale2(a, 2), 4.0 * a);
  ok[Q_NEG] = same(neg1(a), a * -1.0);
  ok[Q_SIGN_P] = same(times_sign(a, true), a * 1.0);
  ok[Q_SIGN_N] = same(times_sign(a, false), a * -1.0);
  ok[Q_PNEG] = product_negative(a, b) == (a * b < 0.0);
  ok[Q_LESS] = less64(a, b) == (a < b);
  ok[Q_MAX] = same(max2x(a, b), max2(a, b));
  ok[Q_MIN] = same(min2x(a, b), min2(a, b));
  ok[Q_MINMOD] = same(minmod_x(a, b), minmod(a, b));
  // the unit-weight shortcut: when it applies, (f w) / w is f itself
  ok[Q_UNIT] = !unit_weight_exact(a, b, b) || same(qdiv(a * b, b), a);
  ok[Q_DIV3] = same(div3(a), a / 3.0);
  for (int q = 0; q < NQ; ++q)
    if (!ok[q]) {
      atomicAdd(bad + q, 1ull);
      atomicCAS((unsigned long long*)(first_bad + q), (unsigned long long)-1ll, (unsigned long long)i);
    }
}

int main() {
  std::vector<double> special = {0.0, -0.0, 1.0, -1.0, 0.5, 3.0, -7.25, 1e-300, -1e-300, 1e300, -1e300};
  const double inf = INFINITY;
  special.push_back(inf);
  special.push_back(-inf);
  special.push_back(std::nan(""));
  special.push_back(-std::nan(""));
  for (int e = -1074; e <= 1023; e += 1) {  // every power of two, normal and subnormal, both signs
    special.push_back(std::ldexp(1.0, e));
    special.push_back(-std::ldexp(1.0, e));
  }
  special.push_back(std::nextafter(0.0, 1.0));
  special.push_back(std::nextafter(std::ldexp(1.0, -1022), 0.0));  // largest subnormal
  special.push_back(1.7976931348623157e308);
  special.push_back(-1.7976931348623157e308);
  std::mt19937_64 rng(17);
  std::uniform_real_distribution<double> mant(1.0, 2.0);
  std::uniform_int_distribution<int> ex(-1080, 1030);
  std::vector<double> rnd;
  for (int k = 0; k < 6000; ++k) {
    double v = std::ldexp(mant(rng), ex(rng));
    if (k & 1) v = -v;
    rnd.push_back(v);
  }
  // pairs: every special with every special, and random values against specials and against each other
  std::vector<double> xs, ys;
  for (double a : special)
    for (double b : special) {
      xs.push_back(a);
      ys.push_back(b);
    }
  for (size_t k = 0; k < rnd.size(); ++k) {
    for (int j = 0; j < 24; ++j) {
      xs.push_back(rnd[k]);
      ys.push_back(special[(k * 131 + j * 977) % special.size()]);
      xs.push_back(special[(k * 71 + j * 613) % special.size()]);
      ys.push_back(rnd[k]);
    }
    xs.push_back(rnd[k]);
    ys.push_back(rnd[(k * 7 + 3) % rnd.size()]);
  }
  const int64_t n = (int64_t)xs.size();
  double *dx = nullptr, *dy = nullptr;
  unsigned long long* dbad = nullptr;
  long long* dfirst = nullptr;
  if (cudaMalloc(&dx, n * sizeof(double)) != cudaSuccess || cudaMalloc(&dy, n * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&dbad, NQ * sizeof(unsigned long long)) != cudaSuccess || cudaMalloc(&dfirst, NQ * sizeof(long long)) != cudaSuccess) {
    std::printf("allocation failed\n");
    return 2;
  }
  cudaMemcpy(dx, xs.data(), n * sizeof(double), cudaMemcpyHostToDevice);
  cudaMemcpy(dy, ys.data(), n * sizeof(double), cudaMemcpyHostToDevice);
  cudaMemset(dbad, 0, NQ * sizeof(unsigned long long));
  cudaMemset(dfirst, 0xff, NQ * sizeof(long long));
  k_check<<<(unsigned)((n + 255) / 256), 256>>>(dx, dy, n, dbad, dfirst);
  if (cudaDeviceSynchronize() != cudaSuccess) {
    std::printf("kernel failed: %s\n", cudaGetErrorString(cudaGetLastError()));
    return 2;
  }
  unsigned long long bad[NQ];
  long long first[NQ];
  cudaMemcpy(bad, dbad, sizeof(bad), cudaMemcpyDeviceToHost);
  cudaMemcpy(first, dfirst, sizeof(first), cudaMemcpyDeviceToHost);
  int fails = 0;
  for (int q = 0; q < NQ; ++q)
    if (bad[q]) {
      ++fails;
      const long long i = first[q];
      std::printf("%s: %llu mismatches, first at x=%.17g y=%.17g\n", kNames[q], bad[q], i >= 0 ? xs[i] : 0.0, i >= 0 ? ys[i] : 0.0);
    }
  std::printf("%lld pairs checked\n", (long long)n);
  if (fails) return 1;
  std::printf("fp64 helpers ok\n");
  return 0;
}
