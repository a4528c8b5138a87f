// Analytic level-set functions used to build and seed the benchmark grids (the workloads' phi_exact
// and phi0, sampled like sample_cf_on_nodes and refined like refine_levelset_cf). Host-only, plain
// double arithmetic; each shape is a kind plus a flat parameter list.
//
//   LSG_SHAPE_SPHERE            |x - c| - r                                   params: c[3], r
//   LSG_SHAPE_SPHERE_SCALED     (|x - c| - r) * (a + |x - p|^2)               params: c[3], r, a, p[3]
//   LSG_SHAPE_FLOWER            r - (r0 + amp sin(kt*theta) sin(kp*phi))     params: c[3], r0, amp, kt, kp,
//                               (theta = atan2(y,x), phi = acos(z/r) in 3D;   a, p[3], scaled (0/1)
//                               2D: r - (r0 + amp sin(kt*theta))), optionally times (a + |x - p|^2)
//   LSG_SHAPE_SPHERES           min_i (|x - c_i| - r_i), optionally scaled    params: n, a, p[3], scaled,
//                                                                             then n x (c[3], r)
//   LSG_SHAPE_ELLIPSES          (2D) min_i signed distance to ellipse i,      params: n, a, p[2], s, scaled,
//                               optionally times (a + s*|x - p|^2)            then n x (cx, cy, ax, ay, angle)
#pragma once
#include <math.h>

namespace lsg {

enum {
  LSG_SHAPE_SPHERE = 0,
  LSG_SHAPE_SPHERE_SCALED = 1,
  LSG_SHAPE_FLOWER = 2,
  LSG_SHAPE_SPHERES = 3,
  LSG_SHAPE_ELLIPSES = 4,
};

// Signed distance from (x, y) to the axis-aligned ellipse x^2/a^2 + y^2/b^2 = 1 (negative inside),
// by bisection on the parameter of the closest point (Eberly, "Distance from a point to an ellipse").
inline double ellipse_signed_distance(double px, double py, double a, double b) {
  const double x = fabs(px), y = fabs(py);
  const bool swap = a < b;
  double e0 = swap ? b : a, e1 = swap ? a : b;
  double y0 = swap ? y : x, y1 = swap ? x : y;  // y0 along the major axis
  const double inside = (y0 * y0) / (e0 * e0) + (y1 * y1) / (e1 * e1) - 1.0;
  double dist;
  if (y1 > 0) {
    if (y0 > 0) {
      const double z0 = y0 / e0, z1 = y1 / e1;
      const double r0 = (e0 / e1) * (e0 / e1);
      const double g = z0 * z0 + z1 * z1 - 1.0;
      if (g != 0) {
        double n0 = r0 * z0;
        double s0 = z1 - 1.0, s1 = (g < 0 ? 0.0 : sqrt(n0 * n0 + z1 * z1) - 1.0), s = 0;
        for (int i = 0; i < 200; ++i) {
          s = 0.5 * (s0 + s1);
          if (s == s0 || s == s1) break;
          const double ratio0 = n0 / (s + r0), ratio1 = z1 / (s + 1.0);
          const double gg = ratio0 * ratio0 + ratio1 * ratio1 - 1.0;
          if (gg > 0) s0 = s;
          else if (gg < 0) s1 = s;
          else break;
        }
        const double x0 = r0 * y0 / (s + r0), x1 = y1 / (s + 1.0);
        dist = sqrt((x0 - y0) * (x0 - y0) + (x1 - y1) * (x1 - y1));
      } else {
        dist = 0.0;
      }
    } else {
      dist = fabs(y1 - e1);
    }
  } else {
    const double numer0 = e0 * y0, denom0 = e0 * e0 - e1 * e1;
    if (numer0 < denom0) {
      const double xde0 = numer0 / denom0;
      const double x0 = e0 * xde0, x1 = e1 * sqrt(fmax(0.0, 1.0 - xde0 * xde0));
      dist = sqrt((x0 - y0) * (x0 - y0) + x1 * x1);
    } else {
      dist = fabs(y0 - e0);
    }
  }
  return inside < 0 ? -dist : dist;
}

template <int D>
inline double shape_eval(int kind, const double* p, const double* x) {
  auto sq = [](double v) { return v * v; };
  switch (kind) {
    case LSG_SHAPE_SPHERE: {
      double r2 = 0;
      for (int a = 0; a < D; ++a) r2 += sq(x[a] - p[a]);
      return sqrt(r2) - p[3];
    }
    case LSG_SHAPE_SPHERE_SCALED: {
      double r2 = 0, s2 = 0;
      for (int a = 0; a < D; ++a) {
        r2 += sq(x[a] - p[a]);
        s2 += sq(x[a] - p[5 + a]);
      }
      return (sqrt(r2) - p[3]) * (p[4] + s2);
    }
    case LSG_SHAPE_FLOWER: {
      double rel[3] = {0, 0, 0}, r2 = 0;
      for (int a = 0; a < D; ++a) {
        rel[a] = x[a] - p[a];
        r2 += rel[a] * rel[a];
      }
      const double r = sqrt(r2);
      const double theta = atan2(rel[1], rel[0]);
      double rs;
      if (D == 3) {
        const double phi = (r > 0) ? acos(fmax(-1.0, fmin(1.0, rel[2] / r))) : 0.0;
        rs = p[3] + p[4] * sin(p[5] * theta) * sin(p[6] * phi);
      } else {
        rs = p[3] + p[4] * sin(p[5] * theta);
      }
      double v = r - rs;
      if (p[11] != 0) {
        double s2 = 0;
        for (int a = 0; a < D; ++a) s2 += sq(x[a] - p[8 + a]);
        v *= (p[7] + s2);
      }
      return v;
    }
    case LSG_SHAPE_SPHERES: {
      const int n = (int)p[0];
      double best = 1e300;
      for (int i = 0; i < n; ++i) {
        const double* s = p + 6 + 4 * i;
        double r2 = 0;
        for (int a = 0; a < D; ++a) r2 += sq(x[a] - s[a]);
        const double v = sqrt(r2) - s[3];
        if (v < best) best = v;
      }
      if (p[5] != 0) {
        double s2 = 0;
        for (int a = 0; a < D; ++a) s2 += sq(x[a] - p[2 + a]);
        best *= (p[1] + s2);
      }
      return best;
    }
    case LSG_SHAPE_ELLIPSES: {
      const int n = (int)p[0];
      double best = 1e300;
      for (int i = 0; i < n; ++i) {
        const double* e = p + 6 + 5 * i;
        const double dx = x[0] - e[0], dy = x[1] - e[1];
        const double c = cos(e[4]), s = sin(e[4]);
        const double u = c * dx + s * dy, v = -s * dx + c * dy;
        const double dist = ellipse_signed_distance(u, v, e[2], e[3]);
        if (dist < best) best = dist;
      }
      if (p[5] != 0) best *= (p[1] + p[4] * (sq(x[0] - p[2]) + sq(x[1] - p[3])));
      return best;
    }
    default:
      return 0.0;
  }
}

}  // namespace lsg
