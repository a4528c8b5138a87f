// The C++ facade (include/lsgpu.hpp) gives exactly the results of the C ABI it wraps:
// reinitialisation, normal advection with a function-object velocity, both extensions,
// node interpolation and the semi-Lagrangian step. Prints "facade ok" on success; exits non-zero otherwise.
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <vector>

#include "lsgpu.hpp"

static double iface_value(int32_t n, int dir, double dist) { return 1.0 + 2.0 * dist + 0.01 * dir + 1e-4 * n; }
static int iface_values(void*, int64_t count, const int32_t* nodes, const int32_t* dirs, const double* dists, double* values) {
  for (int64_t k = 0; k < count; ++k) values[k] = iface_value(nodes[k], dirs[k], dists[k]);
  return 0;
}

static int fail(const char* what) {
  fprintf(stderr, "facade mismatch: %s\n", what);
  return 1;
}

int main() {
  const int n[3] = {1, 1, 1};
  const double lo[3] = {-1, -1, 0}, hi[3] = {1, 1, 1};
  lsg_forest* f = nullptr;
  lsgpu::check(lsg_forest_create(2, n, lo, hi, nullptr, &f));
  const double sphere[3] = {0.1, -0.05, 0.5};  // centre, radius
  lsgpu::check(lsg_forest_refine_levelset(f, 3, 7, 2.4, 0.0, 0, sphere, 3, 7));
  lsgpu::check(lsg_forest_build_nodes(f));
  const int64_t N = lsg_forest_num_nodes(f);
  std::vector<double> xyz((size_t)N * 2);
  lsgpu::check(lsg_forest_node_xyz(f, xyz.data()));
  std::vector<double> phi0((size_t)N);
  for (int64_t i = 0; i < N; ++i) {
    const double x = xyz[2 * i], y = xyz[2 * i + 1];
    phi0[i] = (sqrt((x - 0.1) * (x - 0.1) + (y + 0.05) * (y + 0.05)) - 0.5) * (0.1 + (x - 0.2) * (x - 0.2) + (y - 0.3) * (y - 0.3));
  }

  my_p4est_node_neighbors_t ngbd(f);
  ngbd.init_neighbors();
  my_p4est_level_set_t ls(&ngbd);
  lsgpu_vec phi{phi0};
  ls.reinitialize_2nd_order(&phi, 10);

  lsg_level_set* raw = nullptr;
  lsgpu::check(lsg_level_set_create(f, &raw));
  std::vector<double> ref(phi0);
  lsgpu::check(lsg_reinit_2nd(raw, ref.data(), 10, DBL_MAX, LSG_FP64));
  if (memcmp(ref.data(), phi.values.data(), N * sizeof(double)) != 0) return fail("reinitialize_2nd_order");

  // normal advection with a function-object velocity (CFL 0.8 time step)
  struct unit_speed {
    double operator()(double, double) const { return 1.0; }
  };
  lsgpu_vec adv{phi.values};
  const double dt = ls.advect_in_normal_direction(unit_speed(), &adv);
  std::vector<double> vn((size_t)N, 1.0), ref_adv(phi.values);
  double dt_ref = 0;
  lsgpu::check(lsg_advect_cfl_dt(raw, vn.data(), &dt_ref));
  lsgpu::check(lsg_advect_in_normal_direction(raw, vn.data(), nullptr, ref_adv.data(), dt_ref, nullptr, LSG_FP64));
  if (dt != dt_ref || memcmp(ref_adv.data(), adv.values.data(), N * sizeof(double)) != 0) return fail("advect_in_normal_direction");

  // node interpolation at scattered points, results by output index
  my_p4est_interpolation_nodes_t interp(&ngbd);
  std::vector<double> pts;
  for (int k = 0; k < 500; ++k) {
    const double p[2] = {-1.0 + 2.0 * ((k * 37) % 500) / 499.0, -1.0 + 2.0 * ((k * 91) % 500) / 499.0};
    interp.add_point(499 - k, p);
    pts.push_back(p[0]);
    pts.push_back(p[1]);
  }
  interp.set_input(&phi, quadratic_non_oscillatory_continuous_v2);
  std::vector<double> got(500), want(500);
  interp.interpolate(got.data());
  lsgpu::check(lsg_interpolate_nodes(raw, pts.data(), 500, phi.values.data(), 1, nullptr, LSG_QUADRATIC_NON_OSCILLATORY_CONTINUOUS_V2,
                                     want.data()));
  for (int k = 0; k < 500; ++k)
    if (got[499 - k] != want[k]) return fail("interpolate");

  // two block vectors of two components each, with the second derivatives as block vectors
  {
    const unsigned bs = 2;
    lsgpu_vec A{std::vector<double>((size_t)bs * N)}, B{std::vector<double>((size_t)bs * N)};
    std::vector<double> comps((size_t)4 * N);
    for (int64_t i = 0; i < N; ++i) {
      const double x = xyz[2 * i], y = xyz[2 * i + 1];
      const double v[4] = {x, y * y, x * y, 1.0 + x * x};
      A.values[bs * i] = v[0];
      A.values[bs * i + 1] = v[1];
      B.values[bs * i] = v[2];
      B.values[bs * i + 1] = v[3];
      for (int c = 0; c < 4; ++c) comps[(size_t)c * N + i] = v[c];
    }
    std::vector<double> dd((size_t)4 * 2 * N);
    for (int c = 0; c < 4; ++c) lsgpu::check(lsg_second_derivatives(raw, &comps[(size_t)c * N], &dd[(size_t)c * 2 * N]));
    lsgpu_vec Ab{std::vector<double>((size_t)bs * 2 * N)}, Bb{std::vector<double>((size_t)bs * 2 * N)};
    for (int64_t i = 0; i < N; ++i)
      for (unsigned c = 0; c < bs; ++c)
        for (int a = 0; a < 2; ++a) {
          Ab.values[(i * bs + c) * 2 + a] = dd[((size_t)c * 2 + a) * N + i];
          Bb.values[(i * bs + c) * 2 + a] = dd[((size_t)(2 + c) * 2 + a) * N + i];
        }
    Vec F[2] = {&A, &B}, Fb[2] = {&Ab, &Bb};
    my_p4est_interpolation_nodes_t multi(&ngbd);
    for (int k = 0; k < 500; ++k) multi.add_point(k, &pts[2 * k]);
    std::vector<double> oa((size_t)bs * 500), ob((size_t)bs * 500), ref((size_t)4 * 500);
    double* Fo[2] = {oa.data(), ob.data()};
    multi.set_input(F, Fb, quadratic_non_oscillatory, 2, bs);
    multi.interpolate(Fo);
    lsgpu::check(lsg_interpolate_nodes(raw, pts.data(), 500, comps.data(), 4, dd.data(), LSG_QUADRATIC_NON_OSCILLATORY, ref.data()));
    for (int k = 0; k < 500; ++k)
      for (unsigned c = 0; c < bs; ++c)
        if (oa[bs * k + c] != ref[(size_t)c * 500 + k] || ob[bs * k + c] != ref[(size_t)(2 + c) * 500 + k])
          return fail("interpolate (block vectors)");
    std::vector<double> one(500);
    double* Fo1[2] = {one.data(), one.data()};
    multi.set_input(F, quadratic, 2, bs);
    multi.interpolate(Fo1, 1);  // component 1 of every field (the second field's values end in the buffer)
    lsgpu::check(lsg_interpolate_nodes(raw, pts.data(), 500, &comps[(size_t)3 * N], 1, nullptr, LSG_QUADRATIC, ref.data()));
    for (int k = 0; k < 500; ++k)
      if (one[k] != ref[k]) return fail("interpolate (one component)");
  }

  // semi-Lagrangian step onto the same grid with a rotating node velocity
  lsgpu_vec vx{std::vector<double>((size_t)N)}, vy{std::vector<double>((size_t)N)};
  for (int64_t i = 0; i < N; ++i) {
    vx.values[i] = -xyz[2 * i + 1];
    vy.values[i] = xyz[2 * i];
  }
  Vec v[2] = {&vx, &vy};
  my_p4est_semi_lagrangian_t sl(f, &ngbd);
  std::vector<double> np1((size_t)N), np1_ref((size_t)N), vv((size_t)2 * N);
  sl.advect_from_n_to_np1(0.01, v, nullptr, &phi, nullptr, np1.data());
  memcpy(vv.data(), vx.values.data(), N * sizeof(double));
  memcpy(vv.data() + N, vy.values.data(), N * sizeof(double));
  lsgpu::check(lsg_semi_lagrangian_advect(raw, xyz.data(), N, 0.01, vv.data(), nullptr, phi.values.data(), nullptr,
                                          LSG_QUADRATIC_NON_OSCILLATORY_CONTINUOUS_V2, LSG_QUADRATIC_NON_OSCILLATORY_CONTINUOUS_V2,
                                          np1_ref.data()));
  if (memcmp(np1.data(), np1_ref.data(), N * sizeof(double)) != 0) return fail("advect_from_n_to_np1");

  // the two-velocity step (velocity n-1 a scaled copy on the same grid) against the C ABI
  {
    lsgpu_vec wx{std::vector<double>((size_t)N)}, wy{std::vector<double>((size_t)N)};
    for (int64_t i = 0; i < N; ++i) {
      wx.values[i] = 0.8 * vx.values[i] + 0.1;
      wy.values[i] = 0.8 * vy.values[i];
    }
    Vec w[2] = {&wx, &wy};
    my_p4est_semi_lagrangian_t sl2(f, &ngbd, &ngbd);
    std::vector<double> np2((size_t)N), np2_ref((size_t)N), ww((size_t)2 * N);
    sl2.advect_from_n_to_np1(0.04, 0.05, w, nullptr, v, nullptr, &phi, nullptr, np2.data());
    memcpy(ww.data(), wx.values.data(), N * sizeof(double));
    memcpy(ww.data() + N, wy.values.data(), N * sizeof(double));
    lsgpu::check(lsg_semi_lagrangian_advect2(raw, raw, xyz.data(), N, 0.04, 0.05, ww.data(), nullptr, vv.data(), nullptr, phi.values.data(),
                                             nullptr, LSG_QUADRATIC_NON_OSCILLATORY_CONTINUOUS_V2,
                                             LSG_QUADRATIC_NON_OSCILLATORY_CONTINUOUS_V2, np2_ref.data()));
    if (memcmp(np2.data(), np2_ref.data(), N * sizeof(double)) != 0) return fail("advect_from_n_to_np1 (two velocities)");
    lsg_forest* fu = nullptr;
    lsgpu::check(lsg_forest_copy(f, &fu));
    my_p4est_semi_lagrangian_t up2(fu, &ngbd, &ngbd);
    up2.set_splitting(3, 7, 2.4);
    lsgpu_vec phi2{phi.values};
    Vec p2 = &phi2;
    if (up2.update_p4est(w, v, 0.04, 0.05, p2, nullptr, &phi) < 1 || phi2.values.size() != (size_t)lsg_forest_num_nodes(fu))
      return fail("update_p4est (two velocities)");
    lsg_forest_destroy(fu);
  }

  // extension over the interface with given normals and a mask
  lsgpu_vec q{std::vector<double>((size_t)N)}, nx{std::vector<double>((size_t)N)}, ny{std::vector<double>((size_t)N)};
  for (int64_t i = 0; i < N; ++i) {
    q.values[i] = phi.values[i] < 0 ? xyz[2 * i] * xyz[2 * i + 1] + 1.0 : 0.0;
    const double r = sqrt(xyz[2 * i] * xyz[2 * i] + xyz[2 * i + 1] * xyz[2 * i + 1]) + 1e-3;
    nx.values[i] = xyz[2 * i] / r;
    ny.values[i] = xyz[2 * i + 1] / r;
  }
  std::vector<double> q_ref(q.values), nrm_ref((size_t)2 * N);
  memcpy(nrm_ref.data(), nx.values.data(), N * sizeof(double));
  memcpy(nrm_ref.data() + N, ny.values.data(), N * sizeof(double));
  Vec nrm[2] = {&nx, &ny};
  ls.extend_Over_Interface_TVD(&phi, &q, 8, 2, -DBL_MAX, DBL_MAX, nrm, &phi);
  lsgpu::check(lsg_extend_over_interface_tvd(raw, phi.values.data(), q_ref.data(), 8, 2, -DBL_MAX, DBL_MAX, nrm_ref.data(),
                                             phi.values.data()));
  if (memcmp(q.values.data(), q_ref.data(), N * sizeof(double)) != 0) return fail("extend_Over_Interface_TVD");

  // extension from the interface, two interleaved components against the ABI's component blocks
  lsgpu_vec qi2{std::vector<double>((size_t)2 * N)}, qe2{std::vector<double>((size_t)2 * N)};
  std::vector<double> qi_blocks((size_t)2 * N), qe_ref((size_t)2 * N);
  for (int64_t i = 0; i < N; ++i) {
    qi2.values[2 * i] = qi_blocks[i] = xyz[2 * i] + 2.0 * xyz[2 * i + 1];
    qi2.values[2 * i + 1] = qi_blocks[N + i] = xyz[2 * i] * xyz[2 * i];
  }
  ls.set_interpolation_on_interface(quadratic);
  ls.extend_from_interface_to_whole_domain_TVD(&phi, &qi2, &qe2, 6, nullptr, 2, 10, nullptr, nullptr, 2);
  lsgpu::check(lsg_extend_from_interface_to_whole_domain_tvd(raw, phi.values.data(), qi_blocks.data(), qe_ref.data(), 2, 6, nullptr, 2,
                                                             10, nullptr, LSG_QUADRATIC));
  for (int64_t i = 0; i < N; ++i)
    if (qe2.values[2 * i] != qe_ref[i] || qe2.values[2 * i + 1] != qe_ref[N + i]) return fail("extend_from_interface_to_whole_domain_TVD");

  // the CF overload with a constant velocity: departure points x - dt c, clipped, then the phi
  // interpolation of the C ABI at those points
  struct constant_velocity {
    double c;
    double operator()(double, double) const { return c; }
  };
  const constant_velocity cx{0.3}, cy{-0.2};
  const constant_velocity* cf[2] = {&cx, &cy};
  std::vector<double> np1_cf((size_t)N), xd((size_t)2 * N), np1_cf_ref((size_t)N);
  sl.advect_from_n_to_np1(0.05, cf, &phi, nullptr, np1_cf.data());
  for (int64_t i = 0; i < N; ++i) {
    xd[2 * i] = xyz[2 * i] - 0.05 * 0.3;
    xd[2 * i + 1] = xyz[2 * i + 1] - 0.05 * -0.2;
    for (int a = 0; a < 2; ++a) xd[2 * i + a] = xd[2 * i + a] < lo[a] ? lo[a] : (xd[2 * i + a] > hi[a] ? hi[a] : xd[2 * i + a]);
  }
  lsgpu::check(lsg_interpolate_nodes(raw, xd.data(), N, phi.values.data(), 1, nullptr, LSG_QUADRATIC_NON_OSCILLATORY_CONTINUOUS_V2,
                                     np1_cf_ref.data()));
  if (memcmp(np1_cf.data(), np1_cf_ref.data(), N * sizeof(double)) != 0) return fail("advect_from_n_to_np1 (CF)");

  // the cf form: interface values from a function of (node, direction, distance)
  lsgpu_vec qi1{std::vector<double>((size_t)N)}, qcf{std::vector<double>((size_t)N)};
  for (int64_t i = 0; i < N; ++i) qi1.values[i] = xyz[2 * i] - xyz[2 * i + 1];
  std::vector<double> qcf_ref((size_t)N);
  ls.extend_from_interface_to_whole_domain_TVD(&phi, &qi1, &qcf, 5, nullptr, 2, 10, iface_value, nullptr, 1);
  lsgpu::check(lsg_extend_from_interface_to_whole_domain_tvd_cf(raw, phi.values.data(), qi1.values.data(), qcf_ref.data(), 5, iface_values,
                                                                nullptr, nullptr));
  if (memcmp(qcf.values.data(), qcf_ref.data(), N * sizeof(double)) != 0) return fail("extend_from_interface_to_whole_domain_TVD (cf)");

  // update_p4est with node velocities: the regrid loop against the same loop written with the C ABI
  {
    lsg_forest *fa = nullptr, *fb = nullptr;
    lsgpu::check(lsg_forest_copy(f, &fa));
    lsgpu::check(lsg_forest_copy(f, &fb));
    my_p4est_semi_lagrangian_t up(fa, &ngbd, 3, 7, 2.4);
    lsgpu_vec phi_up{phi.values};
    Vec pv = &phi_up;
    const int passes = up.update_p4est(v, 0.05, pv);
    std::vector<double> vv((size_t)2 * N), vdd((size_t)4 * N), pdd((size_t)2 * N), out;
    memcpy(vv.data(), vx.values.data(), N * sizeof(double));
    memcpy(vv.data() + N, vy.values.data(), N * sizeof(double));
    for (int a = 0; a < 2; ++a) lsgpu::check(lsg_second_derivatives(raw, &vv[(size_t)a * N], &vdd[(size_t)a * 2 * N]));
    lsgpu::check(lsg_second_derivatives(raw, phi.values.data(), pdd.data()));
    int ref_passes = 0;
    for (;;) {
      const int64_t np = lsg_forest_num_nodes(fb);
      std::vector<double> x2((size_t)np * 2);
      out.assign((size_t)np, 0.0);
      lsgpu::check(lsg_forest_node_xyz(fb, x2.data()));
      lsgpu::check(lsg_semi_lagrangian_advect(raw, x2.data(), np, 0.05, vv.data(), vdd.data(), phi.values.data(), pdd.data(),
                                              LSG_QUADRATIC_NON_OSCILLATORY_CONTINUOUS_V2, LSG_QUADRATIC_NON_OSCILLATORY_CONTINUOUS_V2,
                                              out.data()));
      ++ref_passes;
      int changed = 0;
      lsgpu::check(lsg_forest_refine_and_coarsen(fb, 3, 7, 2.4, 0.0, out.data(), &changed));
      if (!changed) break;
      lsgpu::check(lsg_forest_build_nodes(fb));
    }
    if (passes != ref_passes || phi_up.values.size() != out.size() ||
        memcmp(phi_up.values.data(), out.data(), out.size() * sizeof(double)) != 0)
      return fail("update_p4est");
    // the CF form with a constant velocity runs the same loop through the callback
    lsg_forest* fc = nullptr;
    lsgpu::check(lsg_forest_copy(f, &fc));
    my_p4est_semi_lagrangian_t upc(fc, &ngbd, 3, 7, 2.4);
    lsgpu_vec phi_c{phi.values};
    Vec pc = &phi_c;
    if (upc.update_p4est(cf, 0.05, pc) < 1 || phi_c.values.size() != (size_t)lsg_forest_num_nodes(fc)) return fail("update_p4est (CF)");
    lsg_forest_destroy(fa);
    lsg_forest_destroy(fb);
    lsg_forest_destroy(fc);
  }

  // errors come back as exceptions
  try {
    ls.reinitialize_within_range_of_phi_0(&phi, 3, 2, 1.0, -1.0, 5);
    return fail("bad order accepted");
  } catch (const std::invalid_argument&) {
  }
  lsg_level_set_destroy(raw);
  printf("facade ok (%lld nodes)\n", (long long)N);
  return 0;
}
