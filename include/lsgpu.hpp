/*
 * lsgpu.hpp: C++ facade over the C ABI (lsgpu.h) with parCASL's class names and method signatures,
 * so C++ code written against my_p4est_level_set_t, my_p4est_interpolation_nodes_t and
 * my_p4est_semi_lagrangian_t keeps its calls:
 *
 *   my_p4est_level_set_t(my_p4est_node_neighbors_t*)                  src/my_p4est_level_set.h:385-414
 *   reinitialize_{1st,2nd}_order[_above_threshold|_time_...](Vec phi, iterations, limit)
 *                                                                      src/my_p4est_level_set.h:434-613
 *   reinitialize_2nd_order_with_mask(Vec phi, Vec mask, number_of_masked, iterations, limit)
 *                                                                      src/my_p4est_level_set.h:487-525
 *   perturb_level_set_function(Vec phi, epsilon)                       src/my_p4est_level_set.h:621
 *   advect_in_normal_direction(CF / Vec vn[, Vec vn_np1], Vec phi, dt, phi_xx, phi_yy[, phi_zz])
 *                                                                      src/my_p4est_level_set.h:632-659
 *   extend_Over_Interface_TVD(phi, q, iterations, order, band_use, band_extend, normal, mask)
 *                                                                      src/my_p4est_level_set.h:732-735
 *   extend_from_interface_to_whole_domain_TVD(phi, qi, q, iterations, mask, band_zero, band_smooth,
 *                                             cf, grad_phi, blocksize), set_interpolation_on_interface
 *                                                                      src/my_p4est_level_set.h:775-776, 843
 *   my_p4est_interpolation_nodes_t: set_input, add_point, interpolate  src/my_p4est_interpolation_nodes.h:33-103
 *   my_p4est_semi_lagrangian_t::advect_from_n_to_np1, update_p4est (one and two velocities)
 *                                                                      src/my_p4est_semi_lagrangian.h:83-196
 *
 * Vec: with LSGPU_WITH_PETSC defined before inclusion, PETSc's Vec (read through VecGetArray);
 * otherwise a minimal host vector with the same accessor names (VecGetArray / VecRestoreArray /
 * VecGetLocalSize). Node values are in lsgpu's node order (the order my_p4est_nodes_new gives in a
 * single process). Status codes become exceptions: LSG_EINVAL -> std::invalid_argument, anything
 * else -> std::runtime_error, carrying lsg_last_error().
 *
 * The grid side (my_p4est_brick_new, refinement, my_p4est_nodes_new, init_neighbors) is the
 * forest of lsgpu.h; my_p4est_node_neighbors_t here owns the device image of the node neighbours
 * (built on first use) that every object of one grid shares.
 */
#ifndef LSGPU_HPP
#define LSGPU_HPP

#include <float.h>
#include <limits.h>
#include <math.h>

#include <algorithm>
#include <cmath>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "lsgpu.h"

#ifdef LSGPU_WITH_PETSC
#include <petscvec.h>
#else
struct lsgpu_vec {
  std::vector<double> values;
};
typedef lsgpu_vec* Vec;
inline int VecGetArray(Vec x, double** a) {
  *a = x->values.data();
  return 0;
}
inline int VecRestoreArray(Vec, double** a) {
  *a = nullptr;
  return 0;
}
inline int VecGetLocalSize(Vec x, int* n) {
  *n = (int)x->values.size();
  return 0;
}
#endif

namespace lsgpu {

inline void check(int status) {
  if (status == LSG_OK) return;
  const std::string msg = std::string("lsgpu: ") + lsg_last_error();
  if (status == LSG_EINVAL) throw std::invalid_argument(msg);
  throw std::runtime_error(msg);
}

// Evaluate a function object of the node coordinates: (x, y) in 2D, (x, y, z) in 3D (C++17).
template <typename CF>
double eval_cf(const CF& f, const double* x, int dim) {
  if constexpr (std::is_invocable_v<const CF&, double, double, double>) {
    if (dim == 3) return f(x[0], x[1], x[2]);
  }
  if constexpr (std::is_invocable_v<const CF&, double, double>) {
    if (dim == 2) return f(x[0], x[1]);
  }
  throw std::invalid_argument("lsgpu: the velocity function does not take the grid's number of coordinates");
}

// Borrow the host array of a Vec for the duration of one call.
struct VecArray {
  Vec v;
  double* p = nullptr;
  explicit VecArray(Vec v_) : v(v_) {
    if (v) VecGetArray(v, &p);
  }
  ~VecArray() {
    if (v) VecRestoreArray(v, &p);
  }
  VecArray(const VecArray&) = delete;
  VecArray& operator=(const VecArray&) = delete;
};

}  // namespace lsgpu

enum interpolation_method {
  linear = LSG_LINEAR,
  quadratic = LSG_QUADRATIC,
  quadratic_non_oscillatory = LSG_QUADRATIC_NON_OSCILLATORY,
  quadratic_non_oscillatory_continuous_v1 = LSG_QUADRATIC_NON_OSCILLATORY_CONTINUOUS_V1,
  quadratic_non_oscillatory_continuous_v2 = LSG_QUADRATIC_NON_OSCILLATORY_CONTINUOUS_V2
};

// Node neighbours of one grid (the forest must have its nodes built and outlive this object).
class my_p4est_node_neighbors_t {
 public:
  explicit my_p4est_node_neighbors_t(lsg_forest* forest) : forest_(forest) {}
  ~my_p4est_node_neighbors_t() {
    if (ls_) lsg_level_set_destroy(ls_);
  }
  my_p4est_node_neighbors_t(const my_p4est_node_neighbors_t&) = delete;
  my_p4est_node_neighbors_t& operator=(const my_p4est_node_neighbors_t&) = delete;
  void init_neighbors() { device(); }
  lsg_forest* forest() const { return forest_; }
  int dim() const { return lsg_forest_dim(forest_); }
  int64_t num_nodes() const { return lsg_forest_num_nodes(forest_); }
  // device image shared by the level-set, interpolation and semi-Lagrangian objects of this grid
  lsg_level_set* device() const {
    if (!ls_) lsgpu::check(lsg_level_set_create(forest_, &ls_));
    return ls_;
  }
  std::vector<double> node_xyz() const {
    std::vector<double> xyz((size_t)num_nodes() * dim());
    lsgpu::check(lsg_forest_node_xyz(forest_, xyz.data()));
    return xyz;
  }

 private:
  lsg_forest* forest_;
  mutable lsg_level_set* ls_ = nullptr;
};

class my_p4est_level_set_t {
 public:
  // precision: LSG_FP64 (the reference's arithmetic) or LSG_MIXED (FP32 stencil, FP64 subcell step)
  explicit my_p4est_level_set_t(my_p4est_node_neighbors_t* ngbd, int precision = LSG_FP64) : ngbd_(ngbd), precision_(precision) {}
  explicit my_p4est_level_set_t(const my_p4est_node_neighbors_t* ngbd, int precision = LSG_FP64)
      : ngbd_(const_cast<my_p4est_node_neighbors_t*>(ngbd)), precision_(precision) {}
  void update(my_p4est_node_neighbors_t* ngbd) { ngbd_ = ngbd; }

  void reinitialize_within_range_of_phi_0(Vec phi, const unsigned char order_space, const unsigned char order_pseudotime,
                                          const double& limit_high, const double& limit_low, const int& number_of_iterations) const {
    lsgpu::VecArray p(phi);
    lsgpu::check(lsg_reinitialize(ngbd_->device(), p.p, order_space, order_pseudotime, limit_high, limit_low, number_of_iterations,
                                  precision_));
  }
  void reinitialize_1st_order(Vec phi, const int& number_of_iterations = 50, const double& limit_absolute_value_phi_0 = DBL_MAX) const {
    reinitialize_within_range_of_phi_0(phi, 1, 1, limit_absolute_value_phi_0, -limit_absolute_value_phi_0, number_of_iterations);
  }
  void reinitialize_1st_order_above_threshold(Vec phi, const double& threshold, const int& number_of_iterations = 50,
                                              const double& upper_limit_phi_0 = DBL_MAX) const {
    reinitialize_within_range_of_phi_0(phi, 1, 1, upper_limit_phi_0, threshold, number_of_iterations);
  }
  void reinitialize_2nd_order(Vec phi, const int& number_of_iterations = 50, const double& limit_absolute_value_phi_0 = DBL_MAX) const {
    reinitialize_within_range_of_phi_0(phi, 2, 2, limit_absolute_value_phi_0, -limit_absolute_value_phi_0, number_of_iterations);
  }
  void reinitialize_2nd_order_above_threshold(Vec phi, const double& threshold, const int& number_of_iterations = 50,
                                              const double& upper_limit_phi_0 = DBL_MAX) const {
    reinitialize_within_range_of_phi_0(phi, 2, 2, upper_limit_phi_0, threshold, number_of_iterations);
  }
  void reinitialize_2nd_order_time_1st_order_space(Vec phi, const int& number_of_iterations = 50,
                                                   const double& limit_absolute_value_phi_0 = DBL_MAX) const {
    reinitialize_within_range_of_phi_0(phi, 1, 2, limit_absolute_value_phi_0, -limit_absolute_value_phi_0, number_of_iterations);
  }
  void reinitialize_2nd_order_time_1st_order_space_above_threshold(Vec phi, const double& threshold, const int& number_of_iterations = 50,
                                                                  const double& upper_limit_phi_0 = DBL_MAX) const {
    reinitialize_within_range_of_phi_0(phi, 1, 2, upper_limit_phi_0, threshold, number_of_iterations);
  }
  void reinitialize_1st_order_time_2nd_order_space(Vec phi, const int& number_of_iterations = 50,
                                                   const double& limit_absolute_value_phi_0 = DBL_MAX) const {
    reinitialize_within_range_of_phi_0(phi, 2, 1, limit_absolute_value_phi_0, -limit_absolute_value_phi_0, number_of_iterations);
  }
  void reinitialize_1st_order_time_2nd_order_space_above_threshold(Vec phi, const double& threshold, const int& number_of_iterations = 50,
                                                                  const double& upper_limit_phi_0 = DBL_MAX) const {
    reinitialize_within_range_of_phi_0(phi, 2, 1, upper_limit_phi_0, threshold, number_of_iterations);
  }
  void reinitialize_2nd_order_with_mask(Vec phi, Vec mask, const int& number_of_masked, const int& number_of_iterations = 50,
                                        const double& limit_absolute_value_phi_0 = DBL_MAX) const {
    (void)number_of_masked;  // a reservation hint in the reference
    lsgpu::VecArray p(phi), m(mask);
    lsgpu::check(lsg_reinitialize_with_mask(ngbd_->device(), p.p, m.p, 2, 2, limit_absolute_value_phi_0, -limit_absolute_value_phi_0,
                                            number_of_iterations, precision_));
  }
  void perturb_level_set_function(Vec phi, const double& epsilon) const {
    lsgpu::VecArray p(phi);
    lsgpu::check(lsg_perturb_level_set_function(ngbd_->device(), p.p, epsilon));
  }

  // boundary conditions (bc) are not supported: passing them raises std::invalid_argument
  template <typename BC = void>
  void extend_Over_Interface_TVD(Vec phi, Vec q, int iterations = 20, int order = 2, double band_use = -DBL_MAX,
                                 double band_extend = DBL_MAX, Vec normal[] = nullptr, Vec mask = nullptr, BC* bc = nullptr,
                                 bool use_nonzero_guess = false, Vec q_n = nullptr, Vec q_nn = nullptr) const {
    if (bc != nullptr) throw std::invalid_argument("extend_Over_Interface_TVD: boundary conditions are not supported");
    lsgpu::VecArray p(phi), v(q), m(mask), qn(q_n), qnn(q_nn);
    const int D = ngbd_->dim();
    const size_t N = (size_t)ngbd_->num_nodes();
    std::vector<double> nrm;
    if (normal != nullptr) {
      nrm.resize((size_t)D * N);
      for (int a = 0; a < D; ++a) {
        lsgpu::VecArray x(normal[a]);
        for (size_t n = 0; n < N; ++n) nrm[a * N + n] = x.p[n];
      }
    }
    lsgpu::check(lsg_extend_over_interface_tvd_ex(ngbd_->device(), p.p, v.p, iterations, order, band_use, band_extend,
                                                  normal ? nrm.data() : nullptr, mask ? m.p : nullptr, use_nonzero_guess ? 1 : 0,
                                                  q_n ? qn.p : nullptr, q_nn ? qnn.p : nullptr));
  }

  void set_interpolation_on_interface(interpolation_method value) { interpolation_on_interface_ = value; }

  // q_interface, q: blocksize values per node, interleaved as in the reference's block vectors; grad_phi_in:
  // dim values per node, interleaved. cf (interface values by node, direction and distance) needs no mask
  // and a block size of 1, as in the reference.
  void extend_from_interface_to_whole_domain_TVD(Vec phi, Vec q_interface, Vec q, int iterations = 20, Vec mask = nullptr,
                                                 double band_zero = 2, double band_smooth = 10,
                                                 double (*cf)(int32_t, int, double) = nullptr, Vec grad_phi_in = nullptr,
                                                 const unsigned int& blocksize = 1) const {
    const int D = ngbd_->dim();
    if (cf != nullptr) {
      if (mask != nullptr || blocksize != 1)
        throw std::invalid_argument("extend_from_interface_to_whole_domain_TVD: cf needs no mask and a block size of 1");
      lsg_interface_values_fn fn = [](void* c, int64_t count, const int32_t* nodes, const int32_t* dirs, const double* dists,
                                      double* values) -> int {
        auto f = reinterpret_cast<double (*)(int32_t, int, double)>(c);
        for (int64_t k = 0; k < count; ++k) values[k] = f(nodes[k], dirs[k], dists[k]);
        return 0;
      };
      lsgpu::VecArray p(phi), qi(q_interface), qo(q), g(grad_phi_in);
      const size_t N = (size_t)ngbd_->num_nodes();
      std::vector<double> g_b;
      if (grad_phi_in != nullptr) {
        g_b.resize((size_t)D * N);
        for (size_t n = 0; n < N; ++n)
          for (int a = 0; a < D; ++a) g_b[a * N + n] = g.p[(size_t)D * n + a];
      }
      lsgpu::check(lsg_extend_from_interface_to_whole_domain_tvd_cf(ngbd_->device(), p.p, qi.p, qo.p, iterations, fn,
                                                                    reinterpret_cast<void*>(cf), grad_phi_in ? g_b.data() : nullptr));
      return;
    }
    const size_t N = (size_t)ngbd_->num_nodes(), bs = blocksize;
    lsgpu::VecArray p(phi), qi(q_interface), qo(q), m(mask), g(grad_phi_in);
    std::vector<double> qi_b(bs * N), q_b(bs * N), g_b;
    for (size_t n = 0; n < N; ++n)
      for (size_t k = 0; k < bs; ++k) qi_b[k * N + n] = qi.p[bs * n + k];
    if (grad_phi_in != nullptr) {
      g_b.resize((size_t)D * N);
      for (size_t n = 0; n < N; ++n)
        for (int a = 0; a < D; ++a) g_b[a * N + n] = g.p[(size_t)D * n + a];
    }
    lsgpu::check(lsg_extend_from_interface_to_whole_domain_tvd(ngbd_->device(), p.p, qi_b.data(), q_b.data(), (int)bs, iterations,
                                                               mask ? m.p : nullptr, band_zero, band_smooth,
                                                               grad_phi_in ? g_b.data() : nullptr, interpolation_on_interface_));
    for (size_t n = 0; n < N; ++n)
      for (size_t k = 0; k < bs; ++k) qo.p[bs * n + k] = q_b[k * N + n];
  }

  // node-sampled velocity: returns dt unchanged
  double advect_in_normal_direction(const Vec vn, Vec phi, const double& dt, Vec phi_xx = nullptr, Vec phi_yy = nullptr,
                                    Vec phi_zz = nullptr) const {
    return advect_in_normal_direction(vn, nullptr, phi, dt, phi_xx, phi_yy, phi_zz);
  }
  double advect_in_normal_direction(const Vec vn, const Vec vn_np1, Vec phi, const double& dt, Vec phi_xx = nullptr,
                                    Vec phi_yy = nullptr, Vec phi_zz = nullptr) const {
    lsgpu::VecArray v(vn), v1(vn_np1), p(phi);
    const int D = ngbd_->dim();
    const size_t N = (size_t)ngbd_->num_nodes();
    // the derivative Vecs are separate in the reference; the ABI takes them as D blocks of N
    std::vector<double> dd;
    Vec xx[3] = {phi_xx, phi_yy, phi_zz};
    const bool given = phi_xx != nullptr;
    if (given) {
      dd.resize((size_t)D * N);
      for (int a = 0; a < D; ++a) {
        lsgpu::VecArray x(xx[a]);
        for (size_t n = 0; n < N; ++n) dd[a * N + n] = x.p[n];
      }
    }
    lsgpu::check(lsg_advect_in_normal_direction(ngbd_->device(), v.p, vn_np1 ? v1.p : nullptr, p.p, dt, given ? dd.data() : nullptr,
                                                precision_));
    if (given)
      for (int a = 0; a < D; ++a) {
        lsgpu::VecArray x(xx[a]);
        for (size_t n = 0; n < N; ++n) x.p[n] = dd[a * N + n];
      }
    return dt;
  }
  // velocity given as a function object of the node coordinates (x, y[, z]): dt from CFL 0.8, returned
  template <typename CF>
  double advect_in_normal_direction(const CF& vn, Vec phi, Vec phi_xx = nullptr, Vec phi_yy = nullptr, Vec phi_zz = nullptr) const {
    const int D = ngbd_->dim();
    const std::vector<double> xyz = ngbd_->node_xyz();
    const size_t N = xyz.size() / D;
    lsgpu_vec_values v(N);
    for (size_t n = 0; n < N; ++n) v.data[n] = lsgpu::eval_cf(vn, &xyz[(size_t)D * n], D);
    double dt = 0;
    lsgpu::check(lsg_advect_cfl_dt(ngbd_->device(), v.data.data(), &dt));
    lsgpu::VecArray p(phi);
    std::vector<double> dd;
    Vec xx[3] = {phi_xx, phi_yy, phi_zz};
    if (phi_xx) {
      dd.resize((size_t)D * N);
      for (int a = 0; a < D; ++a) {
        lsgpu::VecArray x(xx[a]);
        for (size_t n = 0; n < N; ++n) dd[a * N + n] = x.p[n];
      }
    }
    lsgpu::check(lsg_advect_in_normal_direction(ngbd_->device(), v.data.data(), nullptr, p.p, dt, phi_xx ? dd.data() : nullptr,
                                                precision_));
    return dt;
  }

 private:
  struct lsgpu_vec_values {
    explicit lsgpu_vec_values(size_t n) : data(n) {}
    std::vector<double> data;
  };
  my_p4est_node_neighbors_t* ngbd_;
  int precision_;
  interpolation_method interpolation_on_interface_ = quadratic_non_oscillatory_continuous_v2;
};

// Node interpolation at buffered points (one process: every point is local).
class my_p4est_interpolation_nodes_t {
 public:
  static const unsigned int ALL_COMPONENTS = UINT_MAX;
  explicit my_p4est_interpolation_nodes_t(const my_p4est_node_neighbors_t* ngbd) : ngbd_(ngbd) {}
  void clear() {
    idx_.clear();
    xyz_.clear();
  }
  void add_point(int64_t node_idx_on_output, const double* xyz) {
    idx_.push_back(node_idx_on_output);
    for (int a = 0; a < ngbd_->dim(); ++a) xyz_.push_back(xyz[a]);
  }
  // n_vecs input fields, each a block vector of block_size_f components per node (interleaved)
  void set_input(Vec* F, interpolation_method method, size_t n_vecs, unsigned int block_size_f = 1) {
    F_.assign(F, F + n_vecs);
    for (auto& v : Fdd_) v.clear();
    Fblock_.clear();
    bs_ = block_size_f;
    method_ = method;
  }
  void set_input(Vec F, interpolation_method method, unsigned int block_size_f = 1) { set_input(&F, method, 1, block_size_f); }
  // second derivatives given component by component (Fxx[k], Fyy[k][, Fzz[k]] block vectors like F[k])
  void set_input(Vec* F, Vec* Fxx, Vec* Fyy, Vec* Fzz, interpolation_method method, size_t n_vecs, unsigned int block_size_f = 1) {
    set_input(F, method, n_vecs, block_size_f);
    Vec* dd[3] = {Fxx, Fyy, Fzz};
    for (int a = 0; a < ngbd_->dim(); ++a)
      if (dd[a]) Fdd_[a].assign(dd[a], dd[a] + n_vecs);
  }
  void set_input(Vec F, Vec Fxx, Vec Fyy, Vec Fzz, interpolation_method method, unsigned int block_size_f = 1) {
    set_input(&F, &Fxx, &Fyy, Fzz ? &Fzz : nullptr, method, 1, block_size_f);
  }
  void set_input(Vec F, Vec Fxx, Vec Fyy, interpolation_method method) { set_input(F, Fxx, Fyy, nullptr, method); }
  // second derivatives as one block vector per field: [(node * block_size_f + component) * dim + direction]
  void set_input(Vec* F, Vec* Fxxyyzz_block, interpolation_method method, size_t n_vecs, unsigned int block_size_f = 1) {
    set_input(F, method, n_vecs, block_size_f);
    Fblock_.assign(Fxxyyzz_block, Fxxyyzz_block + n_vecs);
  }
  void set_input(Vec F, Vec Fxxyyzz_block, interpolation_method method, unsigned int block_size_f = 1) {
    set_input(&F, &Fxxyyzz_block, method, 1, block_size_f);
  }
  // Fo[k][bs * node_idx_on_output + c] (all components) or Fo[k][node_idx_on_output] (one component)
  void interpolate(double* const* Fo, unsigned int comp = ALL_COMPONENTS) const {
    const int D = ngbd_->dim();
    const size_t N = (size_t)ngbd_->num_nodes(), nv = F_.size();
    if (comp != ALL_COMPONENTS && comp >= bs_) throw std::invalid_argument("interpolate: component out of range");
    const unsigned int nc = (comp == ALL_COMPONENTS) ? bs_ : 1;
    const size_t nf = nv * nc;
    const bool have_dd = method_ != linear && (!Fblock_.empty() || !Fdd_[0].empty());
    std::vector<double> f(nf * N), dd(have_dd ? nf * D * N : 0);
    for (size_t k = 0; k < nv; ++k) {
      lsgpu::VecArray x(F_[k]);
      for (unsigned int c = 0; c < nc; ++c) {
        const unsigned int cc = comp == ALL_COMPONENTS ? c : comp;
        const size_t fi = k * nc + c;
        for (size_t n = 0; n < N; ++n) f[fi * N + n] = x.p[bs_ * n + cc];
        if (!have_dd) continue;
        if (!Fblock_.empty()) {
          lsgpu::VecArray b(Fblock_[k]);
          for (int a = 0; a < D; ++a)
            for (size_t n = 0; n < N; ++n) dd[(fi * D + a) * N + n] = b.p[(n * bs_ + cc) * D + a];
        } else {
          for (int a = 0; a < D; ++a) {
            lsgpu::VecArray y(Fdd_[a][k]);
            for (size_t n = 0; n < N; ++n) dd[(fi * D + a) * N + n] = y.p[bs_ * n + cc];
          }
        }
      }
    }
    const size_t np = idx_.size();
    std::vector<double> out(nf * np);
    lsgpu::check(lsg_interpolate_nodes(ngbd_->device(), xyz_.data(), (int64_t)np, f.data(), (int)nf, have_dd ? dd.data() : nullptr,
                                       (int)method_, out.data()));
    for (size_t k = 0; k < nv; ++k)
      for (unsigned int c = 0; c < nc; ++c)
        for (size_t i = 0; i < np; ++i) {
          const double v = out[(k * nc + c) * np + i];
          if (comp == ALL_COMPONENTS)
            Fo[k][bs_ * idx_[i] + c] = v;
          else
            Fo[k][idx_[i]] = v;
        }
  }
  // one field: results[node_idx_on_output] (block size 1) or results[bs * node_idx_on_output + c]
  void interpolate(double* results) const { interpolate(&results); }
  void interpolate(Vec out) const {
    lsgpu::VecArray o(out);
    interpolate(o.p);
  }
  void interpolate(Vec* out, unsigned int comp = ALL_COMPONENTS) const {
    std::vector<std::unique_ptr<lsgpu::VecArray>> arr;
    std::vector<double*> ptr;
    for (size_t k = 0; k < F_.size(); ++k) {
      arr.emplace_back(new lsgpu::VecArray(out[k]));
      ptr.push_back(arr.back()->p);
    }
    interpolate(ptr.data(), comp);
  }

 private:
  const my_p4est_node_neighbors_t* ngbd_;
  std::vector<int64_t> idx_;
  std::vector<double> xyz_;
  std::vector<Vec> F_;
  std::vector<Vec> Fdd_[3];
  std::vector<Vec> Fblock_;
  unsigned int bs_ = 1;
  interpolation_method method_ = linear;
};

// Semi-Lagrangian step from the grid at n (ngbd_n) onto the nodes of the grid at n+1.
class my_p4est_semi_lagrangian_t {
 public:
  my_p4est_semi_lagrangian_t(lsg_forest* forest_np1, my_p4est_node_neighbors_t* ngbd_n) : forest_np1_(forest_np1), ngbd_n_(ngbd_n) {}
  // with the splitting criterion of grid n+1 (the reference reads it from p4est->user_pointer)
  my_p4est_semi_lagrangian_t(lsg_forest* forest_np1, my_p4est_node_neighbors_t* ngbd_n, int min_lvl, int max_lvl, double lip)
      : forest_np1_(forest_np1), ngbd_n_(ngbd_n), min_lvl_(min_lvl), max_lvl_(max_lvl), lip_(lip) {}
  // with the grid at n-1 as well (the reference's ngbd_nm1), for the two-velocity forms
  my_p4est_semi_lagrangian_t(lsg_forest* forest_np1, my_p4est_node_neighbors_t* ngbd_n, my_p4est_node_neighbors_t* ngbd_nm1)
      : forest_np1_(forest_np1), ngbd_n_(ngbd_n), ngbd_nm1_(ngbd_nm1) {}
  void set_splitting(int min_lvl, int max_lvl, double lip) {
    min_lvl_ = min_lvl;
    max_lvl_ = max_lvl;
    lip_ = lip;
  }
  // update_p4est(v, dt, phi) (src/my_p4est_semi_lagrangian.cpp:394-529) with node velocities v[D] of
  // grid n: phi is advected onto forest_np1, which is refined and coarsened from the advected values
  // until it no longer changes; phi is then replaced by its values at the final nodes. Returns the number
  // of advection passes.
  // phi_xx: phi's second derivatives on grid n (computed when null); band: the splitting criterion's band.
  // phi_add_refine: an extra field of grid n whose |value| also drives the refinement.
  int update_p4est(Vec* v, double dt, Vec& phi, Vec* phi_xx = nullptr, Vec phi_add_refine = nullptr, const double& band = 0) {
    const int D = ngbd_n_->dim();
    const size_t N = (size_t)ngbd_n_->num_nodes();
    std::vector<double> vv((size_t)D * N), vdd((size_t)D * D * N);
    for (int a = 0; a < D; ++a) {
      lsgpu::VecArray x(v[a]);
      for (size_t n = 0; n < N; ++n) vv[a * N + n] = x.p[n];
    }
    // the velocity's second derivatives on grid n once, as the reference computes them once
    for (int a = 0; a < D; ++a) lsgpu::check(lsg_second_derivatives(ngbd_n_->device(), &vv[a * N], &vdd[(size_t)a * D * N]));
    return regrid(dt, phi, phi_xx, phi_add_refine, band, [&](const std::vector<double>& xyz, const std::vector<double>& pn,
                                                              const std::vector<double>& pdd, std::vector<double>& out) {
      lsgpu::check(lsg_semi_lagrangian_advect(ngbd_n_->device(), xyz.data(), (int64_t)out.size(), dt, vv.data(), vdd.data(), pn.data(),
                                              pdd.data(), (int)velo_, (int)phi_, out.data()));
    });
  }
  // update_p4est(vnm1, vn, dt_nm1, dt_n, phi, phi_xx, phi_add_refine) (src/my_p4est_semi_lagrangian.cpp:779-939):
  // the two-velocity second-order step (vn[D] on grid n, vnm1[D] on grid n-1) repeated while forest_np1 is
  // refined and coarsened from the advected values (or from min(|phi_np1|, |phi_add_refine|) with
  // phi_add_refine on grid n interpolated linearly); phi then holds the values at the final nodes.
  int update_p4est(Vec* vnm1, Vec* vn, double dt_nm1, double dt_n, Vec& phi, Vec* phi_xx = nullptr, Vec phi_add_refine = nullptr) {
    if (!ngbd_nm1_) throw std::invalid_argument("update_p4est: the two-velocity form needs the grid at n-1 (ngbd_nm1)");
    const int D = ngbd_n_->dim();
    const size_t N = (size_t)ngbd_n_->num_nodes(), Nm = (size_t)ngbd_nm1_->num_nodes();
    std::vector<double> vn_v = gather(vn, D, N), vm_v = gather(vnm1, D, Nm), vn_dd((size_t)D * D * N), vm_dd((size_t)D * D * Nm);
    for (int a = 0; a < D; ++a) {
      lsgpu::check(lsg_second_derivatives(ngbd_n_->device(), &vn_v[a * N], &vn_dd[(size_t)a * D * N]));
      lsgpu::check(lsg_second_derivatives(ngbd_nm1_->device(), &vm_v[a * Nm], &vm_dd[(size_t)a * D * Nm]));
    }
    return regrid(dt_n, phi, phi_xx, phi_add_refine, 0.0, [&](const std::vector<double>& xyz, const std::vector<double>& pn,
                                                              const std::vector<double>& pdd, std::vector<double>& out) {
      lsgpu::check(lsg_semi_lagrangian_advect2(ngbd_n_->device(), ngbd_nm1_->device(), xyz.data(), (int64_t)out.size(), dt_nm1, dt_n,
                                               vm_v.data(), vm_dd.data(), vn_v.data(), vn_dd.data(), pn.data(), pdd.data(), (int)velo_,
                                               (int)phi_, out.data()));
    });
  }
  // update_p4est(const CF** v, dt, phi, phi_xx) (src/my_p4est_semi_lagrangian.cpp:321-392): v[D] function
  // objects of the coordinates, evaluated on the host at the nodes of grid n+1 and at the midpoints.
  template <typename CF>
  int update_p4est(const CF* const* v, double dt, Vec& phi, Vec* phi_xx = nullptr) {
    struct Ctx {
      const CF* const* v;
      int D;
    } ctx{v, ngbd_n_->dim()};
    lsg_velocity_fn fn = [](void* c, int64_t npts, const double* xyz, double* out) -> int {
      const Ctx* k = static_cast<const Ctx*>(c);
      try {
        for (int64_t p = 0; p < npts; ++p)
          for (int a = 0; a < k->D; ++a) out[p * k->D + a] = lsgpu::eval_cf(*k->v[a], &xyz[p * k->D], k->D);
      } catch (...) {
        return 1;
      }
      return 0;
    };
    return regrid(dt, phi, phi_xx, nullptr, 0.0, [&](const std::vector<double>& xyz, const std::vector<double>& pn,
                                                       const std::vector<double>& pdd, std::vector<double>& out) {
      lsgpu::check(lsg_semi_lagrangian_advect_callback(ngbd_n_->device(), xyz.data(), (int64_t)out.size(), dt, fn, &ctx, pn.data(),
                                                       pdd.data(), (int)phi_, out.data()));
    });
  }
  void set_velo_interpolation(interpolation_method m) { velo_ = m; }
  void set_phi_interpolation(interpolation_method m) { phi_ = m; }
  // advect_from_n_to_np1(dt, v, vxx, phi_n, phi_xx_n, phi_np1): v[D] node velocities of grid n;
  // vxx[D][D] and phi_xx_n[D] may be null (computed); phi_np1 has one value per node of grid n+1.
  void advect_from_n_to_np1(double dt, Vec* v, Vec** vxx, Vec phi_n, Vec* phi_xx_n, double* phi_np1) const {
    const int D = ngbd_n_->dim();
    const size_t N = (size_t)ngbd_n_->num_nodes();
    std::vector<double> vv((size_t)D * N), vdd, pdd;
    for (int a = 0; a < D; ++a) {
      lsgpu::VecArray x(v[a]);
      for (size_t n = 0; n < N; ++n) vv[a * N + n] = x.p[n];
    }
    if (vxx) {
      vdd.resize((size_t)D * D * N);
      for (int c = 0; c < D; ++c)
        for (int a = 0; a < D; ++a) {
          lsgpu::VecArray x(vxx[c][a]);
          for (size_t n = 0; n < N; ++n) vdd[((size_t)c * D + a) * N + n] = x.p[n];
        }
    }
    if (phi_xx_n) {
      pdd.resize((size_t)D * N);
      for (int a = 0; a < D; ++a) {
        lsgpu::VecArray x(phi_xx_n[a]);
        for (size_t n = 0; n < N; ++n) pdd[a * N + n] = x.p[n];
      }
    }
    const int64_t np = lsg_forest_num_nodes(forest_np1_);
    std::vector<double> xyz((size_t)np * D);
    lsgpu::check(lsg_forest_node_xyz(forest_np1_, xyz.data()));
    lsgpu::VecArray p(phi_n);
    lsgpu::check(lsg_semi_lagrangian_advect(ngbd_n_->device(), xyz.data(), np, dt, vv.data(), vdd.empty() ? nullptr : vdd.data(), p.p,
                                            pdd.empty() ? nullptr : pdd.data(), (int)velo_, (int)phi_, phi_np1));
  }
  // advect_from_n_to_np1(dt_nm1, dt_n, vnm1, vxx_nm1, vn, vxx_n, phi_n, phi_xx_n, phi_np1)
  // (src/my_p4est_semi_lagrangian.cpp:225-319): vnm1[D] on grid n-1, vn[D] and phi_n on grid n; vxx_nm1,
  // vxx_n ([D][D]) and phi_xx_n ([D]) may be null (computed); phi_np1 has one value per node of grid n+1.
  void advect_from_n_to_np1(double dt_nm1, double dt_n, Vec* vnm1, Vec** vxx_nm1, Vec* vn, Vec** vxx_n, Vec phi_n, Vec* phi_xx_n,
                            double* phi_np1) const {
    if (!ngbd_nm1_) throw std::invalid_argument("advect_from_n_to_np1: the two-velocity form needs the grid at n-1 (ngbd_nm1)");
    const int D = ngbd_n_->dim();
    const size_t N = (size_t)ngbd_n_->num_nodes(), Nm = (size_t)ngbd_nm1_->num_nodes();
    std::vector<double> vn_v = gather(vn, D, N), vm_v = gather(vnm1, D, Nm), vn_dd, vm_dd, pdd;
    if (vxx_n) vn_dd = gather2(vxx_n, D, N);
    if (vxx_nm1) vm_dd = gather2(vxx_nm1, D, Nm);
    if (phi_xx_n) pdd = gather(phi_xx_n, D, N);
    const int64_t np = lsg_forest_num_nodes(forest_np1_);
    std::vector<double> xyz((size_t)np * D);
    lsgpu::check(lsg_forest_node_xyz(forest_np1_, xyz.data()));
    lsgpu::VecArray p(phi_n);
    lsgpu::check(lsg_semi_lagrangian_advect2(ngbd_n_->device(), ngbd_nm1_->device(), xyz.data(), np, dt_nm1, dt_n, vm_v.data(),
                                             vm_dd.empty() ? nullptr : vm_dd.data(), vn_v.data(), vn_dd.empty() ? nullptr : vn_dd.data(), p.p,
                                             pdd.empty() ? nullptr : pdd.data(), (int)velo_, (int)phi_, phi_np1));
  }
  // advect_from_n_to_np1(dt, const CF** v, phi_n, phi_xx_n, phi_np1): v[D] function objects of the
  // coordinates, evaluated on the host at the nodes of grid n+1 and at the midpoints.
  template <typename CF>
  void advect_from_n_to_np1(double dt, const CF* const* v, Vec phi_n, Vec* phi_xx_n, double* phi_np1) const {
    const int D = ngbd_n_->dim();
    const size_t N = (size_t)ngbd_n_->num_nodes();
    std::vector<double> pdd;
    if (phi_xx_n) {
      pdd.resize((size_t)D * N);
      for (int a = 0; a < D; ++a) {
        lsgpu::VecArray x(phi_xx_n[a]);
        for (size_t n = 0; n < N; ++n) pdd[a * N + n] = x.p[n];
      }
    }
    struct Ctx {
      const CF* const* v;
      int D;
    } ctx{v, D};
    lsg_velocity_fn fn = [](void* c, int64_t npts, const double* xyz, double* out) -> int {
      const Ctx* k = static_cast<const Ctx*>(c);
      try {
        for (int64_t p = 0; p < npts; ++p)
          for (int a = 0; a < k->D; ++a) out[p * k->D + a] = lsgpu::eval_cf(*k->v[a], &xyz[p * k->D], k->D);
      } catch (...) {
        return 1;
      }
      return 0;
    };
    const int64_t np = lsg_forest_num_nodes(forest_np1_);
    std::vector<double> xyz((size_t)np * D);
    lsgpu::check(lsg_forest_node_xyz(forest_np1_, xyz.data()));
    lsgpu::VecArray p(phi_n);
    lsgpu::check(lsg_semi_lagrangian_advect_callback(ngbd_n_->device(), xyz.data(), np, dt, fn, &ctx, p.p, pdd.empty() ? nullptr : pdd.data(),
                                                     (int)phi_, phi_np1));
  }

 private:
  // D vectors of n values each, packed component after component
  static std::vector<double> gather(Vec* v, int D, size_t n) {
    std::vector<double> out((size_t)D * n);
    for (int a = 0; a < D; ++a) {
      lsgpu::VecArray x(v[a]);
      for (size_t i = 0; i < n; ++i) out[a * n + i] = x.p[i];
    }
    return out;
  }
  // D x D vectors (component, derivative axis) of n values each
  static std::vector<double> gather2(Vec** v, int D, size_t n) {
    std::vector<double> out((size_t)D * D * n);
    for (int c = 0; c < D; ++c)
      for (int a = 0; a < D; ++a) {
        lsgpu::VecArray x(v[c][a]);
        for (size_t i = 0; i < n; ++i) out[((size_t)c * D + a) * n + i] = x.p[i];
      }
    return out;
  }
  // advect phi onto forest_np1 with `advect`, refine/coarsen from the result (or from
  // min(|result|, |phi_add_refine|), phi_add_refine on grid n interpolated linearly at the new nodes),
  // repeat until the grid settles; phi becomes the values at the final nodes
  template <typename Advect>
  int regrid(double dt, Vec& phi, Vec* phi_xx, Vec phi_add_refine, double band, Advect advect) {
    (void)dt;
    if (max_lvl_ < 0) throw std::invalid_argument("update_p4est: set the splitting criterion first");
    const int D = ngbd_n_->dim();
    const size_t N = (size_t)ngbd_n_->num_nodes();
    std::vector<double> pn(N), pdd((size_t)D * N);
    {
      lsgpu::VecArray p(phi);
      for (size_t n = 0; n < N; ++n) pn[n] = p.p[n];
    }
    if (phi_xx) {
      for (int a = 0; a < D; ++a) {
        lsgpu::VecArray x(phi_xx[a]);
        for (size_t n = 0; n < N; ++n) pdd[a * N + n] = x.p[n];
      }
    } else {
      lsgpu::check(lsg_second_derivatives(ngbd_n_->device(), pn.data(), pdd.data()));
    }
    std::vector<double> out, xyz;
    int passes = 0;
    for (;;) {
      if (lsg_forest_num_nodes(forest_np1_) < 0) lsgpu::check(lsg_forest_build_nodes(forest_np1_));
      const int64_t np = lsg_forest_num_nodes(forest_np1_);
      xyz.resize((size_t)np * D);
      out.resize((size_t)np);
      lsgpu::check(lsg_forest_node_xyz(forest_np1_, xyz.data()));
      advect(xyz, pn, pdd, out);
      ++passes;
      int changed = 0;
      const double* tag_from = out.data();
      std::vector<double> eff;
      if (phi_add_refine != nullptr) {
        eff.resize((size_t)np);
        lsgpu::VecArray add(phi_add_refine);
        lsgpu::check(lsg_interpolate_nodes(ngbd_n_->device(), xyz.data(), np, add.p, 1, nullptr, (int)linear, eff.data()));
        for (int64_t n = 0; n < np; ++n) eff[(size_t)n] = std::min(std::fabs(eff[(size_t)n]), std::fabs(out[(size_t)n]));
        tag_from = eff.data();
      }
      lsgpu::check(lsg_forest_refine_and_coarsen(forest_np1_, min_lvl_, max_lvl_, lip_, band, tag_from, &changed));
      if (!changed) break;
      lsgpu::check(lsg_forest_build_nodes(forest_np1_));
    }
#ifdef LSGPU_WITH_PETSC
    VecDestroy(&phi);
    VecCreateSeq(PETSC_COMM_SELF, (PetscInt)out.size(), &phi);
    lsgpu::VecArray p(phi);
    for (size_t n = 0; n < out.size(); ++n) p.p[n] = out[n];
#else
    phi->values = out;
#endif
    return passes;
  }

  lsg_forest* forest_np1_;
  my_p4est_node_neighbors_t* ngbd_n_;
  my_p4est_node_neighbors_t* ngbd_nm1_ = nullptr;
  int min_lvl_ = 0, max_lvl_ = -1;
  double lip_ = 1.2;
  interpolation_method velo_ = quadratic_non_oscillatory_continuous_v2;
  interpolation_method phi_ = quadratic_non_oscillatory_continuous_v2;
};

#endif  // LSGPU_HPP
