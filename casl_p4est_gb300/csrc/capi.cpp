// extern "C" boundary (include/lsgpu.h): argument checks, dimension dispatch and error capture.
#include <float.h>
#include <string.h>

#include <exception>
#include <new>
#include <string>
#include <type_traits>
#include <vector>

#include "../../include/lsgpu.h"
#include "flatten.hpp"
#include "io.hpp"
#include "level_set.hpp"
#include "shapes.h"

using namespace lsg;

struct lsg_forest {
  int dim = 2;
  Forest<2>* f2 = nullptr;
  Forest<3>* f3 = nullptr;
  ~lsg_forest() {
    delete f2;
    delete f3;
  }
};

// A level set lives on the device that was current when it was created: every call on it runs there
// (the caller's current device is restored afterwards), whatever device the caller has current.
struct lsg_level_set {
  int dim = 2;
  int device = 0;
  LevelSet<2>* l2 = nullptr;
  LevelSet<3>* l3 = nullptr;
  ~lsg_level_set() {
    int prev = 0;
    const bool switched = cudaGetDevice(&prev) == cudaSuccess && prev != device && cudaSetDevice(device) == cudaSuccess;
    delete l2;
    delete l3;
    if (switched) cudaSetDevice(prev);
  }
};

namespace {

thread_local std::string g_last_error;

struct InvalidArg : std::invalid_argument {
  using std::invalid_argument::invalid_argument;
};
struct StateError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

template <typename Fn>
int guard(Fn&& fn) {
  try {
    fn();
    return LSG_OK;
  } catch (const CudaOutOfMemory& e) {
    g_last_error = e.what();
    return LSG_ENOMEM;
  } catch (const DeviceTimeout& e) {
    g_last_error = e.what();
    return LSG_ETIMEOUT;
  } catch (const CudaError& e) {
    g_last_error = e.what();
    return LSG_EDEVICE;
  } catch (const StateError& e) {
    g_last_error = e.what();
    return LSG_ESTATE;
  } catch (const std::bad_alloc&) {
    g_last_error = "allocation failed";
    return LSG_ENOMEM;
  } catch (const std::invalid_argument& e) {
    g_last_error = e.what();
    return LSG_EINVAL;
  } catch (const std::exception& e) {
    g_last_error = e.what();
    return LSG_EDEVICE;
  } catch (...) {
    g_last_error = "unknown error";
    return LSG_EDEVICE;
  }
}

void need(bool cond, const char* msg) {
  if (!cond) throw InvalidArg(msg);
}

template <typename Fn>
void with_forest(const lsg_forest* f, Fn&& fn) {
  need(f != nullptr, "null forest");
  if (f->dim == 2)
    fn(*f->f2);
  else
    fn(*f->f3);
}

template <typename Fn>
void with_ls(lsg_level_set* ls, Fn&& fn) {
  need(ls != nullptr, "null level set");
  DeviceGuard on(ls->device);
  if (ls->dim == 2)
    fn(*ls->l2);
  else
    fn(*ls->l3);
}

// the two level sets of a two-velocity step: same dimension, same device
template <typename Fn>
void with_ls_pair(lsg_level_set* n, lsg_level_set* nm1, Fn&& fn) {
  need(n != nullptr && nm1 != nullptr, "null level set");
  need(n->dim == nm1->dim, "the grids at n and n-1 must have the same dimension");
  need(n->device == nm1->device, "the grids at n and n-1 must live on the same device");
  DeviceGuard on(n->device);
  if (n->dim == 2)
    fn(*n->l2, *nm1->l2);
  else
    fn(*n->l3, *nm1->l3);
}

template <int D>
void need_nodes(const Forest<D>& F) {
  if (!F.nodes_built) throw StateError("the forest's nodes are not built (call lsg_forest_build_nodes)");
}

// refine_levelset_cf (src/my_p4est_refine_coarsen.cpp:18-90) with refine_only_inside = false.
template <int D>
void tag_levelset(const Forest<D>& F, int min_lvl, int max_lvl, double lip, double band_rel, int shape, const double* params,
                  uint8_t* tags) {
  using DD = Dim<D>;
  const size_t nl = F.leaves.size();
#pragma omp parallel for schedule(dynamic, 1024)
  for (long long ii = 0; ii < (long long)nl; ++ii) {
    const Quad& qd = F.leaves[(size_t)ii];
    uint8_t tag = 0;
    if (qd.level < min_lvl) {
      tag = 1;
    } else if (qd.level >= max_lvl) {
      tag = 0;
    } else {
      const int t = qd.tree;
      double tmin[3], tmax[3];
      for (int a = 0; a < 3; ++a) {
        tmin[a] = F.brick.tmin[3 * t + a];
        tmax[a] = F.brick.tmax[3 * t + a];
      }
      const double dmin = (double)quadrant_len(DD::MAXLEVEL, qd.level) / (double)DD::ROOT_LEN;
      double dxyz[3];
      for (int a = 0; a < D; ++a) dxyz[a] = (tmax[a] - tmin[a]) * dmin;
      double smallest = max2(tmax[0] - tmin[0], tmax[1] - tmin[1]) * ((double)quadrant_len(DD::MAXLEVEL, max_lvl)) / ((double)DD::ROOT_LEN);
      if (D == 3)
        smallest = max2(smallest, (tmax[2] - tmin[2]) * ((double)quadrant_len(DD::MAXLEVEL, max_lvl)) / ((double)DD::ROOT_LEN));
      const double dd = (D == 3) ? sqrt(dxyz[0] * dxyz[0] + dxyz[1] * dxyz[1] + dxyz[2] * dxyz[2])
                                 : sqrt(dxyz[0] * dxyz[0] + dxyz[1] * dxyz[1]);
      double xq[3];
      for (int a = 0; a < D; ++a) xq[a] = (tmax[a] - tmin[a]) * (double)qd.x[a] / (double)DD::ROOT_LEN + tmin[a];
      const double band = band_rel * smallest;
      double fv[8];
      for (int c = 0; c < DD::CHILDREN && !tag; ++c) {
        double p[3];
        for (int a = 0; a < D; ++a) p[a] = xq[a] + ((c >> a) & 1) * dxyz[a];
        fv[c] = shape_eval<D>(shape, params, p);
        if (fabs(fv[c]) - band <= 0.5 * lip * dd) tag = 1;
      }
      if (!tag) {
        if (D == 3) {
          if (fv[0] * fv[1] < 0 || fv[0] * fv[2] < 0 || fv[1] * fv[3] < 0 || fv[2] * fv[3] < 0 || fv[3] * fv[4] < 0 ||
              fv[4] * fv[5] < 0 || fv[5] * fv[6] < 0 || fv[6] * fv[7] < 0)
            tag = 1;
        } else {
          if (fv[0] * fv[1] < 0 || fv[0] * fv[2] < 0 || fv[1] * fv[3] < 0 || fv[2] * fv[3] < 0) tag = 1;
        }
      }
    }
    tags[ii] = tag;
  }
}

// Host forms of the derivative family: inputs of n_in x N doubles, outputs of n_out x N (+ N).
template <typename L, typename Fn>
void host_fields(L& ls, const double* in, size_t n_in, double* out, size_t n_out, double* out2, Fn&& fn) {
  const size_t N = (size_t)ls.N;
  ls.ws_f.ensure(n_in * N + (n_out + (out2 ? 1 : 0)) * N + 1);
  double* din = ls.ws_f.p;
  double* dout = din + n_in * N;
  double* dout2 = dout + n_out * N;
  if (N) cuda_check(cudaMemcpyAsync(din, in, n_in * N * sizeof(double), cudaMemcpyHostToDevice, ls.stream), "H2D");
  fn(din, dout, dout2);
  if (N) cuda_check(cudaMemcpyAsync(out, dout, n_out * N * sizeof(double), cudaMemcpyDeviceToHost, ls.stream), "D2H");
  if (N && out2) cuda_check(cudaMemcpyAsync(out2, dout2, N * sizeof(double), cudaMemcpyDeviceToHost, ls.stream), "D2H");
  cuda_check(cudaStreamSynchronize(ls.stream), "sync");
}

}  // namespace

extern "C" {

const char* lsg_last_error(void) { return g_last_error.c_str(); }
int lsg_version(void) { return 1; }

int lsg_forest_create(int dim, const int n_xyz[3], const double xyz_min[3], const double xyz_max[3], const int periodic[3],
                      lsg_forest** out) {
  return guard([&] {
    need(out != nullptr, "null output pointer");
    need(dim == 2 || dim == 3, "dim must be 2 or 3");
    need(n_xyz && xyz_min && xyz_max, "null brick description");
    lsg_forest* f = new lsg_forest();
    f->dim = dim;
    try {
      if (dim == 2) {
        f->f2 = new Forest<2>();
        f->f2->init(n_xyz, xyz_min, xyz_max, periodic);
      } else {
        f->f3 = new Forest<3>();
        f->f3->init(n_xyz, xyz_min, xyz_max, periodic);
      }
    } catch (...) {
      delete f;
      throw;
    }
    *out = f;
  });
}

int lsg_forest_destroy(lsg_forest* f) {
  return guard([&] { delete f; });
}

int lsg_forest_dim(const lsg_forest* f) { return f ? f->dim : 0; }

int64_t lsg_forest_num_leaves(const lsg_forest* f) {
  int64_t n = -1;
  guard([&] { with_forest(f, [&](auto& F) { n = (int64_t)F.num_leaves(); }); });
  return n;
}

int lsg_forest_leaves(const lsg_forest* f, int32_t* tree, int32_t* level, int32_t* xyz) {
  return guard([&] {
    with_forest(f, [&](auto& F) {
      for (size_t i = 0; i < F.leaves.size(); ++i) {
        const Quad& q = F.leaves[i];
        if (tree) tree[i] = q.tree;
        if (level) level[i] = q.level;
        if (xyz)
          for (int a = 0; a < 3; ++a) xyz[3 * i + a] = q.x[a];
      }
    });
  });
}

int lsg_forest_refine(lsg_forest* f, const uint8_t* tags, int64_t n) {
  return guard([&] {
    with_forest(f, [&](auto& F) {
      need(tags != nullptr && n == (int64_t)F.num_leaves(), "refine: one tag per leaf required");
      F.refine(tags);
    });
  });
}

int lsg_forest_coarsen(lsg_forest* f, const uint8_t* tags, int64_t n) {
  return guard([&] {
    with_forest(f, [&](auto& F) {
      need(tags != nullptr && n == (int64_t)F.num_leaves(), "coarsen: one tag per leaf required");
      F.coarsen(tags);
    });
  });
}

int lsg_forest_copy(const lsg_forest* f, lsg_forest** out) {
  return guard([&] {
    need(f != nullptr && out != nullptr, "null argument");
    lsg_forest* c = new lsg_forest();
    c->dim = f->dim;
    try {
      if (f->dim == 2)
        c->f2 = new Forest<2>(*f->f2);
      else
        c->f3 = new Forest<3>(*f->f3);
    } catch (...) {
      delete c;
      throw;
    }
    *out = c;
  });
}

int lsg_forest_set_leaves(lsg_forest* f, int64_t n, const int32_t* tree, const int32_t* level, const int32_t* xyz) {
  return guard([&] {
    need(tree != nullptr && level != nullptr && xyz != nullptr && n > 0, "set_leaves: null arguments");
    with_forest(f, [&](auto& F) { F.set_leaves((size_t)n, tree, level, xyz); });
  });
}

int lsg_forest_refine_and_coarsen(lsg_forest* f, int min_lvl, int max_lvl, double lip, double band, const double* phi,
                                  int* changed) {
  return guard([&] {
    need(phi != nullptr && changed != nullptr, "refine_and_coarsen: null arguments");
    need(min_lvl >= 0 && min_lvl <= max_lvl, "refine_and_coarsen: need 0 <= min_lvl <= max_lvl");
    with_forest(f, [&](auto& F) {
      using FT = std::decay_t<decltype(F)>;
      need(max_lvl <= FT::DD::QMAXLEVEL, "refine_and_coarsen: max_lvl above the maximum quadrant level");
      need_nodes(F);
      std::vector<int8_t> tag(F.num_leaves());
      F.tag_refine_coarsen(min_lvl, max_lvl, lip, band, phi, tag.data());
      *changed = F.coarsen_then_refine(tag.data()) ? 1 : 0;
    });
  });
}

int lsg_forest_tag_levelset(const lsg_forest* f, int min_lvl, int max_lvl, double lip, double band, int shape,
                            const double* params, int nparams, uint8_t* tags) {
  return guard([&] {
    need(params != nullptr && nparams > 0 && tags != nullptr, "tag_levelset: null arguments");
    need(min_lvl >= 0 && min_lvl <= max_lvl, "tag_levelset: need 0 <= min_lvl <= max_lvl");
    with_forest(f, [&](auto& F) {
      using FT = std::decay_t<decltype(F)>;
      need(max_lvl <= FT::DD::QMAXLEVEL, "tag_levelset: max_lvl above the maximum quadrant level");
      tag_levelset(F, min_lvl, max_lvl, lip, band, shape, params, tags);
    });
  });
}

int lsg_forest_refine_levelset(lsg_forest* f, int min_lvl, int max_lvl, double lip, double band, int shape,
                               const double* params, int nparams, int passes) {
  return guard([&] {
    need(params != nullptr && nparams > 0, "refine_levelset: null params");
    need(min_lvl >= 0 && min_lvl <= max_lvl, "refine_levelset: need 0 <= min_lvl <= max_lvl");
    with_forest(f, [&](auto& F) {
      using FT = std::decay_t<decltype(F)>;
      need(max_lvl <= FT::DD::QMAXLEVEL, "refine_levelset: max_lvl above the maximum quadrant level");
      for (int p = 0; p < passes; ++p) {
        std::vector<uint8_t> tags(F.num_leaves());
        tag_levelset(F, min_lvl, max_lvl, lip, band, shape, params, tags.data());
        bool any = false;
        for (uint8_t t : tags) any = any || t;
        if (!any) break;
        F.refine(tags.data());
      }
    });
  });
}

int lsg_forest_build_nodes(lsg_forest* f) {
  return guard([&] { with_forest(f, [&](auto& F) { const_cast<std::decay_t<decltype(F)>&>(F).build_nodes(); }); });
}

int lsg_forest_build_nodes_device(lsg_forest* f, void* stream) {
  return guard([&] {
    with_forest(f, [&](auto& F) { build_nodes_device(const_cast<std::decay_t<decltype(F)>&>(F), (cudaStream_t)stream); });
  });
}

int lsg_forest_node_xyz_device(lsg_forest* f, double* xyz_dev, void* stream) {
  return guard([&] {
    need(xyz_dev != nullptr, "null output");
    with_forest(f, [&](auto& F) {
      need_nodes(F);
      node_xyz_device(const_cast<std::decay_t<decltype(F)>&>(F), xyz_dev, (cudaStream_t)stream);
    });
  });
}

int lsg_forest_refine_and_coarsen_device(lsg_forest* f, int min_lvl, int max_lvl, double lip, double band, const double* phi_dev,
                                         int* changed, void* stream) {
  return guard([&] {
    need(phi_dev != nullptr && changed != nullptr, "refine_and_coarsen: null arguments");
    need(min_lvl >= 0 && min_lvl <= max_lvl, "refine_and_coarsen: need 0 <= min_lvl <= max_lvl");
    with_forest(f, [&](auto& F) {
      using FT = std::decay_t<decltype(F)>;
      need(max_lvl <= FT::DD::QMAXLEVEL, "refine_and_coarsen: max_lvl above the maximum quadrant level");
      need_nodes(F);
      *changed = refine_and_coarsen_device(const_cast<FT&>(F), min_lvl, max_lvl, lip, band, phi_dev, (cudaStream_t)stream) ? 1 : 0;
    });
  });
}

int lsg_vtk_write_all(const lsg_forest* f, const char* filename, int write_tree, int num_point, const char* const* point_names,
                      const double* const* point_values, int num_cell, const char* const* cell_names, const double* const* cell_values,
                      int binary) {
  return guard([&] {
    need(filename != nullptr && num_point >= 0 && num_cell >= 0, "vtk: bad arguments");
    need(num_point == 0 || (point_names != nullptr && point_values != nullptr), "vtk: null point data");
    need(num_cell == 0 || (cell_names != nullptr && cell_values != nullptr), "vtk: null cell data");
    std::vector<std::string> pn, cn;
    std::vector<const double*> pv, cv;
    for (int k = 0; k < num_point; ++k) {
      need(point_names[k] != nullptr && point_values[k] != nullptr, "vtk: null point field");
      pn.push_back(point_names[k]);
      pv.push_back(point_values[k]);
    }
    for (int k = 0; k < num_cell; ++k) {
      need(cell_names[k] != nullptr && cell_values[k] != nullptr, "vtk: null cell field");
      cn.push_back(cell_names[k]);
      cv.push_back(cell_values[k]);
    }
    with_forest(f, [&](auto& F) {
      need_nodes(F);
      vtk_write_all(F, filename, write_tree != 0, pn, pv, cn, cv, binary != 0);
    });
  });
}

int lsg_vec_dump(const char* fname, int nvecs, const double* const* vecs, int64_t n, int petsc_int64) {
  return guard([&] {
    need(fname != nullptr && nvecs >= 1 && vecs != nullptr && n >= 0, "VecDump: bad arguments");
    std::vector<const double*> v(vecs, vecs + nvecs);
    for (const double* p : v) need(p != nullptr || n == 0, "VecDump: null vector");
    vec_dump(fname, v, n, petsc_int64 != 0);
  });
}

int lsg_vec_load(const char* fname, int nvecs, double* const* vecs, int64_t n, int petsc_int64) {
  return guard([&] {
    need(fname != nullptr && nvecs >= 1 && vecs != nullptr && n >= 0, "VecLoad: bad arguments");
    std::vector<double*> v(vecs, vecs + nvecs);
    for (double* p : v) need(p != nullptr || n == 0, "VecLoad: null vector");
    vec_load(fname, v, n, petsc_int64 != 0);
  });
}

int lsg_forest_save(const lsg_forest* f, const char* fname) {
  return guard([&] {
    need(fname != nullptr, "forest save: null file name");
    with_forest(f, [&](auto& F) { forest_save(F, fname); });
  });
}

int lsg_forest_load(const char* fname, lsg_forest** out) {
  return guard([&] {
    need(fname != nullptr && out != nullptr, "forest load: null argument");
    int dim = 0, n[3] = {1, 1, 1};
    double lo[3], hi[3];
    int64_t nl = 0;
    forest_header(fname, &dim, n, lo, hi, &nl);
    lsg_forest* f = new lsg_forest();
    f->dim = dim;
    try {
      if (dim == 2) {
        f->f2 = new Forest<2>();
        f->f2->init(n, lo, hi, nullptr);
        forest_load_leaves(*f->f2, fname);
      } else {
        f->f3 = new Forest<3>();
        f->f3->init(n, lo, hi, nullptr);
        forest_load_leaves(*f->f3, fname);
      }
    } catch (...) {
      delete f;
      throw;
    }
    *out = f;
  });
}

int64_t lsg_forest_num_nodes(const lsg_forest* f) {
  int64_t n = -1;
  guard([&] {
    with_forest(f, [&](auto& F) {
      need_nodes(F);
      n = (int64_t)F.num_nodes();
    });
  });
  return n;
}

int lsg_forest_node_xyz(const lsg_forest* f, double* xyz) {
  return guard([&] {
    need(xyz != nullptr, "null output");
    with_forest(f, [&](auto& F) {
      need_nodes(F);
      using FT = std::decay_t<decltype(F)>;
      constexpr int D = FT::DD::CHILDREN == 4 ? 2 : 3;
#pragma omp parallel for schedule(static)
      for (long long n = 0; n < (long long)F.num_nodes(); ++n) F.node_xyz((int32_t)n, xyz + (size_t)D * n);
    });
  });
}

int lsg_forest_nodes(const lsg_forest* f, int32_t* tree, int32_t* xyz) {
  return guard([&] {
    with_forest(f, [&](auto& F) {
      need_nodes(F);
      using FT = std::decay_t<decltype(F)>;
      constexpr int D = FT::DD::CHILDREN == 4 ? 2 : 3;
      for (size_t n = 0; n < F.num_nodes(); ++n) {
        if (tree) tree[n] = F.nd->host().node_tree[n];
        if (xyz)
          for (int a = 0; a < 3; ++a) xyz[3 * n + a] = a < D ? F.nd->host().node_x[D * n + a] : 0;
      }
    });
  });
}

int lsg_forest_local_nodes(const lsg_forest* f, int32_t* out) {
  return guard([&] {
    need(out != nullptr, "null output");
    with_forest(f, [&](auto& F) {
      need_nodes(F);
      memcpy(out, F.nd->host().local_nodes.data(), F.nd->host().local_nodes.size() * sizeof(int32_t));
    });
  });
}

int lsg_forest_sample_shape(const lsg_forest* f, int shape, const double* params, int nparams, double* out) {
  return guard([&] {
    need(params != nullptr && nparams > 0 && out != nullptr, "sample_shape: null arguments");
    with_forest(f, [&](auto& F) {
      need_nodes(F);
      using FT = std::decay_t<decltype(F)>;
      constexpr int D = FT::DD::CHILDREN == 4 ? 2 : 3;
#pragma omp parallel for schedule(static)
      for (long long n = 0; n < (long long)F.num_nodes(); ++n) {
        double x[3] = {0, 0, 0};
        F.node_xyz((int32_t)n, x);
        out[n] = shape_eval<D>(shape, params, x);
      }
    });
  });
}

size_t lsg_qnnn_record_bytes(int dim) { return dim == 2 ? sizeof(Qnnn<2>) : (dim == 3 ? sizeof(Qnnn<3>) : 0); }

int lsg_forest_export_qnnn(const lsg_forest* f, int64_t first, int64_t count, void* out, size_t record_bytes) {
  return guard([&] {
    need(out != nullptr, "null output");
    with_forest(f, [&](auto& F) {
      need_nodes(F);
      using FT = std::decay_t<decltype(F)>;
      constexpr int D = FT::DD::CHILDREN == 4 ? 2 : 3;
      need(record_bytes == sizeof(Qnnn<D>), "export_qnnn: record size mismatch");
      need(first >= 0 && count >= 0 && first + count <= (int64_t)F.num_nodes(), "export_qnnn: range outside the nodes");
      Qnnn<D>* rec = static_cast<Qnnn<D>*>(out);
      int failed = 0;
#pragma omp parallel for schedule(dynamic, 4096) reduction(+ : failed)
      for (long long i = 0; i < (long long)count; ++i) {
        memset(&rec[i], 0, sizeof(Qnnn<D>));
        if (construct_neighbors<D>(F, (int32_t)(first + i), rec[i])) ++failed;
      }
      if (failed) throw std::runtime_error("export_qnnn: incomplete stencil");
    });
  });
}

int lsg_forest_wall_mask(const lsg_forest* f, uint8_t* out) {
  return guard([&] {
    need(out != nullptr, "null output");
    with_forest(f, [&](auto& F) {
      need_nodes(F);
      using FT = std::decay_t<decltype(F)>;
      constexpr int D = FT::DD::CHILDREN == 4 ? 2 : 3;
      for (size_t n = 0; n < F.num_nodes(); ++n) out[n] = (uint8_t)wall_mask<D>(F, (int32_t)n);
    });
  });
}

int lsg_forest_dxyz_min(const lsg_forest* f, double* dxyz) {
  return guard([&] {
    need(dxyz != nullptr, "null output");
    with_forest(f, [&](auto& F) { F.dxyz_min(dxyz); });
  });
}

int lsg_level_set_create_ex(const lsg_forest* f, int flags, lsg_level_set** out) {
  return guard([&] {
    need(out != nullptr, "null output pointer");
    need(f != nullptr, "null forest");
    need((flags & ~LSG_BUILD_ON_DEVICE) == 0, "unknown level set flags");
    const bool on_device = (flags & LSG_BUILD_ON_DEVICE) != 0;
    lsg_level_set* ls = new lsg_level_set();
    ls->dim = f->dim;
    try {
      if (f->dim == 2) {
        need_nodes(*f->f2);
        ls->device = current_device();
        ls->l2 = new LevelSet<2>(*f->f2, true, on_device);
      } else {
        need_nodes(*f->f3);
        ls->device = current_device();
        ls->l3 = new LevelSet<3>(*f->f3, true, on_device);
      }
    } catch (...) {
      delete ls;
      throw;
    }
    *out = ls;
  });
}

int lsg_level_set_create(const lsg_forest* f, lsg_level_set** out) { return lsg_level_set_create_ex(f, 0, out); }

int lsg_level_set_destroy(lsg_level_set* ls) {
  return guard([&] { delete ls; });
}

int lsg_level_set_set_stream(lsg_level_set* ls, void* cuda_stream) {
  return guard([&] { with_ls(ls, [&](auto& L) { L.set_stream((cudaStream_t)cuda_stream); }); });
}

void* lsg_level_set_stream(const lsg_level_set* ls) {
  if (!ls) return nullptr;
  return ls->dim == 2 ? (void*)ls->l2->stream : (void*)ls->l3->stream;
}

int64_t lsg_level_set_num_nodes(const lsg_level_set* ls) {
  if (!ls) return -1;
  return ls->dim == 2 ? ls->l2->N : ls->l3->N;
}

double lsg_level_set_zero_distance_threshold(const lsg_level_set* ls) {
  if (!ls) return 0.0;
  return ls->dim == 2 ? ls->l2->zdt : ls->l3->zdt;
}

int lsg_reinitialize(lsg_level_set* ls, double* phi, int order_space, int order_pseudotime, double limit_high, double limit_low,
                     int iterations, int precision) {
  return guard([&] {
    need(phi != nullptr, "null phi");
    with_ls(ls, [&](auto& L) { L.reinitialize_host(phi, order_space, order_pseudotime, limit_high, limit_low, iterations, precision); });
  });
}

int lsg_reinitialize_device(lsg_level_set* ls, double* phi_dev, int order_space, int order_pseudotime, double limit_high,
                            double limit_low, int iterations, int precision) {
  return guard([&] {
    need(phi_dev != nullptr, "null phi");
    with_ls(ls, [&](auto& L) { L.reinitialize(phi_dev, order_space, order_pseudotime, limit_high, limit_low, iterations, precision); });
  });
}

int lsg_reinitialize_with_mask(lsg_level_set* ls, double* phi, const double* mask, int order_space, int order_pseudotime,
                               double limit_high, double limit_low, int iterations, int precision) {
  return guard([&] {
    need(phi != nullptr && mask != nullptr, "null phi or mask");
    with_ls(ls, [&](auto& L) {
      L.reinitialize_host(phi, order_space, order_pseudotime, limit_high, limit_low, iterations, precision, mask);
    });
  });
}

int lsg_reinitialize_with_mask_device(lsg_level_set* ls, double* phi_dev, const double* mask_dev, int order_space, int order_pseudotime,
                                      double limit_high, double limit_low, int iterations, int precision) {
  return guard([&] {
    need(phi_dev != nullptr && mask_dev != nullptr, "null phi or mask");
    with_ls(ls, [&](auto& L) {
      L.reinitialize(phi_dev, order_space, order_pseudotime, limit_high, limit_low, iterations, precision, mask_dev);
    });
  });
}

int lsg_reinitialize_device_noalloc(lsg_level_set* ls, double* phi_dev, int order_space, int order_pseudotime,
                                    double limit_high, double limit_low, int iterations) {
  return guard([&] {
    need(phi_dev != nullptr, "null phi");
    with_ls(ls, [&](auto& L) { L.reinitialize_fp64_noalloc(phi_dev, order_space, order_pseudotime, limit_high, limit_low, iterations); });
  });
}

int lsg_reinit_2nd(lsg_level_set* ls, double* phi, int iterations, double limit, int precision) {
  return lsg_reinitialize(ls, phi, 2, 2, limit, -limit, iterations, precision);
}

int lsg_advect_in_normal_direction_device(lsg_level_set* ls, const double* vn_dev, const double* vn_np1_dev, double* phi_dev,
                                          double dt, double* phi_dd_dev, int precision) {
  return guard([&] {
    need(vn_dev != nullptr && phi_dev != nullptr, "null vn or phi");
    with_ls(ls, [&](auto& L) { L.advect_normal(vn_dev, vn_np1_dev, phi_dev, dt, phi_dd_dev, precision); });
  });
}

int lsg_advect_in_normal_direction(lsg_level_set* ls, const double* vn, const double* vn_np1, double* phi, double dt,
                                   double* phi_dd, int precision) {
  return guard([&] {
    need(vn != nullptr && phi != nullptr, "null vn or phi");
    with_ls(ls, [&](auto& L) {
      using LT = std::decay_t<decltype(L)>;
      constexpr int D = LT::H == 2 ? 2 : 3;
      const int64_t N = L.N;
      L.ws_phi.alloc(N);
      L.ws_vn.alloc(N);
      if (vn_np1) L.ws_vn1.alloc(N);
      if (phi_dd) L.ws_dd.alloc((size_t)D * N);
      cudaStream_t s = L.stream;
      cuda_check(cudaMemcpyAsync(L.ws_phi.p, phi, N * sizeof(double), cudaMemcpyHostToDevice, s), "H2D");
      cuda_check(cudaMemcpyAsync(L.ws_vn.p, vn, N * sizeof(double), cudaMemcpyHostToDevice, s), "H2D");
      if (vn_np1) cuda_check(cudaMemcpyAsync(L.ws_vn1.p, vn_np1, N * sizeof(double), cudaMemcpyHostToDevice, s), "H2D");
      if (phi_dd) cuda_check(cudaMemcpyAsync(L.ws_dd.p, phi_dd, (size_t)D * N * sizeof(double), cudaMemcpyHostToDevice, s), "H2D");
      L.advect_normal(L.ws_vn.p, vn_np1 ? L.ws_vn1.p : nullptr, L.ws_phi.p, dt, phi_dd ? L.ws_dd.p : nullptr, precision);
      cuda_check(cudaMemcpyAsync(phi, L.ws_phi.p, N * sizeof(double), cudaMemcpyDeviceToHost, s), "D2H");
      if (phi_dd) cuda_check(cudaMemcpyAsync(phi_dd, L.ws_dd.p, (size_t)D * N * sizeof(double), cudaMemcpyDeviceToHost, s), "D2H");
      cuda_check(cudaStreamSynchronize(s), "advect sync");
    });
  });
}

int lsg_advect_cfl_dt(lsg_level_set* ls, const double* vn, double* dt_out) {
  return guard([&] {
    need(vn != nullptr && dt_out != nullptr, "null argument");
    with_ls(ls, [&](auto& L) {
      L.ws_vn.alloc(L.N);
      cuda_check(cudaMemcpyAsync(L.ws_vn.p, vn, L.N * sizeof(double), cudaMemcpyHostToDevice, L.stream), "H2D");
      *dt_out = L.cfl_dt(L.ws_vn.p);
    });
  });
}

int lsg_second_derivatives_device(lsg_level_set* ls, const double* f_dev, double* f_dd_dev) {
  return guard([&] {
    need(f_dev != nullptr && f_dd_dev != nullptr, "null argument");
    with_ls(ls, [&](auto& L) { L.second_derivatives(f_dev, f_dd_dev); });
  });
}

int lsg_second_derivatives(lsg_level_set* ls, const double* f, double* f_dd) {
  return guard([&] {
    need(f != nullptr && f_dd != nullptr, "null argument");
    with_ls(ls, [&](auto& L) {
      using LT = std::decay_t<decltype(L)>;
      constexpr int D = LT::H == 2 ? 2 : 3;
      L.ws_phi.alloc(L.N);
      L.ws_dd.alloc((size_t)D * L.N);
      cuda_check(cudaMemcpyAsync(L.ws_phi.p, f, L.N * sizeof(double), cudaMemcpyHostToDevice, L.stream), "H2D");
      L.second_derivatives(L.ws_phi.p, L.ws_dd.p);
      cuda_check(cudaMemcpyAsync(f_dd, L.ws_dd.p, (size_t)D * L.N * sizeof(double), cudaMemcpyDeviceToHost, L.stream), "D2H");
      cuda_check(cudaStreamSynchronize(L.stream), "dd sync");
    });
  });
}

int lsg_perturb_level_set_function(lsg_level_set* ls, double* phi, double epsilon) {
  return guard([&] {
    need(phi != nullptr, "null phi");
    with_ls(ls, [&](auto& L) {
      for (int64_t n = 0; n < L.N; ++n)
        if (fabs(phi[n]) < epsilon) phi[n] = (phi[n] > 0) ? epsilon : -epsilon;
    });
  });
}

int lsg_first_derivatives(lsg_level_set* ls, const double* f, double* out) {
  return guard([&] {
    need(f != nullptr && out != nullptr, "null argument");
    with_ls(ls, [&](auto& L) {
      const int D = ls->dim;
      host_fields(L, f, 1, out, D, nullptr, [&](double* i, double* o, double*) { L.first_derivatives(i, o); });
    });
  });
}

int lsg_first_derivatives_device(lsg_level_set* ls, const double* f, double* out) {
  return guard([&] {
    need(f != nullptr && out != nullptr, "null argument");
    with_ls(ls, [&](auto& L) { L.first_derivatives(f, out); });
  });
}

int lsg_compute_normals(lsg_level_set* ls, const double* phi, double* normals) {
  return guard([&] {
    need(phi != nullptr && normals != nullptr, "null argument");
    with_ls(ls, [&](auto& L) {
      host_fields(L, phi, 1, normals, ls->dim, nullptr, [&](double* i, double* o, double*) { L.compute_normals(i, o); });
    });
  });
}

int lsg_compute_normals_device(lsg_level_set* ls, const double* phi, double* normals) {
  return guard([&] {
    need(phi != nullptr && normals != nullptr, "null argument");
    with_ls(ls, [&](auto& L) { L.compute_normals(phi, normals); });
  });
}

int lsg_compute_mean_curvature(lsg_level_set* ls, const double* normals, double* kappa) {
  return guard([&] {
    need(normals != nullptr && kappa != nullptr, "null argument");
    with_ls(ls, [&](auto& L) {
      host_fields(L, normals, ls->dim, kappa, 1, nullptr, [&](double* i, double* o, double*) { L.mean_curvature_from_normals(i, o); });
    });
  });
}

int lsg_compute_mean_curvature_device(lsg_level_set* ls, const double* normals, double* kappa) {
  return guard([&] {
    need(normals != nullptr && kappa != nullptr, "null argument");
    with_ls(ls, [&](auto& L) { L.mean_curvature_from_normals(normals, kappa); });
  });
}

int lsg_compute_normals_and_mean_curvature(lsg_level_set* ls, const double* phi, double* normals, double* kappa) {
  return guard([&] {
    need(phi != nullptr && normals != nullptr && kappa != nullptr, "null argument");
    with_ls(ls, [&](auto& L) {
      host_fields(L, phi, 1, normals, ls->dim, kappa,
                  [&](double* i, double* o, double* o2) { L.normals_and_mean_curvature(i, o, o2); });
    });
  });
}

int lsg_compute_normals_and_mean_curvature_device(lsg_level_set* ls, const double* phi, double* normals, double* kappa) {
  return guard([&] {
    need(phi != nullptr && normals != nullptr && kappa != nullptr, "null argument");
    with_ls(ls, [&](auto& L) { L.normals_and_mean_curvature(phi, normals, kappa); });
  });
}

int lsg_extend_over_interface_tvd_device(lsg_level_set* ls, const double* phi, double* q, int iterations, int order, double band_use,
                                         double band_extend, const double* normals, const double* mask) {
  return guard([&] {
    need(phi != nullptr && q != nullptr, "null argument");
    with_ls(ls, [&](auto& L) { L.extend_over_interface(phi, q, iterations, order, band_use, band_extend, normals, mask); });
  });
}

int lsg_extend_over_interface_tvd_ex_device(lsg_level_set* ls, const double* phi, double* q, int iterations, int order, double band_use,
                                            double band_extend, const double* normals, const double* mask, int use_nonzero_guess,
                                            double* q_n, double* q_nn) {
  return guard([&] {
    need(phi != nullptr && q != nullptr, "null argument");
    with_ls(ls, [&](auto& L) {
      L.extend_over_interface(phi, q, iterations, order, band_use, band_extend, normals, mask, use_nonzero_guess != 0, q_n, q_nn);
    });
  });
}

int lsg_extend_over_interface_tvd_ex(lsg_level_set* ls, const double* phi, double* q, int iterations, int order, double band_use,
                                     double band_extend, const double* normals, const double* mask, int use_nonzero_guess, double* q_n,
                                     double* q_nn) {
  return guard([&] {
    need(phi != nullptr && q != nullptr, "null argument");
    with_ls(ls, [&](auto& L) {
      const int D = ls->dim;
      const size_t N = (size_t)L.N;
      L.ws_f.ensure((2 + (normals ? D : 0) + (mask ? 1 : 0) + (q_n ? 1 : 0) + (q_nn ? 1 : 0)) * N + 1);
      double* cur = L.ws_f.p;
      auto take = [&](size_t cnt) {
        double* p = cur;
        cur += cnt;
        return p;
      };
      auto up = [&](double* dst, const double* src, size_t cnt) {
        if (cnt) cuda_check(cudaMemcpyAsync(dst, src, cnt * sizeof(double), cudaMemcpyHostToDevice, L.stream), "H2D");
      };
      auto down = [&](double* dst, const double* src, size_t cnt) {
        if (cnt) cuda_check(cudaMemcpyAsync(dst, src, cnt * sizeof(double), cudaMemcpyDeviceToHost, L.stream), "D2H");
      };
      double* dphi = take(N);
      double* dq = take(N);
      double* dn = normals ? take((size_t)D * N) : nullptr;
      double* dm = mask ? take(N) : nullptr;
      double* dqn = q_n ? take(N) : nullptr;
      double* dqnn = q_nn ? take(N) : nullptr;
      up(dphi, phi, N);
      up(dq, q, N);
      if (dn) up(dn, normals, (size_t)D * N);
      if (dm) up(dm, mask, N);
      if (dqn) up(dqn, q_n, N);
      if (dqnn) up(dqnn, q_nn, N);
      L.extend_over_interface(dphi, dq, iterations, order, band_use, band_extend, dn, dm, use_nonzero_guess != 0, dqn, dqnn);
      down(q, dq, N);
      if (dqn) down(q_n, dqn, N);
      if (dqnn) down(q_nn, dqnn, N);
      cuda_check(cudaStreamSynchronize(L.stream), "sync");
    });
  });
}

int lsg_extend_over_interface_tvd(lsg_level_set* ls, const double* phi, double* q, int iterations, int order, double band_use,
                                  double band_extend, const double* normals, const double* mask) {
  return guard([&] {
    need(phi != nullptr && q != nullptr, "null argument");
    with_ls(ls, [&](auto& L) {
      const int D = ls->dim;
      const size_t N = (size_t)L.N;
      L.ws_f.ensure((2 + (normals ? D : 0) + (mask ? 1 : 0)) * N + 1);
      double* dphi = L.ws_f.p;
      double* dq = dphi + N;
      double* dn = normals ? dq + N : nullptr;
      double* dm = mask ? dq + N + (normals ? (size_t)D * N : 0) : nullptr;
      auto up = [&](double* dst, const double* src, size_t cnt) {
        if (cnt) cuda_check(cudaMemcpyAsync(dst, src, cnt * sizeof(double), cudaMemcpyHostToDevice, L.stream), "H2D");
      };
      up(dphi, phi, N);
      up(dq, q, N);
      if (dn) up(dn, normals, (size_t)D * N);
      if (dm) up(dm, mask, N);
      L.extend_over_interface(dphi, dq, iterations, order, band_use, band_extend, dn, dm);
      if (N) cuda_check(cudaMemcpyAsync(q, dq, N * sizeof(double), cudaMemcpyDeviceToHost, L.stream), "D2H");
      cuda_check(cudaStreamSynchronize(L.stream), "sync");
    });
  });
}

int lsg_extend_from_interface_to_whole_domain_tvd_device(lsg_level_set* ls, const double* phi, const double* q_interface, double* q,
                                                         int nfields, int iterations, const double* mask, double band_zero,
                                                         double band_smooth, const double* grad_phi, int method) {
  return guard([&] {
    need(phi != nullptr && q_interface != nullptr && q != nullptr, "null argument");
    with_ls(ls, [&](auto& L) {
      L.extend_from_interface(phi, q_interface, q, nfields, iterations, mask, band_zero, band_smooth, grad_phi, method);
    });
  });
}

int lsg_extend_from_interface_to_whole_domain_tvd(lsg_level_set* ls, const double* phi, const double* q_interface, double* q, int nfields,
                                                  int iterations, const double* mask, double band_zero, double band_smooth,
                                                  const double* grad_phi, int method) {
  return guard([&] {
    need(phi != nullptr && q_interface != nullptr && q != nullptr, "null argument");
    need(nfields >= 1, "nfields must be at least 1");
    with_ls(ls, [&](auto& L) {
      const int D = ls->dim;
      const size_t N = (size_t)L.N, nf = (size_t)nfields;
      L.ws_f.ensure((1 + 2 * nf + (mask ? 1 : 0) + (grad_phi ? D : 0)) * N + 1);
      double* dphi = L.ws_f.p;
      double* dqi = dphi + N;
      double* dq = dqi + nf * N;
      double* dm = mask ? dq + nf * N : nullptr;
      double* dg = grad_phi ? dq + nf * N + (mask ? N : 0) : nullptr;
      auto up = [&](double* dst, const double* src, size_t cnt) {
        if (cnt) cuda_check(cudaMemcpyAsync(dst, src, cnt * sizeof(double), cudaMemcpyHostToDevice, L.stream), "H2D");
      };
      up(dphi, phi, N);
      up(dqi, q_interface, nf * N);
      if (dm) up(dm, mask, N);
      if (dg) up(dg, grad_phi, (size_t)D * N);
      L.extend_from_interface(dphi, dqi, dq, nfields, iterations, dm, band_zero, band_smooth, dg, method);
      if (N) cuda_check(cudaMemcpyAsync(q, dq, nf * N * sizeof(double), cudaMemcpyDeviceToHost, L.stream), "D2H");
      cuda_check(cudaStreamSynchronize(L.stream), "sync");
    });
  });
}

int lsg_extend_from_interface_to_whole_domain_tvd_cf(lsg_level_set* ls, const double* phi, const double* q_interface, double* q,
                                                     int iterations, lsg_interface_values_fn cf, void* ctx, const double* grad_phi) {
  return guard([&] {
    need(phi != nullptr && q_interface != nullptr && q != nullptr && cf != nullptr, "null argument");
    with_ls(ls, [&](auto& L) {
      const int D = ls->dim;
      const size_t N = (size_t)L.N;
      L.ws_f.ensure((3 + (grad_phi ? D : 0)) * N + 1);
      double* dphi = L.ws_f.p;
      double* dqi = dphi + N;
      double* dq = dqi + N;
      double* dg = grad_phi ? dq + N : nullptr;
      auto up = [&](double* dst, const double* src, size_t cnt) {
        if (cnt) cuda_check(cudaMemcpyAsync(dst, src, cnt * sizeof(double), cudaMemcpyHostToDevice, L.stream), "H2D");
      };
      up(dphi, phi, N);
      up(dqi, q_interface, N);
      if (dg) up(dg, grad_phi, (size_t)D * N);
      L.extend_from_interface(dphi, dqi, dq, 1, iterations, nullptr, 0.0, 1.0, dg, 0, cf, ctx);
      if (N) cuda_check(cudaMemcpyAsync(q, dq, N * sizeof(double), cudaMemcpyDeviceToHost, L.stream), "D2H");
      cuda_check(cudaStreamSynchronize(L.stream), "sync");
    });
  });
}

int lsg_interpolate_nodes(lsg_level_set* ls, const double* xyz, int64_t npts, const double* F, int nfields, const double* Fdd,
                          int method, double* out) {
  return guard([&] {
    need(F != nullptr && out != nullptr && (xyz != nullptr || npts == 0), "null argument");
    with_ls(ls, [&](auto& L) { L.interpolate_host(xyz, npts, nfields, F, Fdd, method, out); });
  });
}

int lsg_interpolate_nodes_device(lsg_level_set* ls, const double* xyz, int64_t npts, const double* F, int nfields, const double* Fdd,
                                 int method, double* out) {
  return guard([&] {
    need(F != nullptr && out != nullptr && (xyz != nullptr || npts == 0), "null argument");
    with_ls(ls, [&](auto& L) { L.interpolate(xyz, npts, nfields, F, Fdd, method, out); });
  });
}

int lsg_locate_points_device(lsg_level_set* ls, const double* xyz, int64_t npts, int32_t* leaf) {
  return guard([&] {
    need(leaf != nullptr && (xyz != nullptr || npts == 0) && npts >= 0, "null argument");
    with_ls(ls, [&](auto& L) { L.locate(xyz, npts, leaf); });
  });
}

int lsg_semi_lagrangian_advect(lsg_level_set* ls, const double* xyz, int64_t npts, double dt, const double* v, const double* vdd,
                               const double* phi, const double* phi_dd, int velo_method, int phi_method, double* phi_np1) {
  return guard([&] {
    need(v != nullptr && phi != nullptr && phi_np1 != nullptr && (xyz != nullptr || npts == 0), "null argument");
    with_ls(ls, [&](auto& L) { L.sl_advect_host(xyz, npts, dt, v, vdd, phi, phi_dd, velo_method, phi_method, phi_np1); });
  });
}

int lsg_semi_lagrangian_advect_device(lsg_level_set* ls, const double* xyz, int64_t npts, double dt, const double* v,
                                      const double* vdd, const double* phi, const double* phi_dd, int velo_method, int phi_method,
                                      double* phi_np1) {
  return guard([&] {
    need(v != nullptr && phi != nullptr && phi_np1 != nullptr && (xyz != nullptr || npts == 0), "null argument");
    with_ls(ls, [&](auto& L) { L.sl_advect(xyz, npts, dt, v, vdd, phi, phi_dd, velo_method, phi_method, phi_np1); });
  });
}

int lsg_semi_lagrangian_advect2(lsg_level_set* ls_n, lsg_level_set* ls_nm1, const double* xyz_np1, int64_t npts, double dt_nm1,
                                double dt_n, const double* vnm1, const double* vnm1_dd, const double* vn, const double* vn_dd,
                                const double* phi_n, const double* phi_dd, int velo_method, int phi_method, double* phi_np1) {
  return guard([&] {
    need(vnm1 != nullptr && vn != nullptr && phi_n != nullptr && phi_np1 != nullptr && (xyz_np1 != nullptr || npts == 0),
         "null argument");
    with_ls_pair(ls_n, ls_nm1, [&](auto& L, auto& M) {
      L.sl_advect2_host(M, xyz_np1, npts, dt_nm1, dt_n, vnm1, vnm1_dd, vn, vn_dd, phi_n, phi_dd, velo_method, phi_method, phi_np1);
    });
  });
}

int lsg_semi_lagrangian_advect2_device(lsg_level_set* ls_n, lsg_level_set* ls_nm1, const double* xyz_np1, int64_t npts, double dt_nm1,
                                       double dt_n, const double* vnm1, const double* vnm1_dd, const double* vn, const double* vn_dd,
                                       const double* phi_n, const double* phi_dd, int velo_method, int phi_method, double* phi_np1) {
  return guard([&] {
    need(vnm1 != nullptr && vn != nullptr && phi_n != nullptr && phi_np1 != nullptr && (xyz_np1 != nullptr || npts == 0),
         "null argument");
    with_ls_pair(ls_n, ls_nm1, [&](auto& L, auto& M) {
      L.sl_advect2(M, xyz_np1, npts, dt_nm1, dt_n, vnm1, vnm1_dd, vn, vn_dd, phi_n, phi_dd, velo_method, phi_method, phi_np1);
    });
  });
}

static double velocity_scale(int velocity, const double* params, int nparams) {
  need(velocity == LSG_VELOCITY_VORTEX, "unknown analytic velocity");
  return (params != nullptr && nparams > 0) ? params[0] : 1.0;
}

int lsg_semi_lagrangian_advect_cf(lsg_level_set* ls, const double* xyz, int64_t npts, double dt, int velocity, const double* params,
                                  int nparams, const double* phi, const double* phi_dd, int phi_method, double* phi_np1) {
  return guard([&] {
    need(phi != nullptr && phi_np1 != nullptr && (xyz != nullptr || npts == 0), "null argument");
    const double s = velocity_scale(velocity, params, nparams);
    with_ls(ls, [&](auto& L) { L.sl_advect_vortex_host(xyz, npts, dt, s, phi, phi_dd, phi_method, phi_np1); });
  });
}

int lsg_semi_lagrangian_advect_cf_device(lsg_level_set* ls, const double* xyz, int64_t npts, double dt, int velocity,
                                         const double* params, int nparams, const double* phi, const double* phi_dd, int phi_method,
                                         double* phi_np1) {
  return guard([&] {
    need(phi != nullptr && phi_np1 != nullptr && (xyz != nullptr || npts == 0), "null argument");
    const double s = velocity_scale(velocity, params, nparams);
    with_ls(ls, [&](auto& L) { L.sl_advect_vortex(xyz, npts, dt, s, phi, phi_dd, phi_method, phi_np1); });
  });
}

int lsg_semi_lagrangian_advect_callback(lsg_level_set* ls, const double* xyz, int64_t npts, double dt, lsg_velocity_fn velocity,
                                        void* ctx, const double* phi, const double* phi_dd, int phi_method, double* phi_np1) {
  return guard([&] {
    need(velocity != nullptr && phi != nullptr && phi_np1 != nullptr && (xyz != nullptr || npts == 0), "null argument");
    need(npts >= 0, "negative number of points");
    with_ls(ls, [&](auto& L) {
      using LT = std::decay_t<decltype(L)>;
      constexpr int D = LT::DIM;
      need(L.F != nullptr, "advect_from_n_to_np1: needs a single grid's level set");
      const Brick& B = L.F->brick;
      const size_t n = (size_t)npts * D;
      std::vector<double> v(n + 1), xs(n + 1), xd(n + 1);
      auto clip = [&](double* x) {
        for (int a = 0; a < D; ++a)
          if (x[a] < B.xyz_min[a] || x[a] > B.xyz_max[a]) x[a] = max2(B.xyz_min[a], min2(B.xyz_max[a], x[a]));
      };
      auto eval = [&](const double* pts) {
        if (npts && velocity(ctx, npts, pts, v.data()) != 0) throw std::runtime_error("advect_from_n_to_np1: the velocity callback failed");
      };
      // x* = x - dt/2 v(x), clipped; x_d = x - dt v(x*), clipped (src/my_p4est_semi_lagrangian.cpp:108-146)
      eval(xyz);
      for (int64_t p = 0; p < npts; ++p) {
        for (int a = 0; a < D; ++a) xs[(size_t)p * D + a] = xyz[(size_t)p * D + a] - 0.5 * dt * v[(size_t)p * D + a];
        clip(&xs[(size_t)p * D]);
      }
      eval(xs.data());
      for (int64_t p = 0; p < npts; ++p) {
        for (int a = 0; a < D; ++a) xd[(size_t)p * D + a] = xyz[(size_t)p * D + a] - dt * v[(size_t)p * D + a];
        clip(&xd[(size_t)p * D]);
      }
      L.interpolate_host(xd.data(), npts, 1, phi, phi_dd, phi_method, phi_np1);
    });
  });
}

int lsg_batch_create(int count, const lsg_forest* const* forests, lsg_level_set** out) {
  return lsg_batch_create_ex(count, forests, 0, out);
}

int lsg_batch_create_ex(int count, const lsg_forest* const* forests, int flags, lsg_level_set** out) {
  return guard([&] {
    need(out != nullptr && forests != nullptr && count > 0, "batch: null arguments or no grids");
    need((flags & ~LSG_BUILD_ON_DEVICE) == 0, "unknown batch flags");
    const bool on_device = (flags & LSG_BUILD_ON_DEVICE) != 0;
    const int dim = forests[0] ? forests[0]->dim : 0;
    need(dim == 2 || dim == 3, "batch: null forest");
    for (int k = 0; k < count; ++k) need(forests[k] != nullptr && forests[k]->dim == dim, "batch: grids of one dimension required");
    lsg_level_set* ls = new lsg_level_set();
    ls->dim = dim;
    ls->device = current_device();
    try {
      if (dim == 2) {
        std::vector<const Forest<2>*> parts;
        for (int k = 0; k < count; ++k) parts.push_back(forests[k]->f2);
        ls->l2 = new LevelSet<2>(parts, on_device);
      } else {
        std::vector<const Forest<3>*> parts;
        for (int k = 0; k < count; ++k) parts.push_back(forests[k]->f3);
        ls->l3 = new LevelSet<3>(parts, on_device);
      }
    } catch (...) {
      delete ls;
      throw;
    }
    *out = ls;
  });
}

int lsg_batch_count(const lsg_level_set* ls) {
  if (!ls) return -1;
  return (int)((ls->dim == 2 ? ls->l2->part_offsets.size() : ls->l3->part_offsets.size()) - 1);
}

int lsg_batch_offsets(const lsg_level_set* ls, int64_t* offsets) {
  return guard([&] {
    need(ls != nullptr && offsets != nullptr, "null argument");
    const auto& o = ls->dim == 2 ? ls->l2->part_offsets : ls->l3->part_offsets;
    for (size_t k = 0; k < o.size(); ++k) offsets[k] = o[k];
  });
}

int lsg_batch_reinitialize_device(lsg_level_set* ls, double* phi_dev, const int* iterations, int use_graph) {
  return guard([&] {
    need(phi_dev != nullptr && iterations != nullptr, "null argument");
    with_ls(ls, [&](auto& L) { L.reinitialize_batch(phi_dev, iterations, use_graph != 0); });
  });
}

int lsg_batch_reinitialize(lsg_level_set* ls, double* phi, const int* iterations, int use_graph) {
  return guard([&] {
    need(phi != nullptr && iterations != nullptr, "null argument");
    with_ls(ls, [&](auto& L) {
      L.ws_phi.alloc(L.N);
      cuda_check(cudaMemcpyAsync(L.ws_phi.p, phi, L.N * sizeof(double), cudaMemcpyHostToDevice, L.stream), "H2D phi");
      L.reinitialize_batch(L.ws_phi.p, iterations, use_graph != 0);
      cuda_check(cudaMemcpyAsync(phi, L.ws_phi.p, L.N * sizeof(double), cudaMemcpyDeviceToHost, L.stream), "D2H phi");
      cuda_check(cudaStreamSynchronize(L.stream), "batch sync");
    });
  });
}

int lsg_level_set_autotune(lsg_level_set* ls, const double* phi, int trials, int* config) {
  return guard([&] {
    need(phi != nullptr, "null phi");
    with_ls(ls, [&](auto& L) {
      L.ws_phi.alloc(L.N);
      cuda_check(cudaMemcpyAsync(L.ws_phi.p, phi, L.N * sizeof(double), cudaMemcpyHostToDevice, L.stream), "H2D phi");
      L.autotune(L.ws_phi.p, trials);
      cuda_check(cudaStreamSynchronize(L.stream), "autotune sync");
      if (config) {
        config[0] = L.cfg.tpb;
        config[1] = L.cfg.uniform_blocks;
        config[2] = L.cfg.regular_blocks;
        config[3] = L.cfg.depth;
        config[4] = L.cfg.halo;
        config[5] = L.cfg.streams;
        config[6] = L.cfg.priority;
      }
    });
  });
}

int lsg_level_set_stage_config(const lsg_level_set* ls, int* config) {
  return guard([&] {
    need(ls != nullptr && config != nullptr, "null argument");
    const StageCfg& c = ls->dim == 2 ? ls->l2->cfg : ls->l3->cfg;
    config[0] = c.tpb;
    config[1] = c.uniform_blocks;
    config[2] = c.regular_blocks;
    config[3] = c.depth;
    config[4] = c.halo;
    config[5] = c.streams;
    config[6] = c.priority;
  });
}

int lsg_level_set_set_stage_config(lsg_level_set* ls, const int* config) {
  return guard([&] {
    need(config != nullptr, "null config");
    need(config[0] == 32 || config[0] == 64 || config[0] == 128 || config[0] == 256, "threads per block must be 32, 64, 128 or 256");
    need(config[1] >= 0 && config[2] >= 0, "grid sizes must be >= 0 (0: one full wave)");
    need(config[3] >= 1 && config[3] <= 5, "uniform kernel variant (pipeline depth) must be 1 to 5");
    need(config[4] >= 0 && config[4] <= 4096 && config[4] % 4 == 0, "window halo must be a multiple of 4 in 0..4096");
    need(config[5] == 1 || config[5] == 2, "streams must be 1 or 2");
    need(config[6] >= 0 && config[6] <= 4, "priority must be 0 .. 4");
    with_ls(ls, [&](auto& L) {
      L.cfg.tpb = config[0];
      L.cfg.uniform_blocks = config[1];
      L.cfg.regular_blocks = config[2];
      L.cfg.depth = config[3];
      L.cfg.halo = config[4];
      L.cfg.streams = config[5];
      L.cfg.priority = config[6];
      L.drop_graph();
    });
  });
}

int lsg_second_derivatives_range_device(lsg_level_set* ls, const double* f_dev, double* f_dd_dev, int64_t first, int64_t count) {
  return guard([&] {
    need(f_dev != nullptr && f_dd_dev != nullptr, "null argument");
    with_ls(ls, [&](auto& L) { L.fp64_dd_range(f_dev, f_dd_dev, first, count); });
  });
}

int lsg_reinit_prep_range_device(lsg_level_set* ls, const double* phi0_dev, const double* phi0_dd_dev, int order_space, double limit_high,
                                 double limit_low, int64_t first, int64_t count) {
  return guard([&] {
    need(phi0_dev != nullptr && phi0_dd_dev != nullptr, "null phi_0 or second derivatives");
    with_ls(ls, [&](auto& L) { L.fp64_prep_range(phi0_dev, phi0_dd_dev, order_space, limit_high, limit_low, first, count); });
  });
}

int lsg_reinit_stage_range_device(lsg_level_set* ls, int order_space, const double* phi0_dev, const double* phin_dev,
                                  const double* phin_dd_dev, double* out_dev, const double* avg_with_dev, int64_t first, int64_t count) {
  return guard([&] {
    need(phi0_dev != nullptr && phin_dev != nullptr && phin_dd_dev != nullptr && out_dev != nullptr, "null argument");
    with_ls(ls, [&](auto& L) { L.fp64_stage_range(order_space, phi0_dev, phin_dev, phin_dd_dev, out_dev, avg_with_dev, first, count); });
  });
}

int lsg_advect_stage_range_device(lsg_level_set* ls, const double* phin_dev, const double* phin_dd_dev, const double* minmod_dd_dev,
                                  const double* vn_dev, double dt, double* out_dev, const double* avg_with_dev, int64_t first,
                                  int64_t count) {
  return guard([&] {
    need(phin_dev != nullptr && phin_dd_dev != nullptr && minmod_dd_dev != nullptr && vn_dev != nullptr && out_dev != nullptr,
         "null argument");
    with_ls(ls, [&](auto& L) { L.fp64_advect_stage_range(phin_dev, phin_dd_dev, minmod_dd_dev, vn_dev, dt, out_dev, avg_with_dev, first, count); });
  });
}

int lsg_mixed_split_begin_device(lsg_level_set* ls, const double* phi_dev, const double* mask_dev, int order_space, double limit_high,
                                 double limit_low) {
  return guard([&] {
    need(phi_dev != nullptr, "null phi");
    with_ls(ls, [&](auto& L) { L.mixed_split_begin(phi_dev, order_space, limit_high, limit_low, mask_dev); });
  });
}

int lsg_mixed_split_stage_device(lsg_level_set* ls, int order_space, int stage) {
  return guard([&] {
    need(order_space == 1 || order_space == 2, "the order in space is 1 or 2");
    need(stage == 0 || stage == 1, "stage is 0 or 1");
    with_ls(ls, [&](auto& L) { L.mixed_step(order_space, stage); });
  });
}

int lsg_mixed_split_field_device(lsg_level_set* ls, int which, float** field_dev) {
  return guard([&] {
    need(field_dev != nullptr && (which == 0 || which == 1), "which is 0 or 1, field_dev not null");
    with_ls(ls, [&](auto& L) {
      float* p = L.mixed_field(which);
      if (!p) throw StateError("mixed split: call lsg_mixed_split_begin_device first");
      *field_dev = p;
    });
  });
}

int lsg_mixed_split_slots_device(lsg_level_set* ls, int32_t* slots_dev) {
  return guard([&] {
    need(slots_dev != nullptr, "null output");
    with_ls(ls, [&](auto& L) { L.mixed_slots(slots_dev); });
  });
}

int lsg_mixed_split_end_device(lsg_level_set* ls, double* phi_dev) {
  return guard([&] {
    need(phi_dev != nullptr, "null phi");
    with_ls(ls, [&](auto& L) {
      if (!L.mixed_field(0)) throw StateError("mixed split: call lsg_mixed_split_begin_device first");
      L.mixed_end(phi_dev);
    });
  });
}

int lsg_interface_location_error_device(lsg_level_set* ls, const double* a_dev, const double* b_dev, double* out, int64_t* edges,
                                        int64_t* mismatched) {
  return guard([&] {
    need(a_dev != nullptr && b_dev != nullptr && out != nullptr, "null argument");
    with_ls(ls, [&](auto& L) { *out = L.interface_location_error(a_dev, b_dev, edges, mismatched); });
  });
}

int lsg_band_linf_device(lsg_level_set* ls, const double* a_dev, const double* b_dev, double band, double* out, int64_t* count) {
  return guard([&] {
    need(a_dev != nullptr && b_dev != nullptr && out != nullptr, "null argument");
    need(band > 0, "band must be positive");
    with_ls(ls, [&](auto& L) { *out = L.band_linf(a_dev, b_dev, band, count); });
  });
}

int lsg_level_set_table_stats(lsg_level_set* ls, int64_t* out) {
  return guard([&] {
    need(out != nullptr, "null output");
    with_ls(ls, [&](auto& L) {
      if (!L.mixed_ready) throw StateError("the mixed tables are not built");
      out[0] = L.N;
      out[1] = L.T32.nR;
      out[2] = L.T32.nU;
      out[3] = L.T32.nI;
      out[4] = L.T32.nX;
      out[5] = L.ncls;
      out[6] = L.num_corrections;
    });
  });
}

int lsg_level_set_enable_kernel_timing(lsg_level_set* ls, int on) {
  return guard([&] { with_ls(ls, [&](auto& L) { L.timer.enabled = on != 0; }); });
}

int lsg_level_set_set_wait_limit(lsg_level_set* ls, long long cycles) {
  return guard([&] { with_ls(ls, [&](auto& L) { L.set_wait_limit(cycles); }); });
}

int lsg_level_set_kernel_times(lsg_level_set* ls, double* ms, int64_t* counts, int nkinds, int reset) {
  return guard([&] {
    need(ms != nullptr && counts != nullptr, "null output");
    with_ls(ls, [&](auto& L) {
      L.timer.collect();
      for (int k = 0; k < nkinds && k < K_NUM_KINDS; ++k) {
        ms[k] = L.timer.ms[k];
        counts[k] = L.timer.count[k];
      }
      if (reset) L.timer.reset();
    });
  });
}

int64_t lsg_level_set_launch_count(const lsg_level_set* ls) {
  if (!ls) return -1;
  return ls->dim == 2 ? ls->l2->timer.launches : ls->l3->timer.launches;
}

int64_t lsg_device_cache_bytes(void) { return (int64_t)DeviceCache::get().cached_bytes(); }

int lsg_device_cache_release(void) {
  return guard([&] { DeviceCache::get().trim(); });
}

}  // extern "C"
