// Host drivers of the device level-set operator (see level_set.hpp).
#include "level_set.hpp"

#include <array>

#include "flatten.hpp"

#include <float.h>

#include <algorithm>
#include <cmath>

#include <cstdlib>
#include <cstring>
#include <stdexcept>

namespace lsg {

// src/my_p4est_utils.h:322-330
double largest_dbl_smaller_than_dbl_max() {
  double p = 1.0;
  while (DBL_MAX - p == DBL_MAX) p *= 2.0;
  return DBL_MAX - p;
}

KernelTimer::~KernelTimer() {
  for (auto& e : pool) {
    cudaEventDestroy(e.first);
    cudaEventDestroy(e.second);
  }
}

void KernelTimer::begin(int kind, cudaStream_t s) {
  ++launches;
  if (!enabled) return;
  if (used == pool.size()) {
    cudaEvent_t a, b;
    cuda_check(cudaEventCreate(&a), "cudaEventCreate");
    cuda_check(cudaEventCreate(&b), "cudaEventCreate");
    pool.push_back({a, b});
  }
  auto ev = pool[used++];
  cuda_check(cudaEventRecord(ev.first, s), "cudaEventRecord");
  pending.push_back({kind, ev});
}

void KernelTimer::end(cudaStream_t s) {
  if (!enabled) return;
  cuda_check(cudaEventRecord(pending.back().second.second, s), "cudaEventRecord");
}

void KernelTimer::collect() {
  for (auto& p : pending) {
    cuda_check(cudaEventSynchronize(p.second.second), "cudaEventSynchronize");
    float t = 0;
    cuda_check(cudaEventElapsedTime(&t, p.second.first, p.second.second), "cudaEventElapsedTime");
    ms[p.first] += t;
    count[p.first] += 1;
  }
  pending.clear();
  used = 0;
}

void KernelTimer::reset() {
  collect();
  for (int k = 0; k < K_NUM_KINDS; ++k) {
    ms[k] = 0;
    count[k] = 0;
  }
  launches = 0;
}

#define LSG_LAUNCH(kind, expr) \
  do {                         \
    timer.begin(kind, stream); \
    expr;                      \
    timer.end(stream);         \
  } while (0)

template <int D>
LevelSet<D>::LevelSet(const Forest<D>& forest, bool with_mixed, bool device_build) : F(&forest) {
  if (!forest.nodes_built) throw std::invalid_argument("level set: the forest's nodes are not built");
  double tdim[3];
  for (int a = 0; a < D; ++a) tdim[a] = (forest.brick.xyz_max[a] - forest.brick.xyz_min[a]) / forest.brick.n[a];
  zdt = EPS * (D == 3 ? min3(tdim[0], tdim[1], tdim[2]) : min2(tdim[0], tdim[1]));
  double ts[3];
  for (int a = 0; a < D; ++a) ts[a] = forest.brick.tmax[a] - forest.brick.tmin[a];
  if (!device_build) {
    Tables64<D> T;
    build_tables64<D>(forest, T);
    init_tables(T, ts, with_mixed);
  } else {
    N = (int64_t)forest.num_nodes();
    init_stream();
    // the forest's device copy (made by the device node numbering, else uploaded now) is shared
    const ForestDevice<D>& X = forest_device(const_cast<Forest<D>&>(forest), stream);
    fdev = forest.device;
    build_locator();
    DForest<D> DF{};
    DF.nleaves = TL.nleaves;
    DF.N = N;
    DF.key = TL.key;
    DF.level = TL.level;
    DF.local_nodes = TL.local_nodes;
    DF.ctab = TL.ctab;
    DF.L0 = TL.L0;
    DF.ncoarse = TL.ncoarse;
    for (int a = 0; a < 3; ++a) DF.n[a] = TL.n[a];
    DF.ijk_to_tree = TL.ijk_to_tree;
    DF.tree_ijk = X.tree_ijk.p;
    DF.tmin = TL.tmin;
    DF.tmax = TL.tmax;
    DF.node_tree = X.node_tree.p;
    DF.node_x = X.node_x.p;
    const Tab64Dev<D> out{&nbr, &w, &nrm, &d, &q, &cidx, &crec, &wall, &smin};
    num_corrections = build_tables64_device<D>(DF, out, stream);
    T64.N = N;
    T64.nbr = nbr.p;
    T64.w = w.p;
    T64.nrm = nrm.p;
    T64.d = d.p;
    T64.q = q.p;
    T64.cidx = cidx.p;
    T64.crec = crec.p;
    T64.wall = wall.p;
    device_flat = true;
    if (with_mixed) build_mixed();
  }
  part_offsets = {0, N};
}

template <int D>
void LevelSet<D>::init_stream() {
  cuda_check(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "cudaStreamCreate");
  own_stream = true;
}

// FP64 tables of one grid built on the device into `out` (the grid's device copy is made if absent);
// returns the number of correction records
template <int D>
static int64_t device_tables_of(const Forest<D>& f, const Tab64Dev<D>& out, cudaStream_t s) {
  using DD = Dim<D>;
  const ForestDevice<D>& X = forest_device(const_cast<Forest<D>&>(f), s);
  const int64_t nl = (int64_t)f.leaves.size();
  const int nt = f.brick.num_trees;
  int L0 = 0;  // the point-location table's uniform level, as build_locator chooses it
  while (L0 < DD::MAXLEVEL && ((int64_t)nt << (D * (L0 + 1))) <= 2 * nl) ++L0;
  DevBuf<int32_t> ctab;
  ctab.alloc((size_t)((int64_t)nt * (int64_t(1) << (D * L0)) + 1));
  coarse_table_device<D>(X.leaf_key.p, nl, nt, L0, ctab.p, s);
  DForest<D> DF{};
  DF.nleaves = nl;
  DF.N = (int64_t)f.num_nodes();
  DF.key = X.leaf_key.p;
  DF.level = X.level.p;
  DF.local_nodes = X.local_nodes.p;
  DF.ctab = ctab.p;
  DF.L0 = L0;
  DF.ncoarse = int64_t(1) << (D * L0);
  for (int a = 0; a < 3; ++a) DF.n[a] = f.brick.n[a];
  DF.ijk_to_tree = X.ijk_to_tree.p;
  DF.tree_ijk = X.tree_ijk.p;
  DF.tmin = X.tmin.p;
  DF.tmax = X.tmax.p;
  DF.node_tree = X.node_tree.p;
  DF.node_x = X.node_x.p;
  return build_tables64_device<D>(DF, out, s);  // synchronises s, so ctab may go
}

template <int D>
LevelSet<D>::LevelSet(const std::vector<const Forest<D>*>& parts, bool device_build) : F(nullptr) {
  if (parts.empty()) throw std::invalid_argument("batch: no grids");
  std::vector<Tables64<D>> T(parts.size());
  std::vector<const Tables64<D>*> ptr(parts.size());
  double ts[3] = {0, 0, 0}, tdim[3] = {0, 0, 0};
  for (size_t k = 0; k < parts.size(); ++k) {
    const Forest<D>& f = *parts[k];
    if (!f.nodes_built) throw std::invalid_argument("batch: a forest's nodes are not built");
    for (int a = 0; a < D; ++a) {
      const double t = f.brick.tmax[a] - f.brick.tmin[a];
      const double dim_a = (f.brick.xyz_max[a] - f.brick.xyz_min[a]) / f.brick.n[a];
      if (k == 0) {
        ts[a] = t;
        tdim[a] = dim_a;
      } else if (t != ts[a] || dim_a != tdim[a]) {
        throw std::invalid_argument("batch: every grid must have the same tree size");
      }
    }
  }
  zdt = EPS * (D == 3 ? min3(tdim[0], tdim[1], tdim[2]) : min2(tdim[0], tdim[1]));
  part_offsets.assign(1, 0);
  if (device_build) {
    init_stream();
    // every grid's tables, then the union: planes [slot][node] concatenated with node indices and
    // correction-record indices offset by the parts before
    std::vector<std::array<DevBuf<int32_t>, 2>> ib(parts.size());   // nbr, cidx
    std::vector<std::array<DevBuf<double>, 6>> db(parts.size());    // w, nrm, d, q, crec, smin
    std::vector<DevBuf<uint8_t>> wb(parts.size());
    std::vector<int64_t> R(parts.size());
    int64_t Rtot = 0;
    for (size_t k = 0; k < parts.size(); ++k) {
      const Tab64Dev<D> out{&ib[k][0], &db[k][0], &db[k][1], &db[k][2], &db[k][3], &ib[k][1], &db[k][4], &wb[k], &db[k][5]};
      R[k] = device_tables_of<D>(*parts[k], out, stream);
      part_offsets.push_back(part_offsets.back() + (int64_t)parts[k]->num_nodes());
      Rtot += R[k];
    }
    N = part_offsets.back();
    num_corrections = Rtot;
    nbr.alloc((size_t)NS * N);
    w.alloc((size_t)NS * N);
    nrm.alloc((size_t)2 * D * N);
    d.alloc((size_t)2 * D * N);
    q.alloc((size_t)2 * D * (D - 1) * N);
    cidx.alloc((size_t)N);
    crec.alloc((size_t)6 * Rtot + 6);
    wall.alloc((size_t)N);
    smin.alloc((size_t)N);
    int64_t roff = 0;
    for (size_t k = 0; k < parts.size(); ++k) {
      const int64_t o = part_offsets[k], nk = part_offsets[k + 1] - o;
      auto planes = [&](void* dst, const void* src, size_t es, int np) {
        if (nk)
          cuda_check(cudaMemcpy2DAsync((char*)dst + o * es, (size_t)N * es, src, (size_t)nk * es, (size_t)nk * es, (size_t)np,
                                       cudaMemcpyDeviceToDevice, stream),
                     "batch table concatenation");
      };
      concat_index_planes(ib[k][0].p, nk, NS, nbr.p, N, o, (int32_t)o, stream);
      concat_index_planes(ib[k][1].p, nk, 1, cidx.p, N, o, (int32_t)roff, stream);
      planes(w.p, db[k][0].p, 8, NS);
      planes(nrm.p, db[k][1].p, 8, 2 * D);
      planes(d.p, db[k][2].p, 8, 2 * D);
      planes(q.p, db[k][3].p, 8, 2 * D * (D - 1));
      planes(smin.p, db[k][5].p, 8, 1);
      planes(wall.p, wb[k].p, 1, 1);
      if (R[k])
        cuda_check(cudaMemcpyAsync(crec.p + 6 * roff, db[k][4].p, (size_t)6 * R[k] * sizeof(double), cudaMemcpyDeviceToDevice, stream),
                   "batch correction records");
      roff += R[k];
    }
    cuda_check(cudaStreamSynchronize(stream), "batch tables");  // the parts' buffers go back to the cache
    T64.N = N;
    T64.nbr = nbr.p;
    T64.w = w.p;
    T64.nrm = nrm.p;
    T64.d = d.p;
    T64.q = q.p;
    T64.cidx = cidx.p;
    T64.crec = crec.p;
    T64.wall = wall.p;
    device_flat = true;
    MixedDev<D> M{&r_meta, &r_nbr, &r_nbr2, &r_meta2, &i_meta, &i_cls, &i_nbr, &i_wf, &i_d, &i_q, &i_cidx, &corr32, &cls32,
                  &i_wf64, &i_d64, &i_q64, &corr64, &perm, &iperm};
    build_mixed_device<D>(T64, num_corrections, ts, M, stream);
    near_list.alloc((size_t)N);
    near_count.alloc(1);
    set_mixed_views(M.nR, M.nI, M.nU, M.base, M.x_first, M.nX, M.ncls, ts);
    return;
  }
#pragma omp parallel for schedule(dynamic, 1)
  for (long long k = 0; k < (long long)parts.size(); ++k) build_tables64<D>(*parts[(size_t)k], T[(size_t)k]);
  for (size_t k = 0; k < parts.size(); ++k) {
    ptr[k] = &T[k];
    part_offsets.push_back(part_offsets.back() + T[k].N);
  }
  Tables64<D> U;
  concat_tables64<D>(ptr, U);
  T.clear();
  init_tables(U, ts, true);
}

template <int D>
void LevelSet<D>::init_tables(const Tables64<D>& T, const double* ts, bool with_mixed) {
  N = T.N;
  init_stream();
  num_corrections = (int64_t)(T.crec.size() / 6);
  nbr.upload(T.nbr, stream);
  w.upload(T.w, stream);
  nrm.upload(T.nrm, stream);
  d.upload(T.d, stream);
  q.upload(T.q, stream);
  cidx.upload(T.cidx, stream);
  crec.upload(T.crec, stream);
  wall.upload(T.wall, stream);
  smin.upload(T.smin, stream);
  if (with_mixed) {
    Tables32<D> M;
    build_tables32<D>(T, ts, M);
    upload_mixed(M, ts);
  }
  cuda_check(cudaStreamSynchronize(stream), "table upload");
  T64.N = N;
  T64.nbr = nbr.p;
  T64.w = w.p;
  T64.nrm = nrm.p;
  T64.d = d.p;
  T64.q = q.p;
  T64.cidx = cidx.p;
  T64.crec = crec.p;
  T64.wall = wall.p;
}

template <int D>
LevelSet<D>::~LevelSet() {
  if (stream) cudaStreamSynchronize(stream);
  drop_graph();
  if (side_stream) {
    cudaStreamSynchronize(side_stream);
    cudaStreamSynchronize(side_hi);
    cudaStreamSynchronize(main_hi);
    cudaStreamDestroy(side_stream);
    cudaStreamDestroy(side_hi);
    cudaStreamDestroy(main_hi);
    cudaEventDestroy(ev_fork);
    cudaEventDestroy(ev_ddx);
    cudaEventDestroy(ev_join);
    cudaEventDestroy(ev_main);
  }
  if (own_stream && stream) cudaStreamDestroy(stream);
  if (capture_stream) cudaStreamDestroy(capture_stream);
}

template <int D>
void LevelSet<D>::set_stream(cudaStream_t s) {
  cuda_check(cudaStreamSynchronize(stream), "stream sync");
  if (own_stream && stream) cudaStreamDestroy(stream);
  own_stream = false;
  stream = s;
}

template <int D>
void LevelSet<D>::second_derivatives(const double* f, double* dd) {
  LSG_LAUNCH(K_DD64, launch_dd64<D>(T64, f, dd, stream));
  cuda_check(cudaGetLastError(), "second derivatives");
}

template <int D>
void LevelSet<D>::reinitialize(double* phi, int os, int ot, double limit_high, double limit_low, int iterations, int precision,
                               const double* mask) {
  if (os < 1 || os > 2 || ot < 1 || ot > 2)
    throw std::invalid_argument(
        "reinitialize_within_range_of_phi_0: valid orders of orders of accuracy for space and pseudotime are 1 and 2 only!");
  if (!(limit_high > limit_low)) throw std::invalid_argument("reinitialize: limit_high must exceed limit_low");
  if (iterations < 0) throw std::invalid_argument("reinitialize: negative number of iterations");
  // phi_0 limits widened as in reinitialize_one_iteration (src/my_p4est_level_set.cpp:75-76)
  const double big = largest_dbl_smaller_than_dbl_max();
  const double lo = (limit_low < -big ? -DBL_MAX : limit_low - max2(zdt, EPS * fabs(limit_low)));
  const double hi = (limit_high > big ? DBL_MAX : limit_high + max2(zdt, EPS * fabs(limit_high)));
  if (precision == PREC_FP64)
    reinit_fp64(phi, os, ot, hi, lo, iterations, mask);
  else if (precision == PREC_MIXED)
    reinit_mixed(phi, os, ot, hi, lo, iterations, mask);
  else
    throw std::invalid_argument("reinitialize: unknown precision mode");
}

template <int D>
void LevelSet<D>::reinitialize_fp64_noalloc(double* phi, int os, int ot, double limit_high, double limit_low, int iterations) {
  if (os < 1 || os > 2 || ot < 1 || ot > 2)
    throw std::invalid_argument(
        "reinitialize_within_range_of_phi_0: valid orders of orders of accuracy for space and pseudotime are 1 and 2 only!");
  if (!(limit_high > limit_low)) throw std::invalid_argument("reinitialize: limit_high must exceed limit_low");
  if (iterations < 0) throw std::invalid_argument("reinitialize: negative number of iterations");
  const double big = largest_dbl_smaller_than_dbl_max();
  const double lo = (limit_low < -big ? -DBL_MAX : limit_low - max2(zdt, EPS * fabs(limit_low)));
  const double hi = (limit_high > big ? DBL_MAX : limit_high + max2(zdt, EPS * fabs(limit_high)));
  reinit_fp64_static<D>(T64, zdt, phi, os, ot, hi, lo, iterations, stream);
}

// reinitialize_within_range_of_phi_0 (src/my_p4est_level_set.cpp:290-557) on one device:
// the ghost updates of a single process are no-ops and the layer/local split merges into one launch.
template <int D>
bool LevelSet<D>::ensure_sorted64() {
  if (sorted64_ready) return true;
  if (sorted64_failed || N == 0) return false;
  // LSGPU_FP64_NODE_ORDER=1 keeps the FP64 sweeps on the node-ordered tables (the layout they fall back to when
  // the sorted copy does not fit), so that path can be exercised without running out of memory
  const char* node_order = std::getenv("LSGPU_FP64_NODE_ORDER");
  if (node_order && node_order[0] == '1') return false;
  constexpr int NS = 2 * D * Dim<D>::HALF;
  try {
    s_perm.alloc(N);
    s_iperm.alloc(N);
    s_nbr.alloc((size_t)NS * N);
    s_w.alloc((size_t)NS * N);
    s_nrm.alloc((size_t)2 * D * N);
    s_d.alloc((size_t)2 * D * N);
    s_q.alloc((size_t)2 * D * (D - 1) * N);
    s_cidx.alloc(N);
    s_wall.alloc(N);
    DevBuf<uint32_t> keys, keys_out;
    DevBuf<int32_t> idx;
    DevBuf<unsigned char> temp;
    keys.alloc(N);
    keys_out.alloc(N);
    idx.alloc(N);
    const size_t tb = sort64_temp_bytes(N);
    temp.alloc(tb > 0 ? tb : 1);
    const Tab64Out out{s_nbr.p, s_w.p, s_nrm.p, s_d.p, s_q.p, s_cidx.p, s_wall.p};
    cuda_check(launch_sort_tab64<D>(T64, keys.p, keys_out.p, idx.p, temp.p, tb, s_perm.p, s_iperm.p, out, stream), "pattern sort");
  } catch (const CudaOutOfMemory&) {
    for (DevBuf<int32_t>* b : {&s_perm, &s_iperm, &s_nbr, &s_cidx}) b->release();
    for (DevBuf<double>* b : {&s_w, &s_nrm, &s_d, &s_q}) b->release();
    s_wall.release();
    sorted64_failed = true;
    return false;
  }
  T64s = T64;
  T64s.nbr = s_nbr.p;
  T64s.w = s_w.p;
  T64s.nrm = s_nrm.p;
  T64s.d = s_d.p;
  T64s.q = s_q.p;
  T64s.cidx = s_cidx.p;
  T64s.wall = s_wall.p;
  T64s.word = nullptr;
  // the per-node pattern word; without the memory for it the sweeps read the full stencil of every face
  try {
    s_word.alloc(N);
    launch_node_word64<D>(T64s, s_word.p, stream);
    cuda_check(cudaGetLastError(), "node pattern words");
    T64s.word = s_word.p;
  } catch (const CudaOutOfMemory&) {
    s_word.release();
  }
  sorted64_ready = true;
  return true;
}

// The FP64 reinitialisation: phi_0's second derivatives and the phi_0-only preparation once, then per
// iteration the second-derivative and stage sweeps of each RK stage. The sweeps run on the tables in
// stencil-pattern order (phi gathered into that order first and scattered back at the end) when those
// could be built, else on the node-ordered tables; the results are the same bits either way.
template <int D>
void LevelSet<D>::reinit_fp64(double* phi_user, int os, int ot, double hi, double lo, int iters, const double* mask) {
  phi0.alloc(N);
  phi1.alloc(N);
  dd0.alloc((size_t)D * N);
  ddc.alloc((size_t)D * N);
  snear.alloc((size_t)2 * D * N);
  status.alloc(N);
  const bool sorted = ensure_sorted64();
  const DTab64<D>& T = sorted ? T64s : T64;
  double* phi = phi_user;
  if (sorted) {
    s_phi.alloc(N);
    phi = s_phi.p;
    launch_gather_perm64(phi_user, s_perm.p, phi, N, stream);
  }
  cuda_check(cudaMemcpyAsync(phi0.p, phi, N * sizeof(double), cudaMemcpyDeviceToDevice, stream), "copy phi_0");
  LSG_LAUNCH(K_DD64, launch_dd64<D>(T, phi0.p, dd0.p, stream));
  LSG_LAUNCH(K_PREP64, launch_reinit_prep64<D>(T, phi0.p, dd0.p, zdt, lo, hi, os, status.p, snear.p, stream));
  if (mask) LSG_LAUNCH(K_PREP64, launch_apply_mask(mask, sorted ? s_perm.p : nullptr, status.p, N, stream));
  for (int it = 0; it < iters; ++it) {
    LSG_LAUNCH(K_DD64, launch_dd64<D>(T, phi, ddc.p, stream));
    LSG_LAUNCH(K_STAGE64, launch_reinit_stage64<D>(T, os, status.p, snear.p, phi0.p, phi, ddc.p, phi1.p, nullptr, stream));
    if (ot > 1) {
      LSG_LAUNCH(K_DD64, launch_dd64<D>(T, phi1.p, ddc.p, stream));
      LSG_LAUNCH(K_STAGE64, launch_reinit_stage64<D>(T, os, status.p, snear.p, phi0.p, phi1.p, ddc.p, phi, phi, stream));
    } else {
      cuda_check(cudaMemcpyAsync(phi, phi1.p, N * sizeof(double), cudaMemcpyDeviceToDevice, stream), "copy phi_np1");
    }
  }
  if (sorted) launch_scatter_perm64(phi, s_perm.p, phi_user, N, stream);
  cuda_check(cudaGetLastError(), "reinitialize (fp64)");
}

static void check_range(int64_t first, int64_t count, int64_t N) {
  if (first < 0 || count < 0 || first > N || count > N - first) throw std::invalid_argument("node range outside the grid");
}

template <int D>
void LevelSet<D>::fp64_dd_range(const double* f, double* dd, int64_t first, int64_t count) {
  check_range(first, count, N);
  LSG_LAUNCH(K_DD64, launch_dd64<D>(T64, f, dd, stream, first, count));
  cuda_check(cudaGetLastError(), "second derivatives (node range)");
}

template <int D>
void LevelSet<D>::fp64_prep_range(const double* phi0_, const double* dd0_, int os, double limit_high, double limit_low, int64_t first,
                                  int64_t count) {
  check_range(first, count, N);
  if (os < 1 || os > 2) throw std::invalid_argument("reinitialize: the order in space must be 1 or 2");
  if (!(limit_high > limit_low)) throw std::invalid_argument("reinitialize: limit_high must exceed limit_low");
  // the quadratic neighbour values read the node's own second derivatives at every order
  if (!phi0_ || !dd0_) throw std::invalid_argument("reinitialize preparation: phi_0 and its second derivatives are required");
  const double big = largest_dbl_smaller_than_dbl_max();
  const double lo = (limit_low < -big ? -DBL_MAX : limit_low - max2(zdt, EPS * fabs(limit_low)));
  const double hi = (limit_high > big ? DBL_MAX : limit_high + max2(zdt, EPS * fabs(limit_high)));
  snear.ensure((size_t)2 * D * N);
  status.ensure((size_t)N);
  LSG_LAUNCH(K_PREP64, launch_reinit_prep64<D>(T64, phi0_, dd0_, zdt, lo, hi, os, status.p, snear.p, stream, first, count));
  cuda_check(cudaGetLastError(), "reinitialize preparation (node range)");
}

template <int D>
void LevelSet<D>::fp64_stage_range(int os, const double* phi0_, const double* phin, const double* dd, double* out, const double* avg_with,
                                   int64_t first, int64_t count) {
  check_range(first, count, N);
  if (!status.p || status.n < (size_t)N) throw std::invalid_argument("reinitialize stage: run the preparation first");
  if (!phi0_ || !phin || !dd || !out) throw std::invalid_argument("reinitialize stage: phi_0, phi_n, its second derivatives and out are required");
  LSG_LAUNCH(K_STAGE64, launch_reinit_stage64<D>(T64, os, status.p, snear.p, phi0_, phin, dd, out, avg_with, stream, first, count));
  cuda_check(cudaGetLastError(), "reinitialize stage (node range)");
}

// one advect_in_normal_direction_one_iteration sweep over the nodes [first, first + count), node-ordered tables
// (the per-rank sweep of a Morton-range split): ddq the second derivatives of phin (its quadratic neighbour values),
// ddm those of the minmod terms, out = phin - dt vn |grad|, averaged with avg_with when given
template <int D>
void LevelSet<D>::fp64_advect_stage_range(const double* phin, const double* ddq, const double* ddm, const double* vn, double dt, double* out,
                                          const double* avg_with, int64_t first, int64_t count) {
  check_range(first, count, N);
  if (!phin || !ddq || !ddm || !vn || !out) throw std::invalid_argument("advection stage: phi_n, both second derivatives, vn and out are required");
  LSG_LAUNCH(K_ADVECT64, launch_advect_stage64<D>(T64, phin, ddq, ddm, vn, dt, out, avg_with, stream, first, count));
  cuda_check(cudaGetLastError(), "advection stage (node range)");
}

template <int D>
void LevelSet<D>::build_mixed() {
  if (mixed_ready) return;
  if (!F) throw std::invalid_argument("level set: mixed tables of a grid union are built at construction");
  if (device_flat) {
    double ts[3];
    for (int a = 0; a < D; ++a) ts[a] = F->brick.tmax[a] - F->brick.tmin[a];
    MixedDev<D> M{&r_meta, &r_nbr, &r_nbr2, &r_meta2, &i_meta, &i_cls, &i_nbr, &i_wf, &i_d, &i_q, &i_cidx, &corr32, &cls32,
                  &i_wf64, &i_d64, &i_q64, &corr64, &perm, &iperm};
    build_mixed_device<D>(T64, num_corrections, ts, M, stream);
    near_list.alloc((size_t)N);
    near_count.alloc(1);
    set_mixed_views(M.nR, M.nI, M.nU, M.base, M.x_first, M.nX, M.ncls, ts);
    return;
  }
  // The FP32 tables derive from the FP64 ones; rebuild those on the host.
  Tables64<D> T;
  build_tables64<D>(*F, T);
  Tables32<D> M;
  double ts[3];
  for (int a = 0; a < D; ++a) ts[a] = F->brick.tmax[a] - F->brick.tmin[a];
  build_tables32<D>(T, ts, M);
  upload_mixed(M, ts);
}

template <int D>
void LevelSet<D>::upload_mixed(const Tables32<D>& M, const double* ts) {
  r_meta.upload(M.r_meta, stream);
  r_nbr.upload(M.r_nbr, stream);
  r_nbr2.upload(M.r_nbr2, stream);
  i_cls.upload(M.i_cls, stream);
  cls32.upload(M.cls32, stream);
  r_meta2.upload(M.r_meta2, stream);
  i_meta.upload(M.i_meta, stream);
  i_nbr.upload(M.i_nbr, stream);
  i_wf.upload(M.i_wf, stream);
  i_d.upload(M.i_d, stream);
  i_q.upload(M.i_q, stream);
  i_cidx.upload(M.i_cidx, stream);
  corr32.upload(M.corr, stream);
  i_wf64.upload(M.i_wf64, stream);
  i_d64.upload(M.i_d64, stream);
  i_q64.upload(M.i_q64, stream);
  corr64.upload(M.corr64, stream);
  perm.upload(M.perm, stream);
  h_perm = M.perm;
  iperm.upload(M.iperm, stream);
  near_list.alloc((size_t)N);
  near_count.alloc(1);
  cuda_check(cudaStreamSynchronize(stream), "mixed table upload");
  set_mixed_views(M.nR, M.nI, M.nU, M.base_level, M.x_first, (int64_t)M.x_list.size(), M.ncls, ts);
}

template <int D>
void LevelSet<D>::set_mixed_views(int64_t nR_, int64_t nI_, int64_t nU_, int base, int64_t x_first, int64_t nX, int64_t ncls_,
                                  const double* ts) {
  nR = nR_;
  nI = nI_;
  ncls = ncls_;
  kerr.alloc(1);
  cuda_check(cudaMemsetAsync(kerr.p, 0, sizeof(int), stream), "memset");
  T32.N = N;
  T32.nR = nR_;
  T32.nI = nI_;
  T32.base = base;
  for (int a = 0; a < 3; ++a) T32.tsize[a] = a < D ? (float)ts[a] : 1.0f;
  for (int a = 0; a < 3; ++a) T32.inv_tsize[a] = 1.0f / T32.tsize[a];
  T32.nU = nU_;
  T32.r_meta = r_meta.p;
  T32.r_nbr = r_nbr.p;
  T32.r_nbr2 = r_nbr2.p;
  T32.i_cls = i_cls.p;
  T32.cls32 = cls32.p;
  T32.x_first = x_first;
  T32.nX = nX;
  T32.r_meta2 = r_meta2.p;
  T32.i_meta = i_meta.p;
  T32.i_nbr = i_nbr.p;
  T32.i_wf = i_wf.p;
  T32.i_d = i_d.p;
  T32.i_q = i_q.p;
  T32.i_cidx = i_cidx.p;
  T32.corr = corr32.p;
  for (int a = 0; a < 3; ++a) T32.tsize64[a] = a < D ? ts[a] : 1.0;
  T32.i_wf64 = i_wf64.p;
  T32.i_d64 = i_d64.p;
  T32.i_q64 = i_q64.p;
  T32.corr64 = corr64.p;
  // the stage kernels' node-major copy of the regular nodes' stencil indices (D int4 per node, 16-byte aligned)
  T32.u_pack = nullptr;
  if (nR_ > 0) {
    u_pack.alloc((size_t)D * nR_);
    launch_pack_uniform32<D>(T32, u_pack.p, stream);
    cuda_check(cudaGetLastError(), "pack uniform indices");
    T32.u_pack = u_pack.p;
  }
  mixed_ready = true;
}

template <int D>
bool LevelSet<D>::take_device_wait_flag() {
  if (!kerr.p) return false;
  int h = 0;
  cuda_check(cudaMemcpyAsync(&h, kerr.p, sizeof(int), cudaMemcpyDeviceToHost, stream), "D2H");
  cuda_check(cudaStreamSynchronize(stream), "device wait check");
  if (h) {
    cuda_check(cudaMemsetAsync(kerr.p, 0, sizeof(int), stream), "memset");
    cuda_check(cudaStreamSynchronize(stream), "device wait check");
  }
  return h != 0;
}

template <int D>
void LevelSet<D>::check_device_waits() {
  if (!kerr.p) return;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cuda_check(cudaStreamIsCapturing(stream, &cs), "cudaStreamIsCapturing");
  if (cs != cudaStreamCaptureStatusNone) return;
  if (take_device_wait_flag())
    throw DeviceTimeout("reinitialize (mixed): a bounded wait for a bulk copy gave up; results of this call are incomplete");
}

// One RK stage of the mixed path on two streams: the side stream computes the extended second
// derivatives and then the irregular nodes while the main stream runs the uniform regular nodes;
// the remaining regular nodes follow once the extended second derivatives are ready. With one stream
// (cfg.streams 1) the four kernels run one after another.
template <int D>
void LevelSet<D>::ensure_side_stream() {
  if (side_stream) return;
  int least = 0, greatest = 0;
  cuda_check(cudaDeviceGetStreamPriorityRange(&least, &greatest), "cudaDeviceGetStreamPriorityRange");
  cuda_check(cudaStreamCreateWithFlags(&side_stream, cudaStreamNonBlocking), "cudaStreamCreate");
  cuda_check(cudaStreamCreateWithPriority(&side_hi, cudaStreamNonBlocking, greatest), "cudaStreamCreateWithPriority");
  cuda_check(cudaStreamCreateWithPriority(&main_hi, cudaStreamNonBlocking, greatest), "cudaStreamCreateWithPriority");
  cuda_check(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming), "cudaEventCreate");
  cuda_check(cudaEventCreateWithFlags(&ev_ddx, cudaEventDisableTiming), "cudaEventCreate");
  cuda_check(cudaEventCreateWithFlags(&ev_join, cudaEventDisableTiming), "cudaEventCreate");
  cuda_check(cudaEventCreateWithFlags(&ev_main, cudaEventDisableTiming), "cudaEventCreate");
}

template <int D>
void LevelSet<D>::mixed_stage(int os, const float* phin, float* out, const float* avg_with, const float* adv_vn, float adv_dt) {
  if (cfg.streams == 1) {
    mixed_join();
    timer.begin(K_STAGE32, stream);
    launch_dd_x32<D>(T32, phin, f_dd.p, stream, cfg.tpb);
    launch_reinit_part32<D>(T32, STAGE_PART_IRREGULAR, os, status.p, f_snear.p, phin, f_dd.p, out, avg_with, stream, cfg, kerr.p, adv_vn, adv_dt);
    launch_reinit_part32<D>(T32, STAGE_PART_UNIFORM, os, status.p, f_snear.p, phin, f_dd.p, out, avg_with, stream, cfg, kerr.p, adv_vn, adv_dt);
    launch_reinit_part32<D>(T32, STAGE_PART_REGULAR, os, status.p, f_snear.p, phin, f_dd.p, out, avg_with, stream, cfg, kerr.p, adv_vn, adv_dt);
    timer.end(stream);
    timer.launches += 3;  // four kernels per stage
    return;
  }
  ensure_side_stream();
  // two chains: A = second derivatives then one of the two kernels that need them, B = the uniform nodes then
  // the other one (which waits for A's second derivatives)
  const bool swap = cfg.priority >= 3;  // A ends with the other regular nodes, B with the irregular ones
  const cudaStream_t a = (cfg.priority == 1 || cfg.priority == 3) ? side_hi : side_stream;
  const cudaStream_t b = (cfg.priority == 2 || cfg.priority == 4) ? main_hi : stream;
  if (chains_open && (timer.enabled || join_each_stage || a != chain_a || b != chain_b)) mixed_join();
  timer.begin(K_STAGE32, stream);
  if (!chains_open) {
    cuda_check(cudaEventRecord(ev_fork, stream), "cudaEventRecord");
    cuda_check(cudaStreamWaitEvent(a, ev_fork, 0), "cudaStreamWaitEvent");
    if (b != stream) cuda_check(cudaStreamWaitEvent(b, ev_fork, 0), "cudaStreamWaitEvent");
  } else {
    // the previous stage's other chain: every kernel of that stage has finished reading and writing before
    // this stage's kernels start (chain order covers the rest)
    cuda_check(cudaStreamWaitEvent(a, ev_main, 0), "cudaStreamWaitEvent");
    cuda_check(cudaStreamWaitEvent(b, ev_join, 0), "cudaStreamWaitEvent");
  }
  launch_dd_x32<D>(T32, phin, f_dd.p, a, cfg.tpb);
  cuda_check(cudaEventRecord(ev_ddx, a), "cudaEventRecord");
  launch_reinit_part32<D>(T32, swap ? STAGE_PART_REGULAR : STAGE_PART_IRREGULAR, os, status.p, f_snear.p, phin, f_dd.p, out, avg_with, a,
                          cfg, kerr.p, adv_vn, adv_dt);
  cuda_check(cudaEventRecord(ev_join, a), "cudaEventRecord");
  launch_reinit_part32<D>(T32, STAGE_PART_UNIFORM, os, status.p, f_snear.p, phin, f_dd.p, out, avg_with, b, cfg, kerr.p, adv_vn, adv_dt);
  cuda_check(cudaStreamWaitEvent(b, ev_ddx, 0), "cudaStreamWaitEvent");
  launch_reinit_part32<D>(T32, swap ? STAGE_PART_IRREGULAR : STAGE_PART_REGULAR, os, status.p, f_snear.p, phin, f_dd.p, out, avg_with, b,
                          cfg, kerr.p, adv_vn, adv_dt);
  cuda_check(cudaEventRecord(ev_main, b), "cudaEventRecord");
  chains_open = true;
  chain_a = a;
  chain_b = b;
  // with the per-stage timer the caller's stream joins every stage (the timing brackets one stage), and so it
  // does in a captured graph (a graph of per-stage forks and joins replayed faster than one of open chains:
  // 18.7 against 19.5 ms on the 256-grid batch); otherwise the chains stay open into the next stage and
  // mixed_join() closes them after the last one (34.6 against 34.8 ms on the 13.7M-node grid)
  if (timer.enabled || join_each_stage) mixed_join();
  timer.end(stream);
  timer.launches += 3;  // four kernels per stage
}

// the caller's stream waits for both chains of the last mixed stage
template <int D>
void LevelSet<D>::mixed_join() {
  if (!chains_open) return;
  if (chain_b != stream) cuda_check(cudaStreamWaitEvent(stream, ev_main, 0), "cudaStreamWaitEvent");
  cuda_check(cudaStreamWaitEvent(stream, ev_join, 0), "cudaStreamWaitEvent");
  chains_open = false;
}

// Mixed precision: phi_n and all per-iteration work in FP32 (device node order); the phi_0-only
// subcell step in FP64.
template <int D>
void LevelSet<D>::reinit_mixed(double* phi, int os, int ot, double hi, double lo, int iters, const double* mask) {
  if (iters == 0) return;  // phi unchanged, as with no iteration in FP64
  mixed_begin(phi, os, hi, lo, mask);
  for (int it = 0; it < iters; ++it) {
    mixed_stage(os, f_phi.p, f_phi1.p, nullptr);
    if (ot > 1) {
      mixed_stage(os, f_phi1.p, f_phi.p, f_phi.p);
    } else {
      std::swap(f_phi.p, f_phi1.p);
    }
  }
  mixed_end(phi);
}

template <int D>
void LevelSet<D>::mixed_split_begin(const double* phi, int os, double limit_high, double limit_low, const double* mask) {
  if (os < 1 || os > 2) throw std::invalid_argument("mixed preparation: the order in space is 1 or 2");
  if (!(limit_high > limit_low)) throw std::invalid_argument("mixed preparation: limit_high must exceed limit_low");
  const double big = largest_dbl_smaller_than_dbl_max();
  const double lo = (limit_low < -big ? -DBL_MAX : limit_low - max2(zdt, EPS * fabs(limit_low)));
  const double hi = (limit_high > big ? DBL_MAX : limit_high + max2(zdt, EPS * fabs(limit_high)));
  mixed_begin(phi, os, hi, lo, mask);
}

// The phi_0-only FP64 step of the mixed path and phi_n in FP32 device order (hi, lo: the widened limits).
template <int D>
void LevelSet<D>::mixed_begin(const double* phi, int os, double hi, double lo, const double* mask) {
  mixed_join();  // chains left open by a call that stopped on an error
  build_mixed();
  f_phi.alloc(N);
  f_phi1.alloc(N);
  f_dd.alloc((size_t)D * N);
  f_snear.alloc((size_t)2 * D * N);
  status.alloc(N);
  phi0.alloc(N);
  dd0.alloc((size_t)D * (nI > 0 ? nI : 1));
  LSG_LAUNCH(K_PREP_MIXED, launch_reinit_prep_mixed<D>(T32, perm.p, phi, zdt, lo, hi, os, phi0.p, dd0.p, status.p, f_snear.p,
                                                       near_list.p, near_count.p, stream));
  timer.launches += 3;  // the FP64 subcell step is four kernels
  if (mask) LSG_LAUNCH(K_PREP_MIXED, launch_apply_mask(mask, perm.p, status.p, N, stream));
  LSG_LAUNCH(K_CONVERT, launch_gather_f32(phi, perm.p, f_phi.p, N, 0, 0, 1, stream));
}

// phi (FP64, node order) from the FP32 phi_n of the last stage; ends the chains
template <int D>
void LevelSet<D>::mixed_end(double* phi) {
  mixed_join();
  LSG_LAUNCH(K_CONVERT, launch_scatter_f64(f_phi.p, perm.p, status.p, phi, N, 0, 0, 1, stream));
  cuda_check(cudaGetLastError(), "reinitialize (mixed)");
  if (cfg.depth == 3 || cfg.depth == 4) check_device_waits();
}

// One RK stage of the mixed path for a caller that updates ghosts between stages (a rank of a Morton split):
// stage 0 phi_n -> phi_1, stage 1 phi_1 -> phi_n averaged with phi_n; the object's stream has the stage's kernels
// behind it on return (both chains joined), so a ghost update issued on that stream follows them.
template <int D>
void LevelSet<D>::mixed_step(int os, int stage) {
  if (!f_phi.p || !f_phi1.p || !status.p) throw std::invalid_argument("mixed stage: call the mixed preparation first");
  if (stage == 0) mixed_stage(os, f_phi.p, f_phi1.p, nullptr);
  else mixed_stage(os, f_phi1.p, f_phi.p, f_phi.p);
  mixed_join();
  cuda_check(cudaGetLastError(), "mixed stage");
}

template <int D>
void LevelSet<D>::mixed_slots(int32_t* out_dev) {
  build_mixed();
  cuda_check(cudaMemcpyAsync(out_dev, iperm.p, (size_t)N * sizeof(int32_t), cudaMemcpyDeviceToDevice, stream), "copy node slots");
}

template <int D>
void LevelSet<D>::drop_graph() {
  if (graph_exec) cudaGraphExecDestroy(graph_exec);
  if (graph) cudaGraphDestroy(graph);
  graph_exec = nullptr;
  graph = nullptr;
  graph_key.clear();
}

// The pseudo-time loop of the mixed path (os: order in space, second order in time); before
// iteration `it` the nodes of every grid whose iteration count is `it` are frozen.
template <int D>
void LevelSet<D>::mixed_loop(int os, int iters, const std::vector<int>& freeze_at) {
  for (int it = 0; it < iters; ++it) {
    if (std::binary_search(freeze_at.begin(), freeze_at.end(), it)) {
      mixed_join();
      timer.launches += 1;
      launch_freeze32(iter_lim.p, it, status.p, N, stream);
    }
    mixed_stage(os, f_phi.p, f_phi1.p, nullptr);
    mixed_stage(os, f_phi1.p, f_phi.p, f_phi.p);
  }
  mixed_join();
}

// phi_0-only preparation of a batched call (reinitialize_2nd_order: limits +-DBL_MAX, second order).
template <int D>
void LevelSet<D>::prep_batch(const double* phi) {
  mixed_join();  // chains left open by a call that stopped on an error
  build_mixed();
  f_phi.alloc(N);
  f_phi1.alloc(N);
  f_dd.alloc((size_t)D * N);
  f_snear.alloc((size_t)2 * D * N);
  status.alloc(N);
  phi0.alloc(N);
  dd0.alloc((size_t)D * (nI > 0 ? nI : 1));
  LSG_LAUNCH(K_PREP_MIXED, launch_reinit_prep_mixed<D>(T32, perm.p, phi, zdt, -DBL_MAX, DBL_MAX, 2, phi0.p, dd0.p, status.p,
                                                       f_snear.p, near_list.p, near_count.p, stream));
  timer.launches += 3;
  LSG_LAUNCH(K_CONVERT, launch_gather_f32(phi, perm.p, f_phi.p, N, 0, 0, 1, stream));
}

template <int D>
void LevelSet<D>::reinitialize_batch(double* phi, const int* iterations, bool use_graph) {
  const size_t nparts = part_offsets.size() - 1;
  std::vector<int> its(iterations, iterations + nparts);
  int max_it = 0;
  for (int v : its) {
    if (v < 0 || v > 65535) throw std::invalid_argument("batch: iteration counts must lie in [0, 65535]");
    max_it = std::max(max_it, v);
  }
  if (its != part_iters) {
    std::vector<uint16_t> lim_node((size_t)N), lim((size_t)N);
    for (size_t k = 0; k < nparts; ++k)
      for (int64_t n = part_offsets[k]; n < part_offsets[k + 1]; ++n) lim_node[(size_t)n] = (uint16_t)its[k];
    if (h_perm.empty() && N) {
      h_perm.resize((size_t)N);
      cuda_check(cudaMemcpyAsync(h_perm.data(), perm.p, (size_t)N * sizeof(int32_t), cudaMemcpyDeviceToHost, stream), "D2H");
      cuda_check(cudaStreamSynchronize(stream), "perm download");
    }
    for (int64_t i = 0; i < N; ++i) lim[(size_t)i] = lim_node[(size_t)h_perm[(size_t)i]];
    iter_lim.upload(lim, stream);
    part_iters = its;
  }
  std::vector<int> freeze_at;
  for (int v : its)
    if (v < max_it) freeze_at.push_back(v);
  std::sort(freeze_at.begin(), freeze_at.end());
  freeze_at.erase(std::unique(freeze_at.begin(), freeze_at.end()), freeze_at.end());
  prep_batch(phi);
  if (use_graph) {
    std::vector<int> key(1, max_it);
    key.insert(key.end(), freeze_at.begin(), freeze_at.end());
    if (!graph_exec || key != graph_key) {
      drop_graph();
      ensure_side_stream();
      const bool timing = timer.enabled;
      timer.enabled = false;
      const int64_t before = timer.launches;
      if (!capture_stream) cuda_check(cudaStreamCreateWithFlags(&capture_stream, cudaStreamNonBlocking), "cudaStreamCreate");
      // capture records work without running it, so it may use a stream of its own; the graph is
      // then launched on the caller's stream
      const cudaStream_t user = stream;
      stream = capture_stream;
      cudaError_t e = cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal);
      if (e == cudaSuccess) {
        join_each_stage = true;
        try {
          mixed_loop(2, max_it, freeze_at);
          join_each_stage = false;
        } catch (...) {
          join_each_stage = false;
          cudaGraph_t g = nullptr;
          cudaStreamEndCapture(stream, &g);
          if (g) cudaGraphDestroy(g);
          stream = user;
          timer.enabled = timing;
          timer.launches = before;
          throw;
        }
        e = cudaStreamEndCapture(stream, &graph);
      }
      stream = user;
      timer.enabled = timing;
      timer.launches = before;
      cuda_check(e, "graph capture");
      cuda_check(cudaGraphInstantiate(&graph_exec, graph, 0), "cudaGraphInstantiate");
      size_t nodes = 0;
      cuda_check(cudaGraphGetNodes(graph, nullptr, &nodes), "cudaGraphGetNodes");
      graph_launches = (int64_t)(4 * 2 * (int64_t)max_it + (int64_t)freeze_at.size());
      graph_key = key;
    }
    timer.begin(K_STAGE32, stream);
    cuda_check(cudaGraphLaunch(graph_exec, stream), "cudaGraphLaunch");
    timer.end(stream);
    timer.launches += graph_launches - 1;
  } else {
    mixed_loop(2, max_it, freeze_at);
  }
  LSG_LAUNCH(K_CONVERT, launch_scatter_f64(f_phi.p, perm.p, status.p, phi, N, 0, 0, 1, stream, iter_lim.p));
  cuda_check(cudaGetLastError(), "reinitialize (batch)");
  if (cfg.depth == 3 || cfg.depth == 4) check_device_waits();
}

// Autotuner: coordinate search over the launch shape of the mixed stage (threads per block, pipeline
// depth and grid of the persistent uniform kernel, the phi window of its bulk-copy form, grid of the
// persistent regular kernel, one or two streams), timing
// `trials` iterations per candidate with CUDA events on the object's stream.
template <int D>
void LevelSet<D>::autotune(const double* phi, int trials) {
  if (trials < 1) trials = 1;
  prep_batch(phi);
  ensure_side_stream();
  cudaEvent_t e0, e1;
  cuda_check(cudaEventCreate(&e0), "cudaEventCreate");
  cuda_check(cudaEventCreate(&e1), "cudaEventCreate");
  const int sms = device_sm_count();
  const bool timing = timer.enabled;
  timer.enabled = false;
  // one timing of `iters` iterations with launch shape c (after one untimed iteration)
  auto time_once = [&](const StageCfg& c, int iters) -> float {
    cfg = c;
    mixed_stage(2, f_phi.p, f_phi1.p, nullptr);
    mixed_stage(2, f_phi1.p, f_phi.p, f_phi.p);
    mixed_join();
    cuda_check(cudaEventRecord(e0, stream), "cudaEventRecord");
    for (int t = 0; t < iters; ++t) {
      mixed_stage(2, f_phi.p, f_phi1.p, nullptr);
      mixed_stage(2, f_phi1.p, f_phi.p, f_phi.p);
    }
    mixed_join();
    cuda_check(cudaEventRecord(e1, stream), "cudaEventRecord");
    cuda_check(cudaEventSynchronize(e1), "cudaEventSynchronize");
    float ms = 0.0f;
    cuda_check(cudaEventElapsedTime(&ms, e0, e1), "cudaEventElapsedTime");
    // a candidate whose bounded waits gave up left CTAs early: it only looks fast, so drop it
    if ((c.depth == 3 || c.depth == 4) && take_device_wait_flag()) return 1e30f;
    return ms;
  };
  // a candidate's time in the search: the median of three timings of `trials` iterations (how the two
  // streams' blocks share the SMs can differ from one run to the next, so a single timing can catch a
  // lucky run); every candidate tried is kept for the final round
  std::vector<std::pair<float, StageCfg>> tried;
  auto run = [&](const StageCfg& c) -> float {
    float rep[3];
    for (int k = 0; k < 3; ++k) rep[k] = time_once(c, trials);
    std::sort(rep, rep + 3);
    tried.emplace_back(rep[1], c);
    return rep[1];
  };
  const long long wait_cycles = cfg.wait_cycles;
  // the clocks ramp up and the tables settle in L2 before the first candidate is timed
  {
    StageCfg w;
    w.wait_cycles = wait_cycles;
    time_once(w, 4 * trials);
  }
  StageCfg best;
  best.wait_cycles = wait_cycles;
  float best_ms = 1e30f;
  const int grids[] = {0, 2, 3, 4, 6};
  for (int tpb : {256, 128}) {
    StageCfg c;
    c.tpb = tpb;
    c.wait_cycles = wait_cycles;
    float c_ms = 1e30f;
    for (int depth : {1, 2, 3, 4, 5})
      for (int g : grids) {
        StageCfg t = c;
        t.depth = depth;
        t.uniform_blocks = g * sms * (256 / tpb);
        const float ms = run(t);
        if (ms < c_ms) {
          c_ms = ms;
          c.depth = depth;
          c.uniform_blocks = t.uniform_blocks;
        }
      }
    if (c.depth == 3 || c.depth == 4)  // the phi window of the bulk-copy kernel
      for (int halo : {128, 256, 1024, 2048}) {
        StageCfg t = c;
        t.halo = halo;
        const float ms = run(t);
        if (ms < c_ms) {
          c_ms = ms;
          c.halo = halo;
        }
      }
    for (int g : grids) {
      if (g == 6) continue;
      StageCfg t = c;
      t.regular_blocks = g * sms * (256 / tpb);
      const float ms = run(t);
      if (ms < c_ms) {
        c_ms = ms;
        c.regular_blocks = t.regular_blocks;
      }
    }
    {  // the four kernels on one stream
      StageCfg t = c;
      t.streams = 1;
      const float ms = run(t);
      if (ms < c_ms) {
        c_ms = ms;
        c.streams = 1;
      }
    }
    // The stream priority stays at its default (2): in whole 50-iteration calls it was the fastest setting on
    // both grids measured and the only one whose calls all took the same time, while in short trials the
    // other settings sometimes timed faster than they run.
    if (c_ms < best_ms) {
      best_ms = c_ms;
      best = c;
    }
  }
  // Final round: the search's four fastest distinct shapes and the default shape, timed again with runs four
  // times longer, round-robin so that a drift of the clocks or of the block scheduling touches them all
  // alike; the lowest median of three wins. Short trials could rank a shape first that ran 12% slower in
  // whole calls.
  {
    auto same = [](const StageCfg& x, const StageCfg& y) {
      return x.tpb == y.tpb && x.uniform_blocks == y.uniform_blocks && x.regular_blocks == y.regular_blocks &&
             x.depth == y.depth && x.halo == y.halo && x.streams == y.streams && x.priority == y.priority;
    };
    std::stable_sort(tried.begin(), tried.end(), [](const auto& x, const auto& y) { return x.first < y.first; });
    std::vector<StageCfg> finalists;
    for (const auto& t : tried) {
      if (t.first >= 1e29f || finalists.size() >= 4) break;
      bool dup = false;
      for (const StageCfg& f : finalists) dup = dup || same(f, t.second);
      if (!dup) finalists.push_back(t.second);
    }
    StageCfg dflt;
    dflt.wait_cycles = wait_cycles;
    bool have_default = false;
    for (const StageCfg& f : finalists) have_default = have_default || same(f, dflt);
    if (!have_default) finalists.push_back(dflt);
    std::vector<std::vector<float>> reps(finalists.size());
    for (int k = 0; k < 3; ++k)
      for (size_t i = 0; i < finalists.size(); ++i) reps[i].push_back(time_once(finalists[i], 4 * trials));
    float final_ms = 1e30f;
    for (size_t i = 0; i < finalists.size(); ++i) {
      std::sort(reps[i].begin(), reps[i].end());
      if (reps[i][1] < final_ms) {
        final_ms = reps[i][1];
        best = finalists[i];
      }
    }
  }
  cfg = best;
  timer.enabled = timing;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  check_device_waits();
  drop_graph();  // launch shapes are baked into a captured graph
  cuda_check(cudaGetLastError(), "autotune");
}

// advect_in_normal_direction (src/my_p4est_level_set.cpp:656-725).
template <int D>
void LevelSet<D>::advect_normal(const double* vn, const double* vn_np1, double* phi, double dt, double* phi_dd, int precision) {
  if (precision == PREC_MIXED) {
    advect_mixed(vn, vn_np1, phi, dt, phi_dd);
    return;
  }
  if (precision != PREC_FP64) throw std::invalid_argument("advect_in_normal_direction: unknown precision mode");
  phi0.alloc(N);
  phi1.alloc(N);
  ddc.alloc((size_t)D * N);
  // the sweeps run on the tables in stencil-pattern order when those exist (phi, the velocities and the given
  // second derivatives gathered into that order, phi and the derivatives scattered back), else on the
  // node-ordered tables; the same bits either way
  const bool sorted = ensure_sorted64();
  const DTab64<D>& T = sorted ? T64s : T64;
  double* phi_u = phi;
  double* dd_u = phi_dd;
  if (sorted) {
    // own buffers: the host entry point passes its staging buffers (ws_vn, ws_dd) in
    s_phi.alloc(N);
    s_vn.alloc(N);
    launch_gather_perm64(phi_u, s_perm.p, s_phi.p, N, stream);
    launch_gather_perm64(vn, s_perm.p, s_vn.p, N, stream);
    phi = s_phi.p;
    vn = s_vn.p;
    if (vn_np1) {
      s_vn1.alloc(N);
      launch_gather_perm64(vn_np1, s_perm.p, s_vn1.p, N, stream);
      vn_np1 = s_vn1.p;
    }
    if (phi_dd) {
      s_dd.alloc((size_t)D * N);
      for (int a = 0; a < D; ++a) launch_gather_perm64(dd_u + (int64_t)a * N, s_perm.p, s_dd.p + (int64_t)a * N, N, stream);
      phi_dd = s_dd.p;
    }
  }
  // stage 1: the quadratic neighbours use laplace(phi) (computed inline by the reference); the
  // minmod terms use the given second derivatives, or the same laplace(phi) when none are given.
  LSG_LAUNCH(K_DD64, launch_dd64<D>(T, phi, ddc.p, stream));
  const double* ddm = phi_dd ? phi_dd : ddc.p;
  cuda_check(cudaMemcpyAsync(phi0.p, phi, N * sizeof(double), cudaMemcpyDeviceToDevice, stream), "copy phi_n");
  LSG_LAUNCH(K_ADVECT64, launch_advect_stage64<D>(T, phi0.p, ddc.p, ddm, vn, dt, phi, nullptr, stream));
  // stage 2 with the derivatives of the intermediate phi (written to the caller's arrays if given)
  double* dd2 = phi_dd ? phi_dd : ddc.p;
  LSG_LAUNCH(K_DD64, launch_dd64<D>(T, phi, dd2, stream));
  LSG_LAUNCH(K_ADVECT64, launch_advect_stage64<D>(T, phi, dd2, dd2, vn_np1 ? vn_np1 : vn, dt, phi1.p, phi0.p, stream));
  if (sorted) {
    launch_scatter_perm64(phi1.p, s_perm.p, phi_u, N, stream);
    if (dd_u)
      for (int a = 0; a < D; ++a) launch_scatter_perm64(phi_dd + (int64_t)a * N, s_perm.p, dd_u + (int64_t)a * N, N, stream);
  } else {
    cuda_check(cudaMemcpyAsync(phi, phi1.p, N * sizeof(double), cudaMemcpyDeviceToDevice, stream), "copy phi");
  }
  cuda_check(cudaGetLastError(), "advect_in_normal_direction");
}

template <int D>
void LevelSet<D>::advect_mixed(const double* vn, const double* vn_np1, double* phi, double dt, double* phi_dd) {
  mixed_join();  // chains left open by a call that stopped on an error
  build_mixed();
  f_phi.alloc(N);
  f_phi0.alloc(N);
  f_phi1.alloc(N);
  f_dd.alloc((size_t)D * N);
  f_vn.alloc(vn_np1 ? 2 * (size_t)N : (size_t)N);
  LSG_LAUNCH(K_CONVERT, launch_gather_f32(phi, perm.p, f_phi0.p, N, 0, 0, 1, stream));
  LSG_LAUNCH(K_CONVERT, launch_gather_f32(vn, perm.p, f_vn.p, N, 0, 0, 1, stream));
  if (vn_np1) LSG_LAUNCH(K_CONVERT, launch_gather_f32(vn_np1, perm.p, f_vn.p + N, N, 0, 0, 1, stream));
  if (!phi_dd) {
    // both RK stages on the reinitialisation's stage kernels (second derivatives rebuilt from second
    // neighbours, the extended set by k_dd_x32, the two-stream schedule); with caller-given second derivatives
    // (used in the minmod terms of the first stage and overwritten) the separate sweeps below run instead
    status.ensure(N);  // the kernels' arguments; the advection stage reads neither
    f_snear.ensure(1);
    mixed_stage(2, f_phi0.p, f_phi.p, nullptr, f_vn.p, (float)dt);
    mixed_stage(2, f_phi.p, f_phi1.p, f_phi0.p, vn_np1 ? f_vn.p + N : f_vn.p, (float)dt);
    mixed_join();
    LSG_LAUNCH(K_CONVERT, launch_scatter_f64(f_phi1.p, perm.p, nullptr, phi, N, 0, 0, 1, stream));
    cuda_check(cudaGetLastError(), "advect_in_normal_direction (mixed)");
    return;
  }
  LSG_LAUNCH(K_DD32, launch_dd32<D>(T32, f_phi0.p, f_dd.p, stream));
  const float* ddm = f_dd.p;
  if (phi_dd) {
    f_ddm.alloc((size_t)D * N);
    LSG_LAUNCH(K_CONVERT, launch_gather_f32(phi_dd, perm.p, f_ddm.p, N, N, N, D, stream));
    ddm = f_ddm.p;
  }
  LSG_LAUNCH(K_ADVECT32, launch_advect_stage32<D>(T32, f_phi0.p, f_dd.p, ddm, f_vn.p, (float)dt, f_phi.p, nullptr, stream));
  LSG_LAUNCH(K_DD32, launch_dd32<D>(T32, f_phi.p, f_dd.p, stream));
  if (phi_dd) LSG_LAUNCH(K_CONVERT, launch_scatter_f64(f_dd.p, perm.p, nullptr, phi_dd, N, N, N, D, stream));
  LSG_LAUNCH(K_ADVECT32, launch_advect_stage32<D>(T32, f_phi.p, f_dd.p, f_dd.p, vn_np1 ? f_vn.p + N : f_vn.p, (float)dt, f_phi1.p,
                                                  f_phi0.p, stream));
  LSG_LAUNCH(K_CONVERT, launch_scatter_f64(f_phi1.p, perm.p, nullptr, phi, N, 0, 0, 1, stream));
  cuda_check(cudaGetLastError(), "advect_in_normal_direction (mixed)");
}

template <int D>
double LevelSet<D>::cfl_dt(const double* vn) {
  dt_dev.alloc(1);
  LSG_LAUNCH(K_CONVERT, launch_min_cfl(smin.p, vn, N, dt_dev.p, stream));
  double dt = 0;
  cuda_check(cudaMemcpyAsync(&dt, dt_dev.p, sizeof(double), cudaMemcpyDeviceToHost, stream), "cfl dt");
  cuda_check(cudaStreamSynchronize(stream), "cfl dt sync");
  return dt;
}

template <int D>
double LevelSet<D>::band_linf(const double* a, const double* b, double band, int64_t* count) {
  linf_buf.ensure(3);
  LSG_LAUNCH(K_CONVERT, launch_band_linf64(a, b, band, N, linf_buf.p, stream));
  unsigned long long h[3] = {0, 0, 0};
  cuda_check(cudaMemcpyAsync(h, linf_buf.p, sizeof(h), cudaMemcpyDeviceToHost, stream), "band check");
  cuda_check(cudaStreamSynchronize(stream), "band check sync");
  if (count) *count = (int64_t)h[1];
  if (h[2]) return NAN;
  double v;
  memcpy(&v, &h[0], sizeof(v));
  return v;
}

template <int D>
double LevelSet<D>::interface_location_error(const double* a, const double* b, int64_t* edges, int64_t* mismatched) {
  linf_buf.ensure(3);
  LSG_LAUNCH(K_CONVERT, launch_iface_err64<D>(T64, a, b, linf_buf.p, stream));
  unsigned long long h[3] = {0, 0, 0};
  cuda_check(cudaMemcpyAsync(h, linf_buf.p, sizeof(h), cudaMemcpyDeviceToHost, stream), "interface check");
  cuda_check(cudaStreamSynchronize(stream), "interface check sync");
  if (edges) *edges = (int64_t)h[1];
  if (mismatched) *mismatched = (int64_t)h[2];
  double v;
  memcpy(&v, &h[0], sizeof(v));
  return v;
}

template <int D>
void LevelSet<D>::reinitialize_host(double* phi, int os, int ot, double hi, double lo, int iters, int precision, const double* mask) {
  ws_phi.alloc(N);
  cuda_check(cudaMemcpyAsync(ws_phi.p, phi, N * sizeof(double), cudaMemcpyHostToDevice, stream), "H2D phi");
  const double* dmask = nullptr;
  if (mask) {
    ws_vn.ensure((size_t)N + 1);
    if (N) cuda_check(cudaMemcpyAsync(ws_vn.p, mask, N * sizeof(double), cudaMemcpyHostToDevice, stream), "H2D mask");
    dmask = ws_vn.p;
  }
  reinitialize(ws_phi.p, os, ot, hi, lo, iters, precision, dmask);
  cuda_check(cudaMemcpyAsync(phi, ws_phi.p, N * sizeof(double), cudaMemcpyDeviceToHost, stream), "D2H phi");
  cuda_check(cudaStreamSynchronize(stream), "reinitialize sync");
}

template <int D>
void LevelSet<D>::build_gradient() {
  if (grad_ready) return;
  if (!F) throw std::invalid_argument("first derivatives need a single grid's level set, not a batch");
  std::vector<int32_t> gidx;
  std::vector<double> grec;
  std::vector<uint8_t> gmask;
  build_gradient_tables<D>(*F, gidx, grec, gmask);
  if (grec.empty()) grec.push_back(0.0);
  if (gmask.empty()) gmask.push_back(0);
  g_idx.upload(gidx, stream);
  g_rec.upload(grec, stream);
  g_mask.upload(gmask, stream);
  cuda_check(cudaStreamSynchronize(stream), "gradient tables upload");
  TG.gidx = g_idx.p;
  TG.grec = g_rec.p;
  TG.gmask = g_mask.p;
  grad_ready = true;
}

template <int D>
void LevelSet<D>::first_derivatives(const double* f, double* out) {
  build_gradient();
  ws_gdd.ensure((size_t)D * N);
  LSG_LAUNCH(K_DD64, launch_dd64<D>(T64, f, ws_gdd.p, stream));
  LSG_LAUNCH(K_DD64, launch_grad64<D>(T64, TG, f, ws_gdd.p, out, (1 << D) - 1, stream));
  cuda_check(cudaGetLastError(), "first_derivatives_central");
}

template <int D>
void LevelSet<D>::compute_normals(const double* phi, double* out) {
  first_derivatives(phi, out);
  LSG_LAUNCH(K_CONVERT, launch_normalize64<D>(out, N, stream));
  cuda_check(cudaGetLastError(), "compute_normals");
}

template <int D>
void LevelSet<D>::mean_curvature_from_normals(const double* nrm, double* kappa) {
  build_gradient();
  ws_gdd2.ensure((size_t)D * D * N);
  for (int a = 0; a < D; ++a) LSG_LAUNCH(K_DD64, launch_dd64<D>(T64, nrm + (size_t)a * N, ws_gdd2.p + (size_t)a * D * N, stream));
  LSG_LAUNCH(K_DD64, launch_div64<D>(T64, TG, nrm, ws_gdd2.p, kappa, stream));
  cuda_check(cudaGetLastError(), "compute_mean_curvature");
}

template <int D>
void LevelSet<D>::normals_and_mean_curvature(const double* phi, double* nrm, double* kappa) {
  first_derivatives(phi, nrm);  // ws_gdd holds the second derivatives of phi
  ws_gdd2.ensure((size_t)D * D * N);
  for (int a = 0; a < D - 1; ++a) LSG_LAUNCH(K_DD64, launch_dd64<D>(T64, nrm + (size_t)a * N, ws_gdd2.p + (size_t)a * D * N, stream));
  LSG_LAUNCH(K_DD64, launch_kappa64<D>(T64, TG, nrm, ws_gdd.p, ws_gdd2.p, ws_gdd2.p + (size_t)D * N, kappa, stream));
  LSG_LAUNCH(K_CONVERT, launch_normalize64<D>(nrm, N, stream));
  cuda_check(cudaGetLastError(), "compute_normals_and_mean_curvature");
}

template <int D>
void LevelSet<D>::extend_over_interface(const double* phi, double* q, int iterations, int order, double band_use, double band_extend,
                                        const double* normals, const double* mask, bool nonzero_guess, double* q_n, double* q_nn) {
  if (order < 0 || order > 2) throw std::invalid_argument("extend_Over_Interface_TVD: order must be 0, 1 or 2.");
  if (iterations < 0) throw std::invalid_argument("extend_Over_Interface_TVD: negative number of iterations");
  build_gradient();
  if (band_use > 0) band_use = -band_use;
  if (!mask) mask = phi;
  const size_t n = (size_t)N;
  // layout of ext_buf: normals D | qx D | qn | qnn | tmp | qdd D | nrmdd D*D | qxdd D*D | qndd D
  ext_buf.ensure((size_t)(2 * D + 3 + D + 2 * D * D + D) * n + 1);
  double* nrm_own = ext_buf.p;
  double* qx = nrm_own + (size_t)D * n;
  double* qn = qx + (size_t)D * n;
  double* qnn = qn + n;
  double* tmp = qnn + n;
  double* qdd = tmp + n;
  double* nrmdd = qdd + (size_t)D * n;
  double* qxdd = nrmdd + (size_t)D * D * n;
  double* qndd = qxdd + (size_t)D * D * n;
  ext_b1.ensure(n + 1);
  ext_b2.ensure(n + 1);
  const double* nrm = normals;
  if (!nrm) {
    compute_normals(phi, nrm_own);
    nrm = nrm_own;
  }
  if (order >= 1) {
    LSG_LAUNCH(K_DD64, launch_dd64<D>(T64, q, qdd, stream));
    // a caller's q_n starts the marching where nothing is computed (the reference works in it)
    if (q_n) cuda_check(cudaMemcpyAsync(qn, q_n, n * sizeof(double), cudaMemcpyDeviceToDevice, stream), "copy q_n");
    const int guess1 = (nonzero_guess ? EXT_GUESS_GRADIENT : 0) | (q_n ? EXT_GUESS_KEEP : 0);
    LSG_LAUNCH(K_DD64, launch_ext_init1<D>(T64, TG, phi, mask, q, qdd, nrm, band_use, guess1, qx, qn, ext_b1.p, stream));
  }
  if (order == 2) {
    if (!cnb.p) {
      std::vector<int32_t> c;
      build_corner_neighbors<D>(*F, c);
      cnb.upload(c, stream);
    }
    for (int a = 0; a < D; ++a) {
      LSG_LAUNCH(K_DD64, launch_dd64<D>(T64, nrm + (size_t)a * n, nrmdd + (size_t)a * D * n, stream));
      LSG_LAUNCH(K_DD64, launch_dd64<D>(T64, qx + (size_t)a * n, qxdd + (size_t)a * D * n, stream));
    }
    if (q_nn) cuda_check(cudaMemcpyAsync(qnn, q_nn, n * sizeof(double), cudaMemcpyDeviceToDevice, stream), "copy q_nn");
    if (nonzero_guess) LSG_LAUNCH(K_DD64, launch_dd64<D>(T64, qn, qndd, stream));
    const int guess2 = (nonzero_guess ? EXT_GUESS_GRADIENT : 0) | (q_nn ? EXT_GUESS_KEEP : 0);
    LSG_LAUNCH(K_DD64, launch_ext_init2<D>(T64, TG, phi, mask, q, qdd, nrm, nrmdd, qx, qxdd, ext_b1.p, cnb.p, band_use, guess2, qn, qndd,
                                           qnn, ext_b2.p, stream));
  }
  // marching: ping-pong between a field and tmp; nodes not marched keep their value in both
  auto march = [&](double* v, const int8_t* b, const double* src) {
    double* a = v;
    double* t = tmp;
    cuda_check(cudaMemcpyAsync(t, a, n * sizeof(double), cudaMemcpyDeviceToDevice, stream), "copy");
    for (int it = 0; it < iterations; ++it) {
      LSG_LAUNCH(K_ADVECT64, launch_ext_march<D>(T64, a, t, b, phi, nrm, src, band_extend, stream));
      std::swap(a, t);
    }
    if (a != v) cuda_check(cudaMemcpyAsync(v, a, n * sizeof(double), cudaMemcpyDeviceToDevice, stream), "copy");
  };
  if (order == 2) march(qnn, ext_b2.p, nullptr);
  if (order >= 1) march(qn, ext_b1.p, order == 2 ? qnn : nullptr);
  {
    double* a = q;
    double* t = tmp;
    cuda_check(cudaMemcpyAsync(t, a, n * sizeof(double), cudaMemcpyDeviceToDevice, stream), "copy");
    for (int it = 0; it < iterations; ++it) {
      if (order == 2) LSG_LAUNCH(K_DD64, launch_dd64<D>(T64, a, qdd, stream));
      LSG_LAUNCH(K_ADVECT64, launch_ext_q<D>(T64, a, t, qdd, phi, mask, nrm, qn, order, band_extend, stream));
      std::swap(a, t);
    }
    if (a != q) cuda_check(cudaMemcpyAsync(q, a, n * sizeof(double), cudaMemcpyDeviceToDevice, stream), "copy");
  }
  // the extended normal derivatives back to the caller
  if (q_n && order >= 1) cuda_check(cudaMemcpyAsync(q_n, qn, n * sizeof(double), cudaMemcpyDeviceToDevice, stream), "copy q_n");
  if (q_nn && order == 2) cuda_check(cudaMemcpyAsync(q_nn, qnn, n * sizeof(double), cudaMemcpyDeviceToDevice, stream), "copy q_nn");
  cuda_check(cudaGetLastError(), "extend_Over_Interface_TVD");
}

template <int D>
void LevelSet<D>::extend_from_interface(const double* phi, const double* qi, double* q, int nf, int iterations, const double* mask,
                                        double band_zero, double band_smooth, const double* grad_phi, int method, InterfaceValuesFn cf,
                                        void* cf_ctx) {
  if (nf < 1) throw std::invalid_argument("extend_from_interface_to_whole_domain_TVD: at least one field");
  if (cf && mask) throw std::invalid_argument("extend_from_interface_to_whole_domain_TVD: no mask and cf simultaneously");
  if (cf && nf > 1) throw std::invalid_argument("extend_from_interface_to_whole_domain_TVD: cf needs a block size of 1");
  if (mask && nf > 1) throw std::invalid_argument("extend_from_interface_to_whole_domain_TVD: a mask needs a block size of 1");
  if (method < 0 || method > 4) throw std::invalid_argument("extend_from_interface_to_whole_domain_TVD: unknown interpolation method");
  if (iterations < 0) throw std::invalid_argument("extend_from_interface_to_whole_domain_TVD: negative number of iterations");
  const size_t n = (size_t)N;
  if (n && q < qi + (size_t)nf * n && qi < q + (size_t)nf * n)
    throw std::invalid_argument("extend_from_interface_to_whole_domain_TVD: q and q_interface overlap");
  build_gradient();
  build_locator();
  if (!node_xyz_dev.p) {
    std::vector<double> x((size_t)D * n + 1);
    for (int64_t k = 0; k < N; ++k) F->node_xyz((int32_t)k, &x[(size_t)D * k]);
    node_xyz_dev.upload(x, stream);
  }
  // dl = max over the axes of the tree size / 2^max_lvl
  const int max_lvl = F->max_level();
  double dl = TL.tree_dim[0] / pow(2., (double)max_lvl);
  for (int a = 1; a < D; ++a) dl = std::max(dl, TL.tree_dim[a] / pow(2., (double)max_lvl));
  // layout of efi_buf: grad D | phi dd D | qi dd D | qi_nb 2D | s_nb 2D | q1 | qdd D | qdd2 D*D
  efi_buf.ensure((size_t)(8 * D + 1 + D * D) * n + 1);
  double* grad_own = efi_buf.p;
  double* pdd = grad_own + (size_t)D * n;
  double* qidd = pdd + (size_t)D * n;
  double* qi_nb = qidd + (size_t)D * n;
  double* s_nb = qi_nb + (size_t)2 * D * n;
  double* q1 = s_nb + (size_t)2 * D * n;
  double* qdd = q1 + n;
  double* qdd2 = qdd + (size_t)D * n;
  efi_cross.ensure(n + 1);
  const double* grad = grad_phi;
  if (!grad) {
    first_derivatives(phi, grad_own);
    grad = grad_own;
  }
  LSG_LAUNCH(K_DD64, launch_dd64<D>(T64, phi, pdd, stream));
  auto derivatives = [&](const double* f) {
    LSG_LAUNCH(K_DD64, launch_dd64<D>(T64, f, qdd, stream));
    for (int a = 0; a < D; ++a) LSG_LAUNCH(K_DD64, launch_dd64<D>(T64, qdd + (size_t)a * n, qdd2 + (size_t)a * D * n, stream));
  };
  for (int k = 0; k < nf; ++k) {
    const double* qik = qi + (size_t)k * n;
    double* qk = q + (size_t)k * n;
    LSG_LAUNCH(K_DD64, launch_dd64<D>(T64, qik, qidd, stream));
    LSG_LAUNCH(K_INTERP, launch_efi_init64<D>(T64, TL, cf ? -1 : method, node_xyz_dev.p, phi, pdd, qik, qidd, mask, dl, band_zero * dl,
                                              band_smooth * dl, qk, qi_nb, s_nb, efi_cross.p, stream));
    if (cf) {
      // the crossing (node, direction) pairs in node order, their distances to the host, the caller's
      // values back into qi_nb
      std::vector<uint8_t> cross(n);
      if (n) cuda_check(cudaMemcpyAsync(cross.data(), efi_cross.p, n, cudaMemcpyDeviceToHost, stream), "D2H");
      cuda_check(cudaStreamSynchronize(stream), "interface crossings");
      std::vector<int64_t> idx;
      std::vector<int32_t> nodes, dirs;
      for (size_t m = 0; m < n; ++m)
        for (int dir = 0; dir < 2 * D; ++dir)
          if ((cross[m] >> dir) & 1) {
            idx.push_back((int64_t)dir * N + (int64_t)m);
            nodes.push_back((int32_t)m);
            dirs.push_back(dir);
          }
      const int64_t cnt = (int64_t)idx.size();
      std::vector<double> dist((size_t)cnt), val((size_t)cnt);
      efi_idx.ensure((size_t)cnt + 1);
      efi_val.ensure((size_t)cnt + 1);
      if (cnt) {
        cuda_check(cudaMemcpyAsync(efi_idx.p, idx.data(), (size_t)cnt * sizeof(int64_t), cudaMemcpyHostToDevice, stream), "H2D");
        LSG_LAUNCH(K_INTERP, launch_gather_idx64(s_nb, efi_idx.p, cnt, efi_val.p, stream));
        cuda_check(cudaMemcpyAsync(dist.data(), efi_val.p, (size_t)cnt * sizeof(double), cudaMemcpyDeviceToHost, stream), "D2H");
        cuda_check(cudaStreamSynchronize(stream), "interface distances");
        if (cf(cf_ctx, cnt, nodes.data(), dirs.data(), dist.data(), val.data()) != 0)
          throw std::runtime_error("extend_from_interface_to_whole_domain_TVD: the cf callback failed");
        cuda_check(cudaMemcpyAsync(efi_val.p, val.data(), (size_t)cnt * sizeof(double), cudaMemcpyHostToDevice, stream), "H2D");
        LSG_LAUNCH(K_INTERP, launch_scatter_idx64(efi_val.p, efi_idx.p, cnt, qi_nb, stream));
        cuda_check(cudaStreamSynchronize(stream), "interface values");  // the host vectors go out of scope
      }
    }
    for (int it = 0; it < iterations; ++it) {
      derivatives(qk);
      LSG_LAUNCH(K_ADVECT64, launch_efi_stage64<D>(T64, phi, grad, qk, qdd, qdd2, qi_nb, s_nb, efi_cross.p, zdt, false, q1, stream));
      derivatives(q1);
      LSG_LAUNCH(K_ADVECT64, launch_efi_stage64<D>(T64, phi, grad, q1, qdd, qdd2, qi_nb, s_nb, efi_cross.p, zdt, true, qk, stream));
    }
  }
  cuda_check(cudaGetLastError(), "extend_from_interface_to_whole_domain_TVD");
}

// Point location tables: sorted leaf keys and levels, local_nodes, and the coarse-cell table
// (my_p4est_hierarchy_t's role, src/my_p4est_hierarchy.cpp:264-567).
template <int D>
void LevelSet<D>::build_locator() {
  if (loc_ready) return;
  if (!F) throw std::invalid_argument("interpolation needs a single grid's level set, not a batch");
  using DD = Dim<D>;
  const Forest<D>& f = *F;
  const int64_t nl = (int64_t)f.leaves.size();
  const int nt = f.brick.num_trees;
  int L0 = 0;
  while (L0 < DD::MAXLEVEL && ((int64_t)nt << (D * (L0 + 1))) <= 2 * nl) ++L0;
  const int64_t ncoarse = int64_t(1) << (D * L0);
  if (fdev) {
    // the coarse-cell table by binary searches over the device copy's leaf keys
    const ForestDevice<D>& X = *static_cast<const ForestDevice<D>*>(fdev.get());
    loc_ctab.alloc((size_t)(nt * ncoarse + 1));
    coarse_table_device<D>(X.leaf_key.p, nl, nt, L0, loc_ctab.p, stream);
  } else {
    std::vector<int32_t> ctab((size_t)(nt * ncoarse + 1));
    // merge the coarse cells' first points (in key order) with the sorted leaf keys
    int64_t j = 0;
    for (int64_t i = 0; i < nt * ncoarse; ++i) {
      const uint64_t t = (uint64_t)(i / ncoarse), c = (uint64_t)(i % ncoarse);
      const uint64_t key = (t << tree_shift<D>()) | (c << (D * (DD::MAXLEVEL - L0)));
      while (j + 1 < nl && f.leaf_key[(size_t)(j + 1)] <= key) ++j;
      ctab[(size_t)i] = (int32_t)j;
    }
    ctab[(size_t)(nt * ncoarse)] = (int32_t)(nl - 1);
    loc_ctab.upload(ctab, stream);
  }
  if (fdev) {
    // the forest's device copy already holds the leaves, corner nodes and brick
    const ForestDevice<D>& X = *static_cast<const ForestDevice<D>*>(fdev.get());
    TL.key = X.leaf_key.p;
    TL.level = X.level.p;
    TL.local_nodes = X.local_nodes.p;
    TL.ijk_to_tree = X.ijk_to_tree.p;
    TL.tmin = X.tmin.p;
    TL.tmax = X.tmax.p;
  } else {
    std::vector<int8_t> lvl((size_t)nl);
    for (int64_t q = 0; q < nl; ++q) lvl[(size_t)q] = (int8_t)f.leaves[(size_t)q].level;
    loc_key.upload(f.leaf_key.vec(), stream);
    loc_level.upload(lvl, stream);
    loc_nodes.upload(f.nd->host().local_nodes, stream);
    loc_ijk.upload(f.brick.ijk_to_tree, stream);
    loc_tmin.upload(f.brick.tmin, stream);
    loc_tmax.upload(f.brick.tmax, stream);
    TL.key = loc_key.p;
    TL.level = loc_level.p;
    TL.local_nodes = loc_nodes.p;
    TL.ijk_to_tree = loc_ijk.p;
    TL.tmin = loc_tmin.p;
    TL.tmax = loc_tmax.p;
  }
  cuda_check(cudaStreamSynchronize(stream), "locator upload");
  TL.nleaves = nl;
  TL.N = N;
  TL.ctab = loc_ctab.p;
  TL.L0 = L0;
  TL.ncoarse = ncoarse;
  for (int a = 0; a < 3; ++a) {
    TL.n[a] = f.brick.n[a];
    TL.xyz_min[a] = f.brick.xyz_min[a];
    TL.xyz_max[a] = f.brick.xyz_max[a];
    TL.tree_dim[a] = (f.brick.xyz_max[a] - f.brick.xyz_min[a]) / f.brick.n[a];
  }
  loc_ready = true;
}

// Second derivatives of nf fields (nf x D x N): the caller's, or computed as compute_derivatives does.
template <int D>
const double* LevelSet<D>::derivatives_of(int nf, const double* Fv, const double* Fdd, DevBuf<double>& store) {
  if (Fdd) return Fdd;
  store.ensure((size_t)nf * D * N);
  for (int k = 0; k < nf; ++k) LSG_LAUNCH(K_DD64, launch_dd64<D>(T64, Fv + (size_t)k * N, store.p + (size_t)k * D * N, stream));
  return store.p;
}

static void check_method(int m) {
  if (m < 0 || m > 4) throw std::invalid_argument("unknown interpolation_method");
}

template <int D>
void LevelSet<D>::interpolate(const double* xyz, int64_t np, int nf, const double* Fv, const double* Fdd, int method, double* out) {
  check_method(method);
  if (nf < 1) throw std::invalid_argument("interpolate: at least one input field is needed");
  if (np < 0) throw std::invalid_argument("interpolate: negative number of points");
  build_locator();
  const double* dd = method == 0 ? nullptr : derivatives_of(nf, Fv, Fdd, ws_fdd);
  LSG_LAUNCH(K_INTERP, launch_interp64<D>(TL, method, xyz, np, nullptr, 0.0, nf, Fv, dd, out, stream));
  cuda_check(cudaGetLastError(), "interpolate");
}

template <int D>
void LevelSet<D>::locate(const double* xyz, int64_t np, int32_t* leaf) {
  build_locator();
  LSG_LAUNCH(K_INTERP, launch_locate64<D>(TL, xyz, np, leaf, stream));
  cuda_check(cudaGetLastError(), "locate");
}

// advect_from_n_to_np1 (src/my_p4est_semi_lagrangian.cpp:148-223): three interpolation rounds, the
// second and third at x - dt/2 v and x - dt v* (clipped), each one launch.
template <int D>
void LevelSet<D>::sl_advect(const double* xyz, int64_t np, double dt, const double* v, const double* vdd, const double* phi,
                            const double* phi_dd, int velo_method, int phi_method, double* phi_np1) {
  check_method(velo_method);
  check_method(phi_method);
  if (np < 0) throw std::invalid_argument("advect_from_n_to_np1: negative number of points");
  build_locator();
  const double* vd = velo_method == 0 ? nullptr : derivatives_of(D, v, vdd, ws_fdd);
  const double* pd = phi_method == 0 ? nullptr : derivatives_of(1, phi, phi_dd, ws_fdd2);
  ws_v1.ensure((size_t)D * np);
  ws_v2.ensure((size_t)D * np);
  LSG_LAUNCH(K_INTERP, launch_interp64<D>(TL, velo_method, xyz, np, nullptr, 0.0, D, v, vd, ws_v1.p, stream));
  LSG_LAUNCH(K_INTERP, launch_interp64<D>(TL, velo_method, xyz, np, ws_v1.p, 0.5 * dt, D, v, vd, ws_v2.p, stream));
  LSG_LAUNCH(K_INTERP, launch_interp64<D>(TL, phi_method, xyz, np, ws_v2.p, dt, 1, phi, pd, phi_np1, stream));
  cuda_check(cudaGetLastError(), "advect_from_n_to_np1");
}

// advect_from_n_to_np1(dt_nm1, dt_n, vnm1, vxx_nm1, vn, vxx_n, phi_n, phi_xx_n, phi_np1)
// (src/my_p4est_semi_lagrangian.cpp:225-319): v_n at the new nodes by quadratic interpolation (the
// reference fixes that method for this round), then at x* = x - dt_n/2 v_n (clipped) v_n on this grid and
// v_nm1 on grid n-1 with velo_method, and phi_n at x_d = x - dt_n v* with v* = (1 + dt_n/(2 dt_nm1)) v_n(x*) -
// dt_n/(2 dt_nm1) v_nm1(x*). Four launches, all on this object's stream.
template <int D>
void LevelSet<D>::sl_advect2(LevelSet<D>& nm1, const double* xyz, int64_t np, double dt_nm1, double dt_n, const double* vnm1,
                             const double* vnm1_dd, const double* vn, const double* vn_dd, const double* phi, const double* phi_dd,
                             int velo_method, int phi_method, double* phi_np1) {
  check_method(velo_method);
  check_method(phi_method);
  if (np < 0) throw std::invalid_argument("advect_from_n_to_np1: negative number of points");
  if (!(dt_nm1 > 0.0)) throw std::invalid_argument("advect_from_n_to_np1: dt_nm1 must be positive");
  build_locator();
  nm1.build_locator();
  const double* vd = derivatives_of(D, vn, vn_dd, ws_fdd);  // the quadratic round needs them whatever velo_method is
  const double* md = nullptr;
  if (velo_method != 0) {
    md = vnm1_dd;
    if (!md) {  // as compute_derivatives does on grid n-1, on this stream
      ws_fdd3.ensure((size_t)D * D * nm1.N);
      for (int k = 0; k < D; ++k)
        LSG_LAUNCH(K_DD64, launch_dd64<D>(nm1.T64, vnm1 + (size_t)k * nm1.N, ws_fdd3.p + (size_t)k * D * nm1.N, stream));
      md = ws_fdd3.p;
    }
  }
  const double* pd = phi_method == 0 ? nullptr : derivatives_of(1, phi, phi_dd, ws_fdd2);
  ws_v1.ensure((size_t)D * np + 1);
  ws_v2.ensure((size_t)D * np + 1);
  ws_v3.ensure((size_t)D * np + 1);
  LSG_LAUNCH(K_INTERP, launch_interp64<D>(TL, 1, xyz, np, nullptr, 0.0, D, vn, vd, ws_v1.p, stream));
  LSG_LAUNCH(K_INTERP, launch_interp64<D>(nm1.TL, velo_method, xyz, np, ws_v1.p, 0.5 * dt_n, D, vnm1, md, ws_v3.p, stream));
  LSG_LAUNCH(K_INTERP, launch_interp64<D>(TL, velo_method, xyz, np, ws_v1.p, 0.5 * dt_n, D, vn, velo_method == 0 ? nullptr : vd,
                                          ws_v2.p, stream));
  const double ca = 1.0 + .5 * dt_n / dt_nm1, cb = 0.5 * dt_n / dt_nm1;
  LSG_LAUNCH(K_INTERP, launch_sl2_phi64<D>(TL, phi_method, xyz, np, ws_v2.p, ws_v3.p, ca, cb, dt_n, phi, pd, phi_np1, stream));
  cuda_check(cudaGetLastError(), "advect_from_n_to_np1 (two velocities)");
}

template <int D>
void LevelSet<D>::sl_advect_vortex(const double* xyz, int64_t np, double dt, double vscale, const double* phi, const double* phi_dd,
                                   int phi_method, double* phi_np1) {
  check_method(phi_method);
  if (np < 0) throw std::invalid_argument("advect_from_n_to_np1: negative number of points");
  build_locator();
  const double* pd = phi_method == 0 ? nullptr : derivatives_of(1, phi, phi_dd, ws_fdd2);
  LSG_LAUNCH(K_INTERP, launch_sl_vortex64<D>(TL, phi_method, xyz, np, dt, vscale, phi, pd, phi_np1, stream));
  cuda_check(cudaGetLastError(), "advect_from_n_to_np1 (single vortex)");
}

static void h2d(double* dst, const double* src, size_t n, cudaStream_t s) {
  if (n) cuda_check(cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyHostToDevice, s), "H2D");
}

template <int D>
void LevelSet<D>::interpolate_host(const double* xyz, int64_t np, int nf, const double* Fv, const double* Fdd, int method, double* out) {
  ws_xyz.ensure((size_t)D * np + 1);
  ws_f.ensure((size_t)nf * N);
  ws_out.ensure((size_t)nf * np + 1);
  h2d(ws_xyz.p, xyz, (size_t)D * np, stream);
  h2d(ws_f.p, Fv, (size_t)nf * N, stream);
  const double* dd = nullptr;
  if (Fdd && method != 0) {
    ws_fdd.ensure((size_t)nf * D * N);
    h2d(ws_fdd.p, Fdd, (size_t)nf * D * N, stream);
    dd = ws_fdd.p;
  }
  interpolate(ws_xyz.p, np, nf, ws_f.p, dd, method, ws_out.p);
  if (np) cuda_check(cudaMemcpyAsync(out, ws_out.p, (size_t)nf * np * sizeof(double), cudaMemcpyDeviceToHost, stream), "D2H");
  cuda_check(cudaStreamSynchronize(stream), "interpolate sync");
}

template <int D>
void LevelSet<D>::sl_advect_host(const double* xyz, int64_t np, double dt, const double* v, const double* vdd, const double* phi,
                                 const double* phi_dd, int velo_method, int phi_method, double* phi_np1) {
  // staging: xyz | v | phi | vdd | phi_dd in ws_f, the result in ws_out
  const size_t nx = (size_t)D * np, nv = (size_t)D * N, nvd = vdd ? (size_t)D * D * N : 0, npd = phi_dd ? (size_t)D * N : 0;
  ws_xyz.ensure(nx + 1);
  ws_f.ensure(nv + N + nvd + npd);
  ws_out.ensure((size_t)np + 1);
  double* dv = ws_f.p;
  double* dphi = dv + nv;
  double* dvdd = vdd ? dphi + N : nullptr;
  double* dpdd = phi_dd ? dphi + N + nvd : nullptr;
  h2d(ws_xyz.p, xyz, nx, stream);
  h2d(dv, v, nv, stream);
  h2d(dphi, phi, N, stream);
  if (vdd) h2d(dvdd, vdd, nvd, stream);
  if (phi_dd) h2d(dpdd, phi_dd, npd, stream);
  sl_advect(ws_xyz.p, np, dt, dv, dvdd, dphi, dpdd, velo_method, phi_method, ws_out.p);
  if (np) cuda_check(cudaMemcpyAsync(phi_np1, ws_out.p, (size_t)np * sizeof(double), cudaMemcpyDeviceToHost, stream), "D2H");
  cuda_check(cudaStreamSynchronize(stream), "advect_from_n_to_np1 sync");
}

template <int D>
void LevelSet<D>::sl_advect_vortex_host(const double* xyz, int64_t np, double dt, double vscale, const double* phi, const double* phi_dd,
                                        int phi_method, double* phi_np1) {
  const size_t nx = (size_t)D * np, npd = phi_dd ? (size_t)D * N : 0;
  ws_xyz.ensure(nx + 1);
  ws_f.ensure(N + npd);
  ws_out.ensure((size_t)np + 1);
  h2d(ws_xyz.p, xyz, nx, stream);
  h2d(ws_f.p, phi, N, stream);
  double* dpdd = phi_dd ? ws_f.p + N : nullptr;
  if (phi_dd) h2d(dpdd, phi_dd, npd, stream);
  sl_advect_vortex(ws_xyz.p, np, dt, vscale, ws_f.p, dpdd, phi_method, ws_out.p);
  if (np) cuda_check(cudaMemcpyAsync(phi_np1, ws_out.p, (size_t)np * sizeof(double), cudaMemcpyDeviceToHost, stream), "D2H");
  cuda_check(cudaStreamSynchronize(stream), "advect_from_n_to_np1 sync");
}

template <int D>
void LevelSet<D>::sl_advect2_host(LevelSet<D>& nm1, const double* xyz, int64_t np, double dt_nm1, double dt_n, const double* vnm1,
                                  const double* vnm1_dd, const double* vn, const double* vn_dd, const double* phi, const double* phi_dd,
                                  int velo_method, int phi_method, double* phi_np1) {
  const size_t Nm = (size_t)nm1.N;
  DevBuf<double> d_xyz, d_vn, d_vm, d_phi, d_vnd, d_vmd, d_pd, d_out;
  d_xyz.alloc((size_t)D * np + 1);
  d_vn.alloc((size_t)D * N);
  d_vm.alloc((size_t)D * Nm + 1);
  d_phi.alloc((size_t)N);
  d_out.alloc((size_t)np + 1);
  h2d(d_xyz.p, xyz, (size_t)D * np, stream);
  h2d(d_vn.p, vn, (size_t)D * N, stream);
  h2d(d_vm.p, vnm1, (size_t)D * Nm, stream);
  h2d(d_phi.p, phi, (size_t)N, stream);
  if (vn_dd) {
    d_vnd.alloc((size_t)D * D * N);
    h2d(d_vnd.p, vn_dd, (size_t)D * D * N, stream);
  }
  if (vnm1_dd) {
    d_vmd.alloc((size_t)D * D * Nm + 1);
    h2d(d_vmd.p, vnm1_dd, (size_t)D * D * Nm, stream);
  }
  if (phi_dd) {
    d_pd.alloc((size_t)D * N);
    h2d(d_pd.p, phi_dd, (size_t)D * N, stream);
  }
  sl_advect2(nm1, d_xyz.p, np, dt_nm1, dt_n, d_vm.p, vnm1_dd ? d_vmd.p : nullptr, d_vn.p, vn_dd ? d_vnd.p : nullptr, d_phi.p,
             phi_dd ? d_pd.p : nullptr, velo_method, phi_method, d_out.p);
  if (np) cuda_check(cudaMemcpyAsync(phi_np1, d_out.p, (size_t)np * sizeof(double), cudaMemcpyDeviceToHost, stream), "D2H");
  cuda_check(cudaStreamSynchronize(stream), "advect_from_n_to_np1 sync");
}

template struct LevelSet<2>;
template struct LevelSet<3>;

}  // namespace lsg
