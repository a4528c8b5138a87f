// Device-resident level-set operator: the GPU counterpart of my_p4est_level_set_t
// (src/my_p4est_level_set.h:203-848) restricted to reinitialisation and normal-direction advection.
//
// One object per grid. Construction flattens the node neighbours into device tables (once per grid,
// as the reference's init_neighbors caches one record per node); the work vectors the reference
// creates and destroys inside every call (src/my_p4est_level_set.cpp:323-344, 527-544) are allocated
// on first use and kept.
#pragma once
#include <cuda_runtime.h>

#include <memory>
#include <utility>
#include <vector>

#include "devbuf.hpp"
#include "kernels.h"
#include "tables.hpp"

namespace lsg {

enum Precision { PREC_FP64 = 0, PREC_MIXED = 1 };

// Kernel classes for the optional per-launch timing (CUDA events around each launch).
enum KernelKind {
  K_DD64 = 0, K_PREP64, K_STAGE64, K_ADVECT64, K_DD32, K_PREP_MIXED, K_STAGE32, K_ADVECT32, K_CONVERT, K_COPY, K_INTERP, K_NUM_KINDS
};

struct KernelTimer {
  bool enabled = false;
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> pending;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pool;
  size_t used = 0;
  double ms[K_NUM_KINDS] = {0};
  int64_t count[K_NUM_KINDS] = {0};
  int64_t launches = 0;  // all launches of this object's kernels, timed or not
  ~KernelTimer();
  void begin(int kind, cudaStream_t s);
  void end(cudaStream_t s);
  void collect();  // synchronises the recorded events and accumulates their durations
  void reset();
};

template <int D>
struct LevelSet {
  static constexpr int DIM = D;
  static constexpr int H = Dim<D>::HALF;
  static constexpr int NS = 2 * D * H;
  const Forest<D>* F = nullptr;
  int64_t N = 0;
  double zdt = 0;  // zero_distance_threshold = EPS * min(tree dimensions) (src/my_p4est_level_set.h:388)
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  KernelTimer timer;
  cudaStream_t side_stream = nullptr;  // second stream of the mixed stage (fork/join with events)
  cudaStream_t side_hi = nullptr, main_hi = nullptr;  // the same at the highest stream priority (cfg.priority 1, 2)
  cudaEvent_t ev_fork = nullptr, ev_ddx = nullptr, ev_join = nullptr, ev_main = nullptr;
  StageCfg cfg;                        // launch shape of the mixed stage kernels (see autotune)
  DevBuf<int> kerr;                    // set by a device-side wait that gave up (bulk-copy uniform kernel)
  int64_t num_corrections = 0;

  // FP64 tables
  DevBuf<int32_t> nbr, cidx;
  DevBuf<double> w, nrm, d, q, crec, smin;
  DevBuf<uint8_t> wall;
  DTab64<D> T64{};
  // the FP64 tables in stencil-pattern order (launch_sort_tab64), built on the first FP64 reinitialisation;
  // if device memory runs out the reinitialisation keeps the node-ordered tables
  bool sorted64_ready = false, sorted64_failed = false;
  DevBuf<int32_t> s_perm, s_iperm, s_nbr, s_cidx;
  DevBuf<double> s_w, s_nrm, s_d, s_q, s_phi, s_vn, s_vn1, s_dd;  // s_vn..s_dd: advection inputs in pattern order
  DevBuf<uint32_t> s_word;  // per-node pattern word of the sorted tables (DTab64::word)
  DevBuf<uint8_t> s_wall;
  DTab64<D> T64s{};
  bool ensure_sorted64();
  // mixed tables (built on first mixed call)
  bool mixed_ready = false;
  DevBuf<uint32_t> r_meta, i_meta, r_meta2, i_cls;
  DevBuf<int32_t> r_nbr, r_nbr2, i_nbr, i_cidx, perm, iperm, near_list;
  DevBuf<int4> u_pack;  // the regular nodes' stencil indices node by node (DTab32::u_pack)
  DevBuf<unsigned> near_count;
  DevBuf<float> i_wf, i_d, i_q, corr32, cls32;
  DevBuf<double> i_wf64, i_d64, i_q64, corr64;
  DTab32<D> T32{};
  int64_t nR = 0, nI = 0, ncls = 0;
  // point location tables for node interpolation (built on first use)
  bool loc_ready = false;
  DevBuf<uint64_t> loc_key;
  DevBuf<int8_t> loc_level;
  DevBuf<int32_t> loc_nodes, loc_ctab, loc_ijk, loc_leaf;
  DevBuf<double> loc_tmin, loc_tmax;
  DLoc<D> TL{};
  // edge-diagonal neighbours for the order-2 extension (built on first use)
  DevBuf<int32_t> cnb;
  DevBuf<int8_t> ext_b1, ext_b2;
  DevBuf<double> ext_buf;
  // extension from the interface: node coordinates (N x D, built on first use), work vectors, crossing bits
  DevBuf<double> node_xyz_dev, efi_buf;
  DevBuf<uint8_t> efi_cross;
  DevBuf<int64_t> efi_idx;
  DevBuf<double> efi_val;
  // first-derivative correction records (built on first use)
  bool grad_ready = false;
  DevBuf<int32_t> g_idx;
  DevBuf<double> g_rec;
  DevBuf<uint8_t> g_mask;
  DGrad TG{};
  // work vectors
  DevBuf<double> ws_phi, phi0, phi1, dd0, ddc, snear, ws_vn, ws_vn1, ws_dd, dt_dev;
  DevBuf<double> ws_gdd, ws_gdd2;
  DevBuf<double> ws_xyz, ws_f, ws_fdd, ws_out, ws_v1, ws_v2, ws_v3, ws_fdd2, ws_fdd3;
  DevBuf<unsigned long long> linf_buf;
  DevBuf<uint16_t> status;
  DevBuf<float> f_phi0, f_phi, f_phi1, f_dd, f_ddm, f_snear, f_vn;

  // batched runs over the disjoint union of several grids (constructed from their tables)
  std::vector<int64_t> part_offsets;   // node offset of each grid (+ total)
  DevBuf<uint16_t> iter_lim;           // device order: iteration count of the node's grid
  std::vector<int> part_iters;         // iteration count of each grid (last batched call)
  cudaStream_t capture_stream = nullptr;  // graphs are captured here (the caller's stream may be the legacy default stream)
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t graph_exec = nullptr;
  std::vector<int> graph_key;          // iteration counts the captured graph was built for
  int64_t graph_launches = 0;          // kernels in the captured graph
  std::vector<int32_t> h_perm;         // device index -> node (host copy of the mixed tables' perm)
  // tables built by the device flattener from the forest's device copy (kept alive here)
  bool device_flat = false;
  std::shared_ptr<void> fdev;

  // device_build: the tables are built on the GPU by the device flattener (same FP64 tables; the
  // mixed tables, built on first use, differ only in the numbering of the irregular geometry classes)
  explicit LevelSet(const Forest<D>& forest, bool with_mixed = true, bool device_build = false);
  // level set over the disjoint union of grids with equal tree sizes: tables concatenated in node
  // order (parts[k] occupies nodes part_offsets[k] .. part_offsets[k+1]-1)
  // device_build: each grid's FP64 tables built on the GPU and concatenated there, then the union's
  // mixed tables built on the GPU (same results as the host build)
  LevelSet(const std::vector<const Forest<D>*>& parts, bool device_build = false);
  ~LevelSet();
  void set_stream(cudaStream_t s);

  // phi: device pointer, N doubles, updated in place (reinitialize_within_range_of_phi_0).
  void reinitialize(double* phi, int order_space, int order_pseudotime, double limit_high, double limit_low, int iterations,
                    int precision, const double* mask = nullptr);
  // advect_in_normal_direction(vn[, vn_np1], phi, dt, phi_xx...): device pointers; phi_dd may be null
  // (D*N doubles, overwritten with the derivatives of the intermediate stage as the reference does).
  void advect_normal(const double* vn, const double* vn_np1, double* phi, double dt, double* phi_dd, int precision);
  // compute_derivatives: dd = D*N doubles.
  void second_derivatives(const double* f, double* dd);
  // dt of the CF overload: min over nodes of 0.8*|s_min/vn| (src/my_p4est_level_set.cpp:752-776).
  double cfl_dt(const double* vn);
  // FP64 band check: max |a - b| over the nodes with |b| < band (device pointers, N values each);
  // NaN if a NaN was met; count: nodes in the band.
  double band_linf(const double* a, const double* b, double band, int64_t* count);
  // interface location check: max over the grid edges cut by b of the distance between a's and b's linear
  // zero crossings (device pointers, N values each); edges: edges cut by b, mismatched: of those, edges a
  // does not cut.
  double interface_location_error(const double* a, const double* b, int64_t* edges, int64_t* mismatched);

  // The per-rank FP64 sweeps of a Morton-range split: each covers nodes [first, first + count) only and
  // reads every other node's value from the full-length (device, node-order) arrays the caller keeps
  // current with its halo exchange. prep: status and subcell distances from phi_0 (kept in this object)
  // with the caller's phi_0 limits; stage: out = stage(phin) or 0.5 (avg_with + stage(phin)).
  void fp64_dd_range(const double* f, double* dd, int64_t first, int64_t count);
  // a rank's mixed reinitialisation with ghost updates between its stages (Morton split): the phi_0-only step
  // (limits as reinitialize_within_range_of_phi_0 takes them; mask == 0 leaves a node out of the updates), one RK
  // stage, the FP32 phi_n (0) or phi_1 (1) in device slot order, the slot of every node, and phi back in FP64
  void mixed_split_begin(const double* phi, int os, double limit_high, double limit_low, const double* mask);
  void mixed_step(int os, int stage);
  float* mixed_field(int which) { return which == 0 ? f_phi.p : f_phi1.p; }
  void mixed_slots(int32_t* out_dev);
  void mixed_end(double* phi);
  void fp64_advect_stage_range(const double* phin, const double* ddq, const double* ddm, const double* vn, double dt, double* out,
                               const double* avg_with, int64_t first, int64_t count);
  void fp64_prep_range(const double* phi0, const double* dd0, int os, double limit_high, double limit_low, int64_t first, int64_t count);
  void fp64_stage_range(int os, const double* phi0, const double* phin, const double* dd, double* out, const double* avg_with,
                        int64_t first, int64_t count);

  // reinitialize() in FP64 with no allocation: the work vectors come from a static device array
  // (reinit_fp64_static) that holds grids up to LSG_NOALLOC_SCRATCH_BYTES of scratch.
  void reinitialize_fp64_noalloc(double* phi, int os, int ot, double limit_high, double limit_low, int iterations);

  // first_derivatives_central (src/my_p4est_node_neighbors.cpp:1643-1948): out = D x N gradient of f.
  void first_derivatives(const double* f, double* out);
  // compute_normals (src/my_p4est_utils.cpp:1717-1739): out = D x N unit normals of phi.
  void compute_normals(const double* phi, double* out);
  // compute_mean_curvature(neighbors, normals, kappa) (src/my_p4est_utils.cpp:1658-1696).
  void mean_curvature_from_normals(const double* normals, double* kappa);
  // compute_normals_and_mean_curvature (src/my_p4est_utils.cpp:2776-2802).
  void normals_and_mean_curvature(const double* phi, double* normals, double* kappa);

  // extend_Over_Interface_TVD(phi, q, iterations, order, band_use, band_extend, normal, mask)
  // (src/my_p4est_level_set.cpp:969-1764) without boundary conditions or initial guesses, one-step
  // extrapolation: q (device, N) is extended from the region phi < 0 (or mask < 0) along the normals.
  // normals (D x N) and mask (N) may be null (computed from phi / taken as phi).
  // nonzero_guess, q_n, q_nn (device, N each, nullable, in/out): use_nonzero_guess and the q_n / q_nn
  // arguments of the reference; a given q_n / q_nn starts the marching where nothing is computed and
  // receives the extended normal derivative.
  void extend_over_interface(const double* phi, double* q, int iterations, int order, double band_use, double band_extend,
                             const double* normals, const double* mask, bool nonzero_guess = false, double* q_n = nullptr,
                             double* q_nn = nullptr);

  // extend_from_interface_to_whole_domain_TVD(phi, qi, q, iterations, mask, band_zero, band_smooth, cf = NULL,
  // grad_phi) (src/my_p4est_level_set.cpp:3181-3767) for nf fields (nf x N; the reference's blocksize):
  // q (device, nf x N, not overlapping qi) receives qi's interface values extended along the normals.
  // mask (only with nf == 1) and grad_phi (D x N) may be null; method = interpolation_on_interface.
  // cf (the reference's cf argument, batched): interface values given by the caller for the crossing
  // (node, direction, distance) triples, in node order; with it q starts at zero and qi only supplies the
  // values of the other directions; no mask and one field only, as in the reference.
  using InterfaceValuesFn = int (*)(void* ctx, int64_t count, const int32_t* nodes, const int32_t* dirs, const double* dists,
                                    double* values);
  void extend_from_interface(const double* phi, const double* qi, double* q, int nf, int iterations, const double* mask,
                             double band_zero, double band_smooth, const double* grad_phi, int method, InterfaceValuesFn cf = nullptr,
                             void* cf_ctx = nullptr);

  // my_p4est_interpolation_nodes_t: nf fields (nf x N) interpolated at np points (D doubles each)
  // with `method` (interpolation_method); Fdd (nf x D x N) may be null and is then computed with
  // compute_derivatives. out: nf x np. Device pointers.
  void interpolate(const double* xyz, int64_t np, int nf, const double* F, const double* Fdd, int method, double* out);
  // leaf index chosen for each point by the point location (clipped into the domain first)
  void locate(const double* xyz, int64_t np, int32_t* leaf);
  // my_p4est_semi_lagrangian_t::advect_from_n_to_np1(dt, v, vxx, phi_n, phi_xx_n, phi_np1): this
  // object's grid is time n; xyz are the np nodes of the grid at n+1. v: D x N, vdd: D x D x N
  // (component, axis, node) or null; phi_dd: D x N or null. Device pointers.
  void sl_advect(const double* xyz, int64_t np, double dt, const double* v, const double* vdd, const double* phi, const double* phi_dd,
                 int velo_method, int phi_method, double* phi_np1);
  // advect_from_n_to_np1(dt_nm1, dt_n, vnm1, vxx_nm1, vn, vxx_n, phi_n, phi_xx_n, phi_np1), the two-velocity
  // second-order step: this object's grid is time n (vn: D x N, phi_n), nm1 the grid at n-1 (vnm1:
  // D x N_nm1); xyz the np nodes of the grid at n+1. vn_dd / vnm1_dd: D x D x N of their grids (component,
  // axis, node) or null; phi_dd: D x N or null. Device pointers, both level sets on the current device.
  void sl_advect2(LevelSet<D>& nm1, const double* xyz, int64_t np, double dt_nm1, double dt_n, const double* vnm1,
                  const double* vnm1_dd, const double* vn, const double* vn_dd, const double* phi, const double* phi_dd, int velo_method,
                  int phi_method, double* phi_np1);
  void sl_advect2_host(LevelSet<D>& nm1, const double* xyz, int64_t np, double dt_nm1, double dt_n, const double* vnm1,
                       const double* vnm1_dd, const double* vn, const double* vn_dd, const double* phi, const double* phi_dd,
                       int velo_method, int phi_method, double* phi_np1);
  // the CF overload with the single-vortex velocity scaled by vscale
  void sl_advect_vortex(const double* xyz, int64_t np, double dt, double vscale, const double* phi, const double* phi_dd, int phi_method,
                        double* phi_np1);

  // Batched reinitialize_2nd_order (mixed precision) of every grid of a union with its own iteration
  // count: phi on the device in union node order. With use_graph the iteration loop runs as one CUDA
  // graph (captured on the first call with these iteration counts, replayed afterwards).
  void reinitialize_batch(double* phi, const int* iterations, bool use_graph);
  // Times candidate launch shapes of the mixed stage on phi (device, node order) and keeps the fastest;
  // a candidate whose bounded waits gave up is discarded.
  void autotune(const double* phi, int trials);
  // bound of the bulk-copy stage kernel's waits in SM clock cycles (0: the default, about a second)
  void set_wait_limit(long long cycles) { cfg.wait_cycles = cycles > 0 ? cycles : 0; }
  void drop_graph();  // forget a captured graph (after a launch-shape change)

  // host-buffer conveniences (copies inside)
  void reinitialize_host(double* phi, int os, int ot, double hi, double lo, int iters, int precision, const double* mask = nullptr);
  void interpolate_host(const double* xyz, int64_t np, int nf, const double* F, const double* Fdd, int method, double* out);
  void sl_advect_host(const double* xyz, int64_t np, double dt, const double* v, const double* vdd, const double* phi,
                      const double* phi_dd, int velo_method, int phi_method, double* phi_np1);
  void sl_advect_vortex_host(const double* xyz, int64_t np, double dt, double vscale, const double* phi, const double* phi_dd,
                             int phi_method, double* phi_np1);

 private:
  void init_tables(const Tables64<D>& T, const double* tree_size, bool with_mixed);
  void mixed_loop(int os, int iters, const std::vector<int>& freeze_at);
  void ensure_side_stream();
  void prep_batch(const double* phi);
  void build_mixed();
  void upload_mixed(const Tables32<D>& M, const double* tree_size);
  void set_mixed_views(int64_t nR_, int64_t nI_, int64_t nU_, int base, int64_t x_first, int64_t nX, int64_t ncls_, const double* ts);
  void init_stream();
  void reinit_fp64(double* phi, int os, int ot, double lim_hi, double lim_lo, int iters, const double* mask = nullptr);
  void reinit_mixed(double* phi, int os, int ot, double lim_hi, double lim_lo, int iters, const double* mask = nullptr);
  void mixed_begin(const double* phi, int os, double lim_hi, double lim_lo, const double* mask);
  void advect_mixed(const double* vn, const double* vn_np1, double* phi, double dt, double* phi_dd);
  // one RK stage on the mixed tables: the reinitialisation, or with adv_vn the normal advection
  void mixed_stage(int os, const float* phin, float* out, const float* avg_with, const float* adv_vn = nullptr, float adv_dt = 0.0f);
  void mixed_join();
  // the two chains of the last mixed stage are still open (not yet joined into the caller's stream)
  bool chains_open = false;
  bool join_each_stage = false;  // set while a graph is captured
  cudaStream_t chain_a = nullptr, chain_b = nullptr;
  // throws DeviceTimeout if a bounded device-side wait gave up since the last check (synchronises the
  // stream; skipped while the stream is being captured)
  void check_device_waits();
  // reads and clears the flag a bounded device-side wait sets when it gives up (synchronises the stream)
  bool take_device_wait_flag();
  void build_locator();
  void build_gradient();
  const double* derivatives_of(int nf, const double* F, const double* Fdd, DevBuf<double>& store);
};

double largest_dbl_smaller_than_dbl_max();

}  // namespace lsg
