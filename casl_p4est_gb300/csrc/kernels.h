// Device table views and kernel launchers shared by the host drivers.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "lsg_common.h"

namespace lsg {

// Status word written once per reinitialisation call by the preparation kernel.
enum : uint16_t {
  ST_ANCHORED = 1,   // |phi_0| < zero_distance_threshold -> 0
  ST_OUTSIDE = 2,    // phi_0 outside (limit_low, limit_high) -> phi_0
  ST_NEAR = 4,       // a neighbour of phi_0 has the opposite sign: subcell distances in s_near
  ST_POSITIVE = 8,   // phi_0 > 0
  ST_FROZEN = 16,    // batched runs: the node's field finished its iterations -> phi_n (set by launch_freeze32)
  ST_CUT_SHIFT = 8,  // bit (8 + dir): the neighbour in direction dir is across the interface
};

// SM count of the device current at the first call (grids of persistent and grid-stride kernels)
inline int device_sm_count() {
  static int sms = 0;
  if (sms <= 0) {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    sms = n > 0 ? n : 1;
  }
  return sms;
}

// Launch shape of the mixed stage kernels (chosen by the autotuner): grid of the persistent uniform
// and regular kernels (0: one full wave at maximum occupancy), threads per block of every stage
// kernel, and the pipeline depth of the uniform kernel.
struct StageCfg {
  int uniform_blocks = 0;
  int regular_blocks = 0;
  int tpb = 256;
  // pipeline of the uniform kernel: 1 or 2 nodes whose gathers are in flight per thread, or 3 (4): the
  // node words and a window of phi bulk-copied into shared memory two (three) tiles ahead
  // (cp.async.bulk + mbarrier), or 5: as 1 with the registers capped at 40 so that more of its warps stay
  // resident beside the side stream's kernels (the default: 5-6% faster stages than 1 on the 13.7M-node grid)
  int depth = 5;
  // nodes on either side of a tile in the phi window of the bulk-copy kernel (a multiple of 4)
  int halo = 512;
  // 2: the second derivatives and the irregular nodes on a side stream while the main stream runs the
  // uniform nodes; 1: the four stage kernels one after another on the object's stream (on grids far larger
  // than L2 the concurrent kernels evict each other's gathered lines)
  int streams = 2;
  // with two streams, how the kernels pair up and which chain the block scheduler prefers. Chain A runs the
  // second derivatives, chain B the uniform nodes; then A runs the irregular and B the other regular nodes
  // (0 both at the default priority, 1 A at the highest, 2 B at the highest), or A the other regular and B
  // the irregular nodes (3 A at the highest, 4 B at the highest). With 2 the persistent uniform kernel's
  // blocks are resident from the start and the short blocks of chain A fill the rest; with equal priorities
  // A's many blocks can take the SMs first and the stage ran 15% slower on most calls (13.7M and 122M-node
  // grids)
  int priority = 2;
  // bound of the bulk kernel's waits for its copies, in SM clock cycles (0: about a second); a wait that
  // runs out makes the call report LSG_ETIMEOUT
  long long wait_cycles = 0;
};

template <int D>
struct DTab64 {
  int64_t N;
  const int32_t* nbr;   // NS x N
  const double* w;      // NS x N
  const double* nrm;    // 2D x N
  const double* d;      // 2D x N
  const double* q;      // 2D(D-1) x N
  const int32_t* cidx;  // N
  const double* crec;   // 6 x R
  const uint8_t* wall;  // N
  // per node (tables in stencil-pattern order only, else null): bits 2dir..2dir+1 face-node count - 1, bit 12 a
  // correction record, bits 13.. the wall bits, bit 20 + dir a single face node whose weight equals the norm and
  // is a power of two in [2^-400, 2^400], bit 26 + dir no tangential correction (both factors zero)
  const uint32_t* word = nullptr;
};

// First-derivative correction records (build_gradient_tables): record index per node (-1: none),
// D*(D-1) weights per record, and the mask of the weights that apply.
struct DGrad {
  const int32_t* gidx;
  const double* grec;
  const uint8_t* gmask;
};

// Point location and corner gathers for node interpolation (my_p4est_hierarchy_t +
// p4est_nodes_t::local_nodes). Leaves in tree-major Morton order; ctab[t*ncoarse + c] is the
// leaf containing the first logical point of coarse cell c (level L0) of tree t, so the leaf that
// contains a point lies in [ctab[i], ctab[i+1]] and is found by a short binary search on the keys.
template <int D>
struct DLoc {
  int64_t nleaves;
  int64_t N;                  // nodes (stride of the field arrays)
  const uint64_t* key;        // (tree << D*MAXLEVEL) | morton(leaf corner)
  const int8_t* level;
  const int32_t* local_nodes; // CHILDREN per leaf
  const int32_t* ctab;        // ntrees * ncoarse + 1
  int L0;
  int64_t ncoarse;
  int n[3];                   // brick size in trees
  const int32_t* ijk_to_tree;
  const double* tmin;         // 3 per tree: tree vertex 0
  const double* tmax;         // 3 per tree: last tree vertex
  double xyz_min[3], xyz_max[3], tree_dim[3];
};

// Mixed-precision tables in device node order (layout described in tables32.cpp).
template <int D>
struct DTab32 {
  int64_t N, nR, nI;
  int base;              // base level of the regular nodes' level codes
  float tsize[3];        // tree size per axis
  float inv_tsize[3];
  int64_t nU;            // regular nodes [0, nU) have uniform stencils
  // the regular nodes' face and second-neighbour indices node by node (D int4 per node: the 2D face indices,
  // then the 2D second neighbours), so the uniform and regular stage kernels load them with D vector loads
  const int4* u_pack;
  const uint32_t* r_meta;
  const int32_t* r_nbr;  // 2D x nR
  const int32_t* r_nbr2; // 2D x nR, -1 when absent
  const uint32_t* r_meta2;
  const uint32_t* i_meta;
  const int32_t* i_nbr;  // NS x nI
  const float* i_wf;     // NS x nI
  const float* i_d;      // 2D x nI
  const float* i_q;      // 2D(D-1) x nI
  const int32_t* i_cidx;
  const float* corr;     // D*D x R
  const uint32_t* i_cls; // nI: geometry class of each irregular node
  const float* cls32;    // class records (cls_words<D>() floats each)
  int64_t x_first, nX;   // regular nodes of the extended second-derivative set: [x_first, x_first + nX)
  // FP64 coefficients of the irregular nodes (subcell step)
  double tsize64[3];
  const double* i_wf64;
  const double* i_d64;
  const double* i_q64;
  const double* corr64;
};

// FP64 sweeps over the nodes [first, first + count) (count < 0: to the last node), by default all of them.
template <int D>
void launch_dd64(const DTab64<D>& T, const double* f, double* dd, cudaStream_t s, int64_t first = 0, int64_t count = -1);
// The FP64 tables in stencil-pattern order (face-node counts, correction, walls; node order within a pattern):
// perm (sorted index -> node), iperm and the permuted arrays (neighbour indices renumbered). keys, keys_out
// and idx hold N entries each; temp holds sort64_temp_bytes(N) bytes.
struct Tab64Out {
  int32_t* nbr;
  double *w, *nrm, *d, *q;
  int32_t* cidx;
  uint8_t* wall;
};
size_t sort64_temp_bytes(int64_t n);
// fills DTab64::word for tables in stencil-pattern order
template <int D>
void launch_node_word64(const DTab64<D>& T, uint32_t* word, cudaStream_t s);
template <int D>
cudaError_t launch_sort_tab64(const DTab64<D>& T, uint32_t* keys, uint32_t* keys_out, int32_t* idx, void* temp, size_t temp_bytes,
                              int32_t* perm, int32_t* iperm, const Tab64Out& out, cudaStream_t s);
void launch_gather_perm64(const double* src, const int32_t* perm, double* dst, int64_t n, cudaStream_t s);   // dst[i] = src[perm[i]]
void launch_scatter_perm64(const double* src, const int32_t* perm, double* dst, int64_t n, cudaStream_t s);  // dst[perm[i]] = src[i]
template <int D>
void launch_reinit_prep64(const DTab64<D>& T, const double* phi0, const double* dd0, double zdt, double lim_lo, double lim_hi,
                          int order_space, uint16_t* status, double* s_near, cudaStream_t s, int64_t first = 0, int64_t count = -1);
// out = stage(phin); if avg_with != nullptr: out = 0.5*(avg_with + stage(phin)) (may alias avg_with).
template <int D>
void launch_reinit_stage64(const DTab64<D>& T, int order_space, const uint16_t* status, const double* s_near, const double* phi0,
                           const double* phin, const double* dd, double* out, const double* avg_with, cudaStream_t s,
                           int64_t first = 0, int64_t count = -1);
// over the nodes [first, first + count) (count < 0: to the last node), by default all of them
template <int D>
void launch_advect_stage64(const DTab64<D>& T, const double* phin, const double* ddq, const double* ddm, const double* vn, double dt,
                           double* out, const double* avg_with, cudaStream_t s, int64_t first = 0, int64_t count = -1);
void launch_copy64(const double* src, double* dst, int64_t n, cudaStream_t s);
void launch_min_cfl(const double* smin, const double* vn, int64_t n, double* dt_out_dev, cudaStream_t s);
// First derivatives (FP64, the reference's expression order). fdd: second derivatives of f (D x N,
// from launch_dd64), read only at nodes with a correction record. which: bit a -> component a.
template <int D>
void launch_grad64(const DTab64<D>& T, const DGrad& G, const double* f, const double* fdd, double* out, int which, cudaStream_t s);
// n / |n| per node, 0 where |n| < EPS (compute_normals), in place on D x N
template <int D>
void launch_normalize64(double* g, int64_t N, cudaStream_t s);
// kappa = sum_a d_a(n_a) (compute_mean_curvature from normals); ndd: D x D x N second derivatives
// of the components
template <int D>
void launch_div64(const DTab64<D>& T, const DGrad& G, const double* nrm, const double* ndd, double* kappa, cudaStream_t s);
// get_curvature from the gradient g (D x N), the second derivatives of phi (D x N) and of the
// gradient components x and y (D x N each)
template <int D>
void launch_kappa64(const DTab64<D>& T, const DGrad& G, const double* g, const double* phidd, const double* gxdd, const double* gydd,
                    double* kappa, cudaStream_t s);
// extend_Over_Interface_TVD (FP64). ext_init1: normal derivative qn, gradient qx (D x N) and the
// well-defined flag bqn (-1/+1) of every node; ext_init2: second normal derivative qnn and bqnn, from
// the second derivatives of the normals (nrmdd, D x D x N) and of qx (qxdd, D x D x N) and the
// edge-diagonal neighbours cnb; ext_march: one upwind marching step of v into tmp on the nodes with
// b > 0 and phi < band_extend (minus src when given); ext_q: one marching step of q with the order-2
// minmod correction from qdd.
// guess for q_n / q_nn where no value can be computed (bits): GRADIENT, the normal derivative of q / q_n
// (use_nonzero_guess); else KEEP, the value already in the array (the caller's q_n / q_nn); else zero.
// Where the reference leaves q_nn as it was, KEEP keeps it and no KEEP writes zero.
enum { EXT_GUESS_ZERO = 0, EXT_GUESS_KEEP = 1, EXT_GUESS_GRADIENT = 2 };
template <int D>
void launch_ext_init1(const DTab64<D>& T, const DGrad& G, const double* phi, const double* mask, const double* q, const double* qdd,
                      const double* nrm, double band_use, int guess, double* qx, double* qn, int8_t* bqn, cudaStream_t s);
// EXT_GUESS_GRADIENT needs qn and its second derivatives qndd
template <int D>
void launch_ext_init2(const DTab64<D>& T, const DGrad& G, const double* phi, const double* mask, const double* q, const double* qdd,
                      const double* nrm, const double* nrmdd, const double* qx, const double* qxdd, const int8_t* bqn, const int32_t* cnb,
                      double band_use, int guess, const double* qn, const double* qndd, double* qnn, int8_t* bqnn, cudaStream_t s);
template <int D>
void launch_ext_march(const DTab64<D>& T, const double* v, double* tmp, const int8_t* b, const double* phi, const double* nrm,
                      const double* src, double band_extend, cudaStream_t s);
template <int D>
void launch_ext_q(const DTab64<D>& T, const double* q, double* tmp, const double* qdd, const double* phi, const double* mask,
                  const double* nrm, const double* qn, int order, double band_extend, cudaStream_t s);
// FP64 band L-infinity: out3 = {bits of max |a-b| over |b| < band, band node count, NaN flag}
// nodes whose mask is 0 (mask in node order; perm maps status indices to nodes, or null) become ST_OUTSIDE
void launch_apply_mask(const double* mask, const int32_t* perm, uint16_t* status, int64_t n, cudaStream_t s);
void launch_band_linf64(const double* a, const double* b, double band, int64_t n, unsigned long long* out3, cudaStream_t s);
// FP64 interface location along cut grid edges: out3 = {bits of max |t_a - t_b|, cut edges of b, edges where a
// does not change sign}, t the linear zero crossing's distance from the edge's first node
template <int D>
void launch_iface_err64(const DTab64<D>& T, const double* a, const double* b, unsigned long long* out3, cudaStream_t s);
// Node interpolation (kernels_interp.cu, FP64). Points: D doubles each. When shift is given, point p
// is first moved to xyz[p] - coef*shift[:, p] and clipped into the domain (the semi-Lagrangian
// backtrace). F: nf x N values, Fdd: nf x D x N second derivatives (ignored for linear), out: nf x np.
template <int D>
void launch_interp64(const DLoc<D>& L, int method, const double* xyz, int64_t np, const double* shift, double coef, int nf,
                     const double* F, const double* Fdd, double* out, cudaStream_t s);
// Semi-Lagrangian step with the analytic single-vortex velocity scaled by vscale: RK2 backtrace from
// xyz, then interpolation of phi at the departure point.
template <int D>
void launch_sl_vortex64(const DLoc<D>& L, int method, const double* xyz, int64_t np, double dt, double vscale, const double* phi,
                        const double* phi_dd, double* out, cudaStream_t s);
// Last round of the two-velocity semi-Lagrangian step: x_d = xyz - dt_n (ca vn_star - cb vnm1_star)
// (D x np each), clipped, and phi interpolated there.
template <int D>
void launch_sl2_phi64(const DLoc<D>& L, int method, const double* xyz, int64_t np, const double* vn_star, const double* vnm1_star,
                      double ca, double cb, double dt_n, const double* phi, const double* phi_dd, double* out, cudaStream_t s);
// Leaf chosen by the point location for each point (clipped first).
template <int D>
void launch_locate64(const DLoc<D>& L, const double* xyz, int64_t np, int32_t* leaf, cudaStream_t s);
// extend_from_interface_to_whole_domain_TVD: set-up (start value of q, interface values and distances
// per direction, crossing bits) and one TVD-RK2 stage (average = second stage fused with the RK average)
template <int D>
void launch_efi_init64(const DTab64<D>& T, const DLoc<D>& L, int method, const double* xyz, const double* phi, const double* pdd,
                       const double* qi, const double* qidd, const double* mask, double dl, double band_zero_dl, double band_smooth_dl,
                       double* q, double* qi_nb, double* s_nb, uint8_t* cross, cudaStream_t s);
// dst[i] = src[idx[i]] / dst[idx[i]] = src[i] for i < m
void launch_gather_idx64(const double* src, const int64_t* idx, int64_t m, double* dst, cudaStream_t s);
void launch_scatter_idx64(const double* src, const int64_t* idx, int64_t m, double* dst, cudaStream_t s);
template <int D>
void launch_efi_stage64(const DTab64<D>& T, const double* phi, const double* grad, const double* q, const double* qdd, const double* qdd2,
                        const double* qi_nb, const double* s_nb, const uint8_t* cross, double zdt, bool average, double* out,
                        cudaStream_t s);

// reinit_fp64's kernel sequence with its work vectors in a static device array (noalloc.cu);
// throws std::invalid_argument when the grid does not fit the array. hi/lo: widened phi_0 limits.
template <int D>
void reinit_fp64_static(const DTab64<D>& T, double zdt, double* phi, int order_space, int order_pseudotime, double lim_hi,
                        double lim_lo, int iterations, cudaStream_t s);

// Mixed precision.
template <int D>
void launch_dd32(const DTab32<D>& T, const float* f, float* dd, cudaStream_t s);
// FP64 subcell step of the mixed path, in device node order: phi0_dev and dd0_irr are work arrays
// (N and D*nI doubles), status/s_near are written in device order.
template <int D>
void launch_reinit_prep_mixed(const DTab32<D>& T, const int32_t* perm, const double* phi0, double zdt, double lim_lo, double lim_hi,
                              int order_space, double* phi0_dev, double* dd0_irr, uint16_t* status, float* s_near, int32_t* near_list,
                              unsigned* near_count, cudaStream_t s);
// fused stage: second derivatives of face nodes rebuilt from recorded second neighbours, or read from
// ddx (D x N, written by launch_dd_x32 for the same phi on the extended set)
template <int D>
void launch_dd_x32(const DTab32<D>& T, const float* f, float* ddx, cudaStream_t s, int tpb = 256);
// Batched runs: nodes whose field stops at iteration `it` (lim[i] <= it, device order) are frozen.
void launch_freeze32(const uint16_t* lim, int it, uint16_t* status, int64_t n, cudaStream_t s);
// One RK stage of the mixed reinitialisation is split in three parts that write disjoint node ranges:
// uniform regular nodes (no dependence on ddx), other regular nodes and irregular nodes (both read ddx).
enum { STAGE_PART_UNIFORM = 0, STAGE_PART_REGULAR = 1, STAGE_PART_IRREGULAR = 2 };
// err: device word that a bounded wait of the bulk-copy uniform kernel (cfg.depth 3) sets when it
// gives up (the kernel then stops; the host reads the word after the call). With adv_vn the same kernels
// run a stage of advect_in_normal_direction instead (normal velocity adv_vn, device order; time step
// adv_dt; every node updated, upwinding by the sign of vn; status and s_near unused).
template <int D>
void launch_reinit_part32(const DTab32<D>& T, int part, int order_space, const uint16_t* status, const float* s_near,
                          const float* phin, const float* ddx, float* out, const float* avg_with, cudaStream_t s, const StageCfg& cfg,
                          int* err, const float* adv_vn = nullptr, float adv_dt = 0.0f);
template <int D>
void launch_advect_stage32(const DTab32<D>& T, const float* phin, const float* ddq, const float* ddm, const float* vn, float dt,
                           float* out, const float* avg_with, cudaStream_t s);
// node order (FP64) <-> device order (FP32): dst[b*dst_stride + i] = src[b*src_stride + perm[i]] and the
// reverse scatter (skipping nodes whose status marks them outside the reinitialisation limits)
// fills T.u_pack's layout (D int4 per regular node) from the r_nbr / r_nbr2 planes
template <int D>
void launch_pack_uniform32(const DTab32<D>& T, int4* out, cudaStream_t s);
void launch_gather_f32(const double* src, const int32_t* perm, float* dst, int64_t n, int64_t src_stride, int64_t dst_stride,
                       int blocks, cudaStream_t s);
void launch_scatter_f64(const float* src, const int32_t* perm, const uint16_t* status, double* dst, int64_t n, int64_t src_stride,
                        int64_t dst_stride, int blocks, cudaStream_t s,
                        const uint16_t* lim = nullptr);

}  // namespace lsg
