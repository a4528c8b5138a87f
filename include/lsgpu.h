/*
 * lsgpu: C ABI of the GB300 level-set path (reinitialisation, normal-direction advection and
 * semi-Lagrangian node interpolation on quadtrees/octrees).
 *
 * Every entry point returns an int status (LSG_OK = 0) and never aborts or throws; the message of
 * the last failure on the calling thread is available from lsg_last_error(). Arrays are plain
 * pointers in node order (the order of lsg_forest_nodes), doubles unless stated otherwise.
 * "_device" entry points take device pointers and run on the level-set object's stream; the other
 * ones take host pointers and copy inside the call.
 *
 * Each declaration names the parCASL interface it replaces (paths inside the parCASL tree).
 */
#ifndef LSGPU_H
#define LSGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  LSG_OK = 0,
  LSG_EINVAL = 1,   /* bad argument (the reference throws std::invalid_argument) */
  LSG_ENOMEM = 2,   /* host or device allocation failed */
  LSG_EDEVICE = 3,  /* CUDA error */
  LSG_ETIMEOUT = 4, /* a bounded device-side wait gave up */
  LSG_ENAN = 5,     /* non-finite input where a finite one is required */
  LSG_ESTATE = 6    /* object not in the required state (e.g. nodes not built) */
};

enum { LSG_FP64 = 0, LSG_MIXED = 1 };

/* interpolation_method, src/my_p4est_utils.h:332-338 */
enum {
  LSG_LINEAR = 0,
  LSG_QUADRATIC = 1,
  LSG_QUADRATIC_NON_OSCILLATORY = 2,
  LSG_QUADRATIC_NON_OSCILLATORY_CONTINUOUS_V1 = 3,
  LSG_QUADRATIC_NON_OSCILLATORY_CONTINUOUS_V2 = 4
};

typedef struct lsg_forest lsg_forest;       /* p4est_t + p4est_nodes_t + my_p4est_hierarchy_t + my_p4est_node_neighbors_t */
typedef struct lsg_level_set lsg_level_set; /* my_p4est_level_set_t */

const char* lsg_last_error(void);
int lsg_version(void);

/* ---- grid (host) ------------------------------------------------------------------------------ */

/* my_p4est_brick_new + my_p4est_new with one level-0 quadrant per tree
 * (src/my_p4est_tools.c:37-170). dim is 2 or 3; periodic may be NULL. */
int lsg_forest_create(int dim, const int n_xyz[3], const double xyz_min[3], const double xyz_max[3], const int periodic[3],
                      lsg_forest** out);
int lsg_forest_destroy(lsg_forest* f);
int lsg_forest_dim(const lsg_forest* f);
int64_t lsg_forest_num_leaves(const lsg_forest* f);
/* leaves in tree-major Morton order: tree, level, logical corner (3 ints per leaf, z = 0 in 2D) */
int lsg_forest_leaves(const lsg_forest* f, int32_t* tree, int32_t* level, int32_t* xyz);
/* one pass of my_p4est_refine / my_p4est_coarsen with per-leaf tags (nonzero = refine/coarsen) */
int lsg_forest_refine(lsg_forest* f, const uint8_t* tags, int64_t n);
int lsg_forest_coarsen(lsg_forest* f, const uint8_t* tags, int64_t n);
/* refine_levelset_cf (src/my_p4est_refine_coarsen.cpp:18-90) evaluated on every leaf for an
 * analytic shape (kind and parameters as in shapes.h); tags has one byte per leaf. */
int lsg_forest_tag_levelset(const lsg_forest* f, int min_lvl, int max_lvl, double lip, double band, int shape,
                            const double* params, int nparams, uint8_t* tags);
/* `passes` rounds of tag + refine, as the examples' loop of my_p4est_refine(refine_levelset_cf) */
int lsg_forest_refine_levelset(lsg_forest* f, int min_lvl, int max_lvl, double lip, double band, int shape,
                               const double* params, int nparams, int passes);
/* my_p4est_nodes_new (src/my_p4est_nodes.c:292-1000): every leaf corner is a node */
int lsg_forest_build_nodes(lsg_forest* f);
int64_t lsg_forest_num_nodes(const lsg_forest* f);
/* node_xyz_fr_n (src/my_p4est_utils.h:1398-1405): dim doubles per node */
int lsg_forest_node_xyz(const lsg_forest* f, double* xyz);
/* owner tree and clamped logical coordinates (3 ints per node) of p4est_indep_t */
int lsg_forest_nodes(const lsg_forest* f, int32_t* tree, int32_t* xyz);
/* p4est_nodes_t::local_nodes: 2^dim node indices per leaf */
int lsg_forest_local_nodes(const lsg_forest* f, int32_t* out);
/* sample_cf_on_nodes for an analytic shape */
int lsg_forest_sample_shape(const lsg_forest* f, int shape, const double* params, int nparams, double* out);
/* quad_neighbor_nodes_of_node_t records of nodes [first, first+count) as built by
 * my_p4est_node_neighbors_t::construct_neighbors (src/my_p4est_node_neighbors.cpp:114-1201).
 * Each record: node_000 (int32), nb[2*dim][2^(dim-1)] (int32), d[2*dim], dt[2*dim][2*(dim-1)],
 * inverse_d_max (doubles), laid out with natural C alignment; record_bytes must equal
 * lsg_qnnn_record_bytes(dim). */
size_t lsg_qnnn_record_bytes(int dim);
int lsg_forest_export_qnnn(const lsg_forest* f, int64_t first, int64_t count, void* out, size_t record_bytes);
/* is_node_{x,y,z}{m,p}Wall (src/my_p4est_utils.cpp:1815-1905): bit 2*axis+side per node */
int lsg_forest_wall_mask(const lsg_forest* f, uint8_t* out);
/* smallest cell size per axis at the finest level present (dxyz_min, src/my_p4est_utils.cpp:1136) */
int lsg_forest_dxyz_min(const lsg_forest* f, double* dxyz);

/* ---- level set (device) ----------------------------------------------------------------------- */

/* my_p4est_level_set_t(my_p4est_node_neighbors_t*) (src/my_p4est_level_set.h:385-392): builds the
 * device tables of the grid. The forest must outlive the object and keep its nodes. */
int lsg_level_set_create(const lsg_forest* f, lsg_level_set** out);
int lsg_level_set_destroy(lsg_level_set* ls);
/* run on the caller's cudaStream_t (NULL keeps the object's own stream) */
int lsg_level_set_set_stream(lsg_level_set* ls, void* cuda_stream);
void* lsg_level_set_stream(const lsg_level_set* ls);
int64_t lsg_level_set_num_nodes(const lsg_level_set* ls);
double lsg_level_set_zero_distance_threshold(const lsg_level_set* ls);

/* reinitialize_within_range_of_phi_0 (src/my_p4est_level_set.cpp:290-557); the public forms
 * reinitialize_{1st,2nd}_order[_above_threshold|_time_*] (src/my_p4est_level_set.h:434-613) are
 * (order_space, order_pseudotime, limit_high, limit_low) choices of this one. */
int lsg_reinitialize(lsg_level_set* ls, double* phi, int order_space, int order_pseudotime, double limit_high,
                     double limit_low, int iterations, int precision);
int lsg_reinitialize_device(lsg_level_set* ls, double* phi_dev, int order_space, int order_pseudotime, double limit_high,
                            double limit_low, int iterations, int precision);
/* No counterpart in the reference. lsg_reinitialize_device with precision LSG_FP64, allocating no
 * memory: the work vectors (114 bytes per node in 3D, 82 in 2D, each array padded to 256 bytes)
 * come from one static device array of LSG_NOALLOC_SCRATCH_BYTES per device; larger grids return
 * LSG_EINVAL. It serves callers that cannot allocate inside the call: a solver whose device memory
 * is handed out by another pool (cudaMalloc there fails or fragments it), a time loop that cannot
 * take the device-wide synchronisation of cudaFree, and programs with many level-set objects on
 * small grids, which would otherwise each keep their own work vectors.
 * The first call on a device (with that device current) takes the array's address with
 * cudaGetSymbolAddress; make it before any stream capture. Nothing in the array must start at
 * zero. Calls that overlap on one device race on the array: serialise them. */
#define LSG_NOALLOC_SCRATCH_BYTES (32u << 20)
int lsg_reinitialize_device_noalloc(lsg_level_set* ls, double* phi_dev, int order_space, int order_pseudotime,
                                    double limit_high, double limit_low, int iterations);
/* reinitialize_2nd_order(phi, iterations, limit) (src/my_p4est_level_set.h:468-472) */
int lsg_reinit_2nd(lsg_level_set* ls, double* phi, int iterations, double limit, int precision);

/* advect_in_normal_direction(const Vec vn[, const Vec vn_np1], Vec phi, dt, phi_xx...)
 * (src/my_p4est_level_set.cpp:656-725, 785-815). vn_np1 and phi_dd may be NULL; phi_dd holds
 * dim*N doubles (xx block, then yy, then zz) and is overwritten as in the reference. */
int lsg_advect_in_normal_direction(lsg_level_set* ls, const double* vn, const double* vn_np1, double* phi, double dt,
                                   double* phi_dd, int precision);
int lsg_advect_in_normal_direction_device(lsg_level_set* ls, const double* vn_dev, const double* vn_np1_dev, double* phi_dev,
                                          double dt, double* phi_dd_dev, int precision);
/* CFL time step of the CF overload: min over nodes of 0.8*|s_min/vn| (src/my_p4est_level_set.cpp:745-783) */
int lsg_advect_cfl_dt(lsg_level_set* ls, const double* vn, double* dt_out);
/* compute_derivatives -> second_derivatives_central (src/my_p4est_node_neighbors.cpp:1422-1640) */
int lsg_second_derivatives(lsg_level_set* ls, const double* f, double* f_dd);
int lsg_second_derivatives_device(lsg_level_set* ls, const double* f_dev, double* f_dd_dev);
/* perturb_level_set_function (src/my_p4est_level_set.cpp:728-743) */
int lsg_perturb_level_set_function(lsg_level_set* ls, double* phi, double epsilon);

/* ---- instrumentation (no reference counterpart; replaces PETSc log events) --------------------- */
/* kernel classes reported by lsg_level_set_kernel_times */
enum {
  LSG_K_DD64 = 0, LSG_K_PREP64, LSG_K_STAGE64, LSG_K_ADVECT64, LSG_K_DD32, LSG_K_PREP_MIXED, LSG_K_STAGE32, LSG_K_ADVECT32,
  LSG_K_CONVERT, LSG_K_COPY, LSG_K_NUM
};
/* record CUDA events around every launch (adds a little overhead) */
int lsg_level_set_enable_kernel_timing(lsg_level_set* ls, int on);
/* per class: total milliseconds and number of launches since the last reset (synchronises) */
int lsg_level_set_kernel_times(lsg_level_set* ls, double* ms, int64_t* counts, int nkinds, int reset);
/* number of kernel launches this object issued since the last kernel-times reset */
int64_t lsg_level_set_launch_count(const lsg_level_set* ls);

#ifdef __cplusplus
}
#endif

#endif /* LSGPU_H */
