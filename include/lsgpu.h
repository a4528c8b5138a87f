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
/* p4est_copy: an independent copy of the forest (leaves and, if built, nodes) */
int lsg_forest_copy(const lsg_forest* f, lsg_forest** out);
/* Replace the leaves by a caller-supplied complete forest in tree-major Morton order (e.g. the
 * quadrants of a p4est_t, tree by tree: tree index, level, logical x y z); LSG_EINVAL unless the
 * leaves cover every tree exactly once. Nodes must be rebuilt afterwards. */
int lsg_forest_set_leaves(lsg_forest* f, int64_t n, const int32_t* tree, const int32_t* level, const int32_t* xyz);
/* splitting_criteria_tag_t::refine_and_coarsen(p4est, nodes, phi) with tag_quadrant
 * (src/my_p4est_refine_coarsen.cpp:422-479, 1170-1205): phi holds one value per node (nodes built);
 * one coarsening pass then one refinement pass; *changed = 1 if any leaf was created. The nodes
 * must be rebuilt afterwards. */
int lsg_forest_refine_and_coarsen(lsg_forest* f, int min_lvl, int max_lvl, double lip, double band, const double* phi,
                                  int* changed);
/* refine_levelset_cf (src/my_p4est_refine_coarsen.cpp:18-90) evaluated on every leaf for an
 * analytic shape (kind and parameters as in shapes.h); tags has one byte per leaf. */
int lsg_forest_tag_levelset(const lsg_forest* f, int min_lvl, int max_lvl, double lip, double band, int shape,
                            const double* params, int nparams, uint8_t* tags);
/* `passes` rounds of tag + refine, as the examples' loop of my_p4est_refine(refine_levelset_cf) */
int lsg_forest_refine_levelset(lsg_forest* f, int min_lvl, int max_lvl, double lip, double band, int shape,
                               const double* params, int nparams, int passes);
/* my_p4est_nodes_new (src/my_p4est_nodes.c:292-1000): every leaf corner is a node */
int lsg_forest_build_nodes(lsg_forest* f);
/* The same node numbering computed on the GPU (corner keys canonicalised, sorted and made unique on
 * the device), copied back into the forest; the device copy of the leaves and nodes stays with the
 * forest for the two calls below and for LSG_BUILD_ON_DEVICE level sets. stream: a cudaStream_t or
 * NULL. No reference counterpart (my_p4est_nodes_new runs on the host). */
int lsg_forest_build_nodes_device(lsg_forest* f, void* stream);
/* node_x_fr_n / node_y_fr_n / node_z_fr_n of every node (src/my_p4est_utils.h:1346-1405) into device
 * memory, N x dim. */
int lsg_forest_node_xyz_device(lsg_forest* f, double* xyz_dev, void* stream);
/* lsg_forest_refine_and_coarsen with phi in device memory: the tags
 * (splitting_criteria_tag_t::tag_quadrant, src/my_p4est_refine_coarsen.cpp:422-479) are evaluated on
 * the GPU and only one byte per leaf is copied to the host for the coarsening and refinement passes
 * (src/my_p4est_refine_coarsen.cpp:1170-1205, used by update_p4est at
 * src/my_p4est_semi_lagrangian.cpp:480-490). */
int lsg_forest_refine_and_coarsen_device(lsg_forest* f, int min_lvl, int max_lvl, double lip, double band, const double* phi_dev,
                                         int* changed, void* stream);
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

/* ---- on-disk formats (host) ------------------------------------------------------------------- */

/* my_p4est_vtk_write_all (src/my_p4est_vtk.h:132-135, src/my_p4est_vtk.cpp:440-1872) for one process:
 * <filename>.pvtu and <filename>.vtu/0000.vtu, an XML unstructured grid with the nodes as points
 * ("Position"), the leaves as VTK_PIXEL / VTK_VOXEL cells, cell arrays proc_rank (and tree_idx when
 * write_tree), then the node fields (N values each) and cell fields (one value per leaf). binary = 0
 * writes ascii (the reference's default), 1 inline base64. */
int lsg_vtk_write_all(const lsg_forest* f, const char* filename, int write_tree, int num_point, const char* const* point_names,
                      const double* const* point_values, int num_cell, const char* const* cell_names, const double* const* cell_values,
                      int binary);
/* VecDump (src/my_p4est_save_load.h:61, src/my_p4est_save_load.cpp:77-98) as one process writes it:
 * nvecs vectors of n doubles as PETSc binary Vec records (big-endian; int32 class id 1211214, the size
 * as a 32-bit PetscInt, or 64-bit when petsc_int64, then the values), readable by PETSc's VecLoad.
 * my_p4est_save_forest_and_data (src/my_p4est_save_load.cpp:350-380) writes one such file,
 * <folder>/<name>.petscbin, per group of vectors. */
int lsg_vec_dump(const char* fname, int nvecs, const double* const* vecs, int64_t n, int petsc_int64);
int lsg_vec_load(const char* fname, int nvecs, double* const* vecs, int64_t n, int petsc_int64);
/* The forest's leaves (and brick) in this library's own file format (p4est's own format is not
 * written); load rebuilds the forest, nodes not built. */
int lsg_forest_save(const lsg_forest* f, const char* fname);
int lsg_forest_load(const char* fname, lsg_forest** out);

/* ---- level set (device) ----------------------------------------------------------------------- */

/* my_p4est_level_set_t(my_p4est_node_neighbors_t*) (src/my_p4est_level_set.h:385-392): builds the
 * device tables of the grid. The forest must outlive the object and keep its nodes. */
int lsg_level_set_create(const lsg_forest* f, lsg_level_set** out);
/* The same with flags. LSG_BUILD_ON_DEVICE: the node-neighbour tables are built on the GPU (the
 * neighbour construction of src/my_p4est_node_neighbors.cpp:114-1201 runs one thread per node) instead
 * of on the host; results are bit-identical either way. No reference counterpart (the reference
 * builds its neighbours on the host). */
#define LSG_BUILD_ON_DEVICE 1
int lsg_level_set_create_ex(const lsg_forest* f, int flags, lsg_level_set** out);
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
/* reinitialize_2nd_order_with_mask(phi, mask, number_of_masked, iterations, limit)
 * (src/my_p4est_level_set.h:487-525) generalised to every order: the nodes where mask == 0 are left out
 * of the updates (their value is kept, their neighbours still read it). mask: N values, host or device
 * like phi. The reference's call is orders (2, 2) with limits (limit, -limit). */
int lsg_reinitialize_with_mask(lsg_level_set* ls, double* phi, const double* mask, int order_space, int order_pseudotime,
                               double limit_high, double limit_low, int iterations, int precision);
int lsg_reinitialize_with_mask_device(lsg_level_set* ls, double* phi_dev, const double* mask_dev, int order_space, int order_pseudotime,
                                      double limit_high, double limit_low, int iterations, int precision);
/* No counterpart in the reference. lsg_reinitialize_device with precision LSG_FP64, allocating no
 * memory: the work vectors (114 bytes per node in 3D, 82 in 2D, each array padded to 256 bytes)
 * come from one static device array of LSG_NOALLOC_SCRATCH_BYTES per device; larger grids return
 * LSG_EINVAL. It serves callers that cannot allocate inside the call: a solver whose device memory
 * is handed out by another pool (cudaMalloc there fails or fragments it), a time loop that cannot
 * take the device-wide synchronisation of cudaFree, and programs with many level-set objects on
 * small grids, which would otherwise each keep their own work vectors.
 * Every call runs on the level set's device and looks the array's address up there with
 * cudaGetSymbolAddress; the first call on a device also loads the array's module, so make it before any
 * stream capture. Nothing in the array must start at zero. All calls on one device share the array:
 * calls that overlap there (other streams, threads or level-set objects) race on it, so the caller must
 * serialise them. */
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
/* ---- first derivatives, normals, curvature (FP64, the reference's arithmetic) ---------------- */

/* my_p4est_node_neighbors_t::first_derivatives_central (src/my_p4est_node_neighbors.cpp:1643-1948):
 * out = dim x N gradient of f (quad_neighbor_nodes_of_node_t::gradient, central differences of the
 * linearly interpolated neighbours with the tangential second-derivative correction,
 * src/my_p4est_quad_neighbor_nodes_of_node.cpp:575-640). */
int lsg_first_derivatives(lsg_level_set* ls, const double* f, double* out);
int lsg_first_derivatives_device(lsg_level_set* ls, const double* f_dev, double* out_dev);
/* compute_normals(neighbors, phi, normals[]) (src/my_p4est_utils.cpp:1717-1739): dim x N unit normals,
 * 0 where |grad phi| < EPS. */
int lsg_compute_normals(lsg_level_set* ls, const double* phi, double* normals);
int lsg_compute_normals_device(lsg_level_set* ls, const double* phi_dev, double* normals_dev);
/* compute_mean_curvature(neighbors, normals[], kappa) (src/my_p4est_utils.cpp:1658-1696): divergence of
 * the normals. */
int lsg_compute_mean_curvature(lsg_level_set* ls, const double* normals, double* kappa);
int lsg_compute_mean_curvature_device(lsg_level_set* ls, const double* normals_dev, double* kappa_dev);
/* compute_normals_and_mean_curvature(neighbors, phi, normals[], kappa) (src/my_p4est_utils.cpp:2776-2802):
 * kappa from the gradient and phi (get_curvature, src/my_p4est_quad_neighbor_nodes_of_node.h:2051-2087),
 * then the normals. */
int lsg_compute_normals_and_mean_curvature(lsg_level_set* ls, const double* phi, double* normals, double* kappa);
int lsg_compute_normals_and_mean_curvature_device(lsg_level_set* ls, const double* phi_dev, double* normals_dev,
                                                  double* kappa_dev);

/* ---- extension over the interface (FP64, the reference's arithmetic) ------------------------ */

/* my_p4est_level_set_t::extend_Over_Interface_TVD(phi, q, iterations, order, band_use, band_extend,
 * normal, mask) (src/my_p4est_level_set.h:732-735, src/my_p4est_level_set.cpp:969-1764) with no
 * boundary conditions, no initial guesses (use_nonzero_guess false, q_n and q_nn NULL) and one-step
 * extrapolation: q (N values) is extended in place from the region where mask < 0 along the normals
 * by `iterations` upwind pseudo-time steps of the constant (order 0), linear (order 1) or quadratic
 * (order 2) extension. normals (dim x N) may be NULL (computed from phi as compute_normals does);
 * mask (N) may be NULL (phi is used). The reference's defaults are band_use = -DBL_MAX and
 * band_extend = DBL_MAX. */
int lsg_extend_over_interface_tvd(lsg_level_set* ls, const double* phi, double* q, int iterations, int order, double band_use,
                                  double band_extend, const double* normals, const double* mask);
int lsg_extend_over_interface_tvd_device(lsg_level_set* ls, const double* phi_dev, double* q_dev, int iterations, int order,
                                         double band_use, double band_extend, const double* normals_dev, const double* mask_dev);
/* The same with the reference's remaining arguments except bc (boundary conditions belong to the
 * Poisson solvers): use_nonzero_guess (where no normal derivative can be computed, start from n . grad q
 * and n . grad q_n instead of zero) and q_n / q_nn (N values each or NULL, in and out: their values are
 * the starting guesses where nothing is computed, and they receive the extended first and second
 * normal derivatives), as in src/my_p4est_level_set.cpp:1049-1360. */
int lsg_extend_over_interface_tvd_ex(lsg_level_set* ls, const double* phi, double* q, int iterations, int order, double band_use,
                                     double band_extend, const double* normals, const double* mask, int use_nonzero_guess, double* q_n,
                                     double* q_nn);
int lsg_extend_over_interface_tvd_ex_device(lsg_level_set* ls, const double* phi_dev, double* q_dev, int iterations, int order,
                                            double band_use, double band_extend, const double* normals_dev, const double* mask_dev,
                                            int use_nonzero_guess, double* q_n_dev, double* q_nn_dev);

/* my_p4est_level_set_t::extend_from_interface_to_whole_domain_TVD(phi, qi, q, iterations, mask, band_zero,
 * band_smooth, cf, grad_phi, blocksize) (src/my_p4est_level_set.h:775-776,
 * src/my_p4est_level_set.cpp:3181-3767) without the cf callback: q (nfields x N, the reference's
 * blocksize with the components as consecutive blocks of N) receives the values of q_interface
 * (nfields x N) on the interface, interpolated with `method` (the reference's
 * interpolation_on_interface, LSG_QUADRATIC_NON_OSCILLATORY_CONTINUOUS_V2 by default) where a grid line
 * crosses the interface, extended in the normal direction on both sides by `iterations` TVD-RK2 steps.
 * mask (N, only with nfields == 1) and grad_phi (dim x N) may be NULL. q and q_interface must not
 * overlap. The reference's defaults are iterations 20, band_zero 2 and band_smooth 10. */
int lsg_extend_from_interface_to_whole_domain_tvd(lsg_level_set* ls, const double* phi, const double* q_interface, double* q, int nfields,
                                                  int iterations, const double* mask, double band_zero, double band_smooth,
                                                  const double* grad_phi, int method);
int lsg_extend_from_interface_to_whole_domain_tvd_device(lsg_level_set* ls, const double* phi_dev, const double* q_interface_dev,
                                                         double* q_dev, int nfields, int iterations, const double* mask_dev,
                                                         double band_zero, double band_smooth, const double* grad_phi_dev, int method);
/* The cf form of extend_from_interface_to_whole_domain_TVD (the reference's
 * double (*cf)(p4est_locidx_t node, int dir, double dist), src/my_p4est_level_set.cpp:3388-3590): the
 * caller gives the interface value of every grid line that crosses the interface, batched: count
 * (node, direction, distance) triples in the reference's call order (node by node, directions m00, p00,
 * 0m0, 0p0[, 00m, 00p]); return 0 on success. q starts at zero; q_interface supplies the values of the
 * other directions. One field, host arrays. */
typedef int (*lsg_interface_values_fn)(void* ctx, int64_t count, const int32_t* nodes, const int32_t* dirs, const double* dists,
                                       double* values);
int lsg_extend_from_interface_to_whole_domain_tvd_cf(lsg_level_set* ls, const double* phi, const double* q_interface, double* q,
                                                     int iterations, lsg_interface_values_fn cf, void* ctx, const double* grad_phi);

/* ---- node interpolation and the semi-Lagrangian step (FP64) --------------------------------- */

/* my_p4est_interpolation_nodes_t(ngbd) + set_input(F, Fxx, Fyy[, Fzz], method) + add_point +
 * interpolate (src/my_p4est_interpolation_nodes.h:33-103, src/my_p4est_interpolation_nodes.cpp:107-288,
 * src/my_p4est_interpolation.cpp:68-124): nfields fields F (nfields x N, node order) evaluated at
 * npts points xyz (dim doubles per point) on the level set's grid. Each point is located after
 * clip_in_domain (src/my_p4est_utils.h:2177-2187) with the face rule of
 * find_smallest_quadrant_containing_point (src/my_p4est_hierarchy.cpp:264-567); the weights use the
 * point as given. Fdd: nfields x dim x N second derivatives (all xx, then yy[, zz]) or NULL to compute
 * them as compute_derivatives does (the reference's on-the-fly laplace at the corners). method: an
 * LSG_LINEAR..LSG_QUADRATIC_NON_OSCILLATORY_CONTINUOUS_V2 value. out: nfields x npts. */
int lsg_interpolate_nodes(lsg_level_set* ls, const double* xyz, int64_t npts, const double* F, int nfields, const double* Fdd,
                          int method, double* out);
int lsg_interpolate_nodes_device(lsg_level_set* ls, const double* xyz_dev, int64_t npts, const double* F_dev, int nfields,
                                 const double* Fdd_dev, int method, double* out_dev);
/* index (in lsg_forest_leaves order) of the leaf find_smallest_quadrant_containing_point picks for
 * each point after clipping (device pointers) */
int lsg_locate_points_device(lsg_level_set* ls, const double* xyz_dev, int64_t npts, int32_t* leaf_dev);

/* my_p4est_semi_lagrangian_t::advect_from_n_to_np1(dt, Vec* v, Vec** vxx, phi_n, phi_xx_n, phi_np1)
 * (src/my_p4est_semi_lagrangian.cpp:148-223): ls is the grid at time n; xyz_np1 holds the npts nodes
 * of the grid at n+1 (lsg_forest_node_xyz of that forest). v: dim x N velocity components; vdd:
 * dim x dim x N (component, axis, node) or NULL; phi_dd: dim x N or NULL. RK2 backtrace
 * x* = x - dt/2 v(x), x_d = x - dt v(x*), both clipped; phi_np1 = phi_n(x_d). */
int lsg_semi_lagrangian_advect(lsg_level_set* ls, const double* xyz_np1, int64_t npts, double dt, const double* v, const double* vdd,
                               const double* phi_n, const double* phi_dd, int velo_method, int phi_method, double* phi_np1);
int lsg_semi_lagrangian_advect_device(lsg_level_set* ls, const double* xyz_np1_dev, int64_t npts, double dt, const double* v_dev,
                                      const double* vdd_dev, const double* phi_n_dev, const double* phi_dd_dev, int velo_method,
                                      int phi_method, double* phi_np1_dev);

/* the two-velocity second-order step my_p4est_semi_lagrangian_t::advect_from_n_to_np1(dt_nm1, dt_n, vnm1,
 * vxx_nm1, vn, vxx_n, phi_n, phi_xx_n, phi_np1) (src/my_p4est_semi_lagrangian.cpp:225-319), the step
 * update_p4est(Vec* vnm1, Vec* vn, dt_nm1, dt_n, phi, ...) (:779-939) repeats while it regrids: ls_n is the
 * grid at time n (vn: dim x N_n, phi_n, phi_dd: dim x N_n or NULL, vn_dd: dim x dim x N_n or NULL), ls_nm1
 * the grid at n-1 (vnm1: dim x N_nm1, vnm1_dd: dim x dim x N_nm1 or NULL), xyz_np1 the npts nodes of the grid
 * at n+1. v_n is interpolated at the new nodes quadratically (as the reference does), x* = x - dt_n/2 v_n
 * (clipped), v* = (1 + dt_n/(2 dt_nm1)) v_n(x*) - dt_n/(2 dt_nm1) v_nm1(x*), both with velo_method, and
 * phi_np1 = phi_n(x - dt_n v*) (clipped) with phi_method. Both level sets must be on one device. */
int lsg_semi_lagrangian_advect2(lsg_level_set* ls_n, lsg_level_set* ls_nm1, const double* xyz_np1, int64_t npts, double dt_nm1,
                                double dt_n, const double* vnm1, const double* vnm1_dd, const double* vn, const double* vn_dd,
                                const double* phi_n, const double* phi_dd, int velo_method, int phi_method, double* phi_np1);
int lsg_semi_lagrangian_advect2_device(lsg_level_set* ls_n, lsg_level_set* ls_nm1, const double* xyz_np1, int64_t npts, double dt_nm1,
                                       double dt_n, const double* vnm1, const double* vnm1_dd, const double* vn, const double* vn_dd,
                                       const double* phi_n, const double* phi_dd, int velo_method, int phi_method, double* phi_np1);

/* the CF overload advect_from_n_to_np1(dt, const CF** v, phi_n, phi_xx_n, phi_np1)
 * (src/my_p4est_semi_lagrangian.cpp:108-146) with an analytic velocity evaluated on the device:
 * velocity LSG_VELOCITY_VORTEX is the single vortex of examples/level_set_advection/main_2d.cpp:116-181
 * times params[0] (the example's direction sign, or cos(pi t/T)). */
enum { LSG_VELOCITY_VORTEX = 0 };
int lsg_semi_lagrangian_advect_cf(lsg_level_set* ls, const double* xyz_np1, int64_t npts, double dt, int velocity,
                                  const double* params, int nparams, const double* phi_n, const double* phi_dd, int phi_method,
                                  double* phi_np1);
int lsg_semi_lagrangian_advect_cf_device(lsg_level_set* ls, const double* xyz_np1_dev, int64_t npts, double dt, int velocity,
                                         const double* params, int nparams, const double* phi_n_dev, const double* phi_dd_dev,
                                         int phi_method, double* phi_np1_dev);
/* advect_from_n_to_np1(dt, const CF** v, phi_n, phi_xx_n, phi_np1) (src/my_p4est_semi_lagrangian.cpp:108-146)
 * for any velocity: the callback evaluates it on the host at npts points (xyz and v both npts x dim,
 * interleaved; return 0 on success), the departure points x* = x - dt/2 v(x) and x_d = x - dt v(x*)
 * (each clipped to the domain) are formed on the host as the reference does, and phi (host, N) is
 * interpolated at x_d on the GPU with phi_method. */
typedef int (*lsg_velocity_fn)(void* ctx, int64_t npts, const double* xyz, double* v);
int lsg_semi_lagrangian_advect_callback(lsg_level_set* ls, const double* xyz_np1, int64_t npts, double dt, lsg_velocity_fn velocity,
                                        void* ctx, const double* phi, const double* phi_dd, int phi_method, double* phi_np1);

/* The band check that accompanies every result: max |a - b| over the nodes with |b| < band, in FP64
 * on the device (warp-shuffle reduction), b the reference field (e.g. the FP64 result), a the field
 * checked; *out is NaN if a NaN was met, *count (may be NULL) the number of nodes in the band. Device
 * pointers of N values; no counterpart in the reference, whose examples compute the same norm on the
 * host (examples/reinitialization/main_2d.cpp:254-262). */
int lsg_band_linf_device(lsg_level_set* ls, const double* a_dev, const double* b_dev, double band, double* out, int64_t* count);
/* The per-rank FP64 sweeps of a Morton-range split of one grid: on one rank of an MPI run the reference
 * sweeps its layer and local node lists (reinitialize_one_iteration(phi_np1, list_of_node_idx, ...),
 * src/my_p4est_level_set.cpp:59-288; second_derivatives_central over the same lists,
 * src/my_p4est_node_neighbors.cpp:1552-1627) between ghost updates (:376-401, :450-464). Each call covers the
 * nodes [first, first + count) only and reads every other node from the full-length device arrays (node
 * order), whose ghost values the caller keeps current with its own halo exchange.
 * lsg_second_derivatives_range_device: f_dd (dim x N) at the range.
 * lsg_reinit_prep_range_device: what the stages derive from phi_0 alone (status, subcell distances, kept in
 * the level set) with the phi_0 limits of reinitialize_within_range_of_phi_0; phi0_dd as from
 * lsg_second_derivatives_range_device.
 * lsg_reinit_stage_range_device: out = one stage of phin (phin_dd its second derivatives), or
 * 0.5 (avg_with + stage) when avg_with is given (the RK average; may alias out).
 * The second derivatives are required at every order (the quadratic neighbour values of
 * ngbd_with_quadratic_interpolation read the node's own); at second order in space the stages also read
 * them at the neighbours, whose ghost values the caller must then update too. */
int lsg_second_derivatives_range_device(lsg_level_set* ls, const double* f_dev, double* f_dd_dev, int64_t first, int64_t count);
int lsg_reinit_prep_range_device(lsg_level_set* ls, const double* phi0_dev, const double* phi0_dd_dev, int order_space, double limit_high,
                                 double limit_low, int64_t first, int64_t count);
int lsg_reinit_stage_range_device(lsg_level_set* ls, int order_space, const double* phi0_dev, const double* phin_dev,
                                  const double* phin_dd_dev, double* out_dev, const double* avg_with_dev, int64_t first, int64_t count);
/* One advect_in_normal_direction_one_iteration sweep (src/my_p4est_level_set.cpp:559-654) over the nodes
 * [first, first + count) of a rank's Morton range: out = phin - dt vn |grad phin| with the quadratic neighbour
 * values from phin_dd (phin's second derivatives) and the minmod terms from minmod_dd (the caller's second
 * derivatives, or phin_dd), or 0.5 (avg_with + that) when avg_with is given (the RK average; may alias out).
 * Reads the ghosts of phin and minmod_dd. */
int lsg_advect_stage_range_device(lsg_level_set* ls, const double* phin_dev, const double* phin_dd_dev, const double* minmod_dd_dev,
                                  const double* vn_dev, double dt, double* out_dev, const double* avg_with_dev, int64_t first,
                                  int64_t count);
/* The mixed-precision reinitialisation of one rank of a Morton split, stage by stage, so that the caller updates
 * ghosts between stages (the mixed tables order nodes by stencil type, so a rank keeps every node and leaves the
 * ones it does not own out of the updates):
 * lsg_mixed_split_begin_device: the phi_0-only FP64 step and phi_n in FP32 (phi_dev: N values, node order, valid
 * at the owned nodes and two rings of ghosts; mask_dev: N values, 0 leaves a node out of the updates, e.g. every
 * node the rank does not own; limits as lsg_reinitialize takes them);
 * lsg_mixed_split_stage_device: one RK stage, second order in time (stage 0: phi_n -> phi_1; stage 1: phi_1 ->
 * phi_n averaged with phi_n), all of it ordered before later work on the level set's stream;
 * lsg_mixed_split_field_device: the device address of the FP32 phi_n (which 0) or phi_1 (1), N values in slot
 * order, for the ghost update; lsg_mixed_split_slots_device: slot of every node (N int32, device);
 * lsg_mixed_split_end_device: phi (FP64, node order) from the last phi_n. */
int lsg_mixed_split_begin_device(lsg_level_set* ls, const double* phi_dev, const double* mask_dev, int order_space, double limit_high,
                                 double limit_low);
int lsg_mixed_split_stage_device(lsg_level_set* ls, int order_space, int stage);
int lsg_mixed_split_field_device(lsg_level_set* ls, int which, float** field_dev);
int lsg_mixed_split_slots_device(lsg_level_set* ls, int32_t* slots_dev);
int lsg_mixed_split_end_device(lsg_level_set* ls, double* phi_dev);

/* The interface-location check that accompanies every mixed-precision result: over the grid edges (a node
 * and a neighbour that its stencil reaches with one node) cut by the reference field b (e.g. the FP64
 * result), the largest distance between the zero crossings of a and b along the edge, each the linear root
 * d b_n / (b_n - b_nb) in FP64 on the device; *edges (may be NULL) counts the cut edges (both ends),
 * *mismatched (may be NULL) those a does not cut. No counterpart in the reference. */
int lsg_interface_location_error_device(lsg_level_set* ls, const double* a_dev, const double* b_dev, double* out, int64_t* edges,
                                        int64_t* mismatched);

/* ---- batched reinitialisation (mixed precision) --------------------------------------------- */

/* No single counterpart in the reference, which reinitialises each field with its own
 * my_p4est_level_set_t::reinitialize_2nd_order(phi_k, iterations_k) call (src/my_p4est_level_set.h:468-472).
 * A batch is a level set over the disjoint union of `count` grids of one dimension and equal tree
 * sizes: their tables are concatenated (grid k owns union nodes offsets[k] .. offsets[k+1]-1, in its
 * own node order) so every stage kernel covers all grids in one launch. The returned handle is a
 * level-set handle, destroyed with lsg_level_set_destroy; the forests must outlive it. */
int lsg_batch_create(int count, const lsg_forest* const* forests, lsg_level_set** out);
/* The same with flags. LSG_BUILD_ON_DEVICE: each grid's node-neighbour tables are built on the GPU
 * and concatenated there, and the union's mixed tables are built on the GPU (same results). */
int lsg_batch_create_ex(int count, const lsg_forest* const* forests, int flags, lsg_level_set** out);
int lsg_batch_count(const lsg_level_set* batch);
int lsg_batch_offsets(const lsg_level_set* batch, int64_t* offsets); /* count + 1 values */
/* reinitialize_2nd_order of every grid, grid k for iterations[k] pseudo-time iterations (mixed
 * precision, limits +-DBL_MAX): phi holds all grids' values in union node order. use_graph: run the
 * iteration loop as one CUDA graph, captured on the first call with these iteration counts and
 * replayed afterwards (make that first call outside any stream capture). */
int lsg_batch_reinitialize(lsg_level_set* batch, double* phi, const int* iterations, int use_graph);
int lsg_batch_reinitialize_device(lsg_level_set* batch, double* phi_dev, const int* iterations, int use_graph);
/* Launch shape of the mixed stage kernels, seven ints: config[0] threads per block (32..256),
 * config[1] grid of the persistent uniform-stencil kernel, config[2] grid of the persistent regular
 * kernel (0: one full wave), config[3] pipeline of the uniform kernel (1 or 2 nodes in flight per
 * thread, or 3 / 4: the nodes' table words and a window of phi bulk-copied into shared memory two /
 * three tiles ahead; a bounded wait of that kernel that gives up makes the call return LSG_ETIMEOUT; or 5,
 * the default: as 1 with the kernel's registers capped so that more of its threads stay resident),
 * config[4] nodes on either side of a tile in that window (a multiple of 4 in 0..4096), config[5] streams
 * of a stage (2: second derivatives and irregular nodes beside the uniform nodes; 1: the four kernels one
 * after another), config[6] with two streams their pairing and the one the block scheduler prefers (0:
 * second derivatives then irregular nodes beside uniform then other regular nodes, neither preferred; 1: the
 * first chain preferred; 2: the second; 3 and 4: the same with the irregular and other regular nodes
 * swapped between the chains, the first / second chain preferred).
 * lsg_level_set_autotune times candidate shapes on phi (host, node order) for `trials` iterations
 * each, times the four fastest and the default shape again with runs four times longer, keeps the fastest
 * and returns it in config (may be NULL). Results do not depend on the shape. */
int lsg_level_set_autotune(lsg_level_set* ls, const double* phi, int trials, int* config);
int lsg_level_set_stage_config(const lsg_level_set* ls, int* config);
int lsg_level_set_set_stage_config(lsg_level_set* ls, const int* config);
/* Bound of the bulk-copy stage kernel's waits for its own copies, in SM clock cycles (0 restores the
 * default, about a second). A wait that runs out stops that kernel's blocks after their copies have landed
 * and makes the call return LSG_ETIMEOUT; the next call starts clean. No counterpart in the reference
 * (which has no device waits); a diagnostic for callers that must bound every device-side wait. */
int lsg_level_set_set_wait_limit(lsg_level_set* ls, long long cycles);

/* Sizes of the mixed tables (7 values): nodes, regular nodes, uniform-stencil nodes, irregular nodes,
 * regular nodes of the extended second-derivative set, geometry classes, cross-term corrections. */
int lsg_level_set_table_stats(lsg_level_set* ls, int64_t* out);

/* kernel classes reported by lsg_level_set_kernel_times */
enum {
  LSG_K_DD64 = 0, LSG_K_PREP64, LSG_K_STAGE64, LSG_K_ADVECT64, LSG_K_DD32, LSG_K_PREP_MIXED, LSG_K_STAGE32, LSG_K_ADVECT32,
  LSG_K_CONVERT, LSG_K_COPY, LSG_K_INTERP, LSG_K_NUM
};
/* record CUDA events around every launch (adds a little overhead) */
int lsg_level_set_enable_kernel_timing(lsg_level_set* ls, int on);
/* per class: total milliseconds and number of launches since the last reset (synchronises) */
int lsg_level_set_kernel_times(lsg_level_set* ls, double* ms, int64_t* counts, int nkinds, int reset);
/* number of kernel launches this object issued since the last kernel-times reset */
int64_t lsg_level_set_launch_count(const lsg_level_set* ls);

/* ---- device memory (no reference counterpart; PETSc owns the reference's Vec memory) ---------- */
/* Device memory released by level sets, grids' device copies and temporaries is kept for reuse
 * (handed out again only after a device synchronisation that follows its release).
 * lsg_device_cache_bytes: bytes held that way now; lsg_device_cache_release: give them all back to
 * the driver (synchronises the device). */
int64_t lsg_device_cache_bytes(void);
int lsg_device_cache_release(void);

#ifdef __cplusplus
}
#endif

#endif /* LSGPU_H */
