// Device flattener (flatten.cu): the FP64 and mixed tables built on the GPU from the grid, with the
// same contents as the host flattener (tables.cpp, tables32.cpp) up to the numbering of the irregular
// geometry classes (and so the order of the irregular nodes), which no result depends on.
#pragma once
#include <stdint.h>

#include "devbuf.hpp"
#include "forest.hpp"
#include "kernels.h"

namespace lsg {

// The grid on the device: leaves (keys, levels, corner nodes, the coarse-cell table of DLoc), the
// brick, and the nodes (owner tree, clamped logical coordinates).
template <int D>
struct DForest {
  int64_t nleaves, N;
  const uint64_t* key;
  const int8_t* level;
  const int32_t* local_nodes;
  const int32_t* ctab;
  int L0;
  int64_t ncoarse;
  int n[3];
  const int32_t* ijk_to_tree;
  const int32_t* tree_ijk;  // 3 per tree
  const double* tmin;
  const double* tmax;
  const int32_t* node_tree;
  const int32_t* node_x;    // D per node
};

// Device copy of a forest's leaves (keys, levels), brick (tree coordinates, tree lookup, tree
// corners) and nodes (keys, owner tree, clamped coordinates, corner nodes of every leaf). Held by
// Forest::device and dropped when the leaves or nodes change.
template <int D>
struct ForestDevice {
  int64_t nl = 0, nn = 0;
  DevBuf<uint64_t> leaf_key, node_key;
  DevBuf<int8_t> level;
  DevBuf<int32_t> local_nodes, node_tree, node_x, tree_ijk, ijk_to_tree;
  DevBuf<double> tmin, tmax;
};

// Node numbering on the device (the same keys, order and corner map as Forest::build_nodes); the
// device copy stays attached to the forest and the host arrays are copied down on first host use.
template <int D>
void build_nodes_device(Forest<D>& F, cudaStream_t s);
// Concatenation of index tables: dst[p * Ndst + off + i] = src[p * n + i] (+ add where src >= 0) for
// every plane p < planes and i < n.
void concat_index_planes(const int32_t* src, int64_t n, int planes, int32_t* dst, int64_t Ndst, int64_t off, int32_t add,
                         cudaStream_t s);
// Coarse-cell table of point location: for each cell i of the uniform level L0 in each tree (ncoarse
// cells per tree, nt trees), the last leaf whose key is <= the cell's first point (0 if none), and
// ctab[nt * ncoarse] = nl - 1; from the sorted leaf keys on the device.
template <int D>
void coarse_table_device(const uint64_t* leaf_key, int64_t nl, int nt, int L0, int32_t* ctab, cudaStream_t s);
// The forest's device copy, uploaded from the host arrays if the forest has none (nodes must be built).
template <int D>
ForestDevice<D>& forest_device(Forest<D>& F, cudaStream_t s);
// Node coordinates (N x D, node_x_fr_n) from the device copy.
template <int D>
void node_xyz_device(Forest<D>& F, double* out, cudaStream_t s);
// splitting_criteria_tag_t::refine_and_coarsen with the tags evaluated on the device from the node
// values phi (device): only one byte per leaf comes back to the host for the coarsen/refine passes.
template <int D>
bool refine_and_coarsen_device(Forest<D>& F, int min_lvl, int max_lvl, double lip, double band, const double* phi, cudaStream_t s);

// FP64 tables (sizes as Tables64); returns the number of correction records.
template <int D>
struct Tab64Dev {
  DevBuf<int32_t>* nbr;
  DevBuf<double>* w;
  DevBuf<double>* nrm;
  DevBuf<double>* d;
  DevBuf<double>* q;
  DevBuf<int32_t>* cidx;
  DevBuf<double>* crec;
  DevBuf<uint8_t>* wall;
  DevBuf<double>* smin;
};
template <int D>
int64_t build_tables64_device(const DForest<D>& F, const Tab64Dev<D>& out, cudaStream_t s);

// Mixed tables from the FP64 tables T (R correction records) and the tree size per axis.
template <int D>
struct MixedDev {
  DevBuf<uint32_t>* r_meta;
  DevBuf<int32_t>* r_nbr;
  DevBuf<int32_t>* r_nbr2;
  DevBuf<uint32_t>* r_meta2;
  DevBuf<uint32_t>* i_meta;
  DevBuf<uint32_t>* i_cls;
  DevBuf<int32_t>* i_nbr;
  DevBuf<float>* i_wf;
  DevBuf<float>* i_d;
  DevBuf<float>* i_q;
  DevBuf<int32_t>* i_cidx;
  DevBuf<float>* corr;
  DevBuf<float>* cls32;
  DevBuf<double>* i_wf64;
  DevBuf<double>* i_d64;
  DevBuf<double>* i_q64;
  DevBuf<double>* corr64;
  DevBuf<int32_t>* perm;
  DevBuf<int32_t>* iperm;
  // scalars
  int64_t nR = 0, nI = 0, nU = 0, x_first = 0, nX = 0, ncls = 0;
  int base = 0;
};
template <int D>
void build_mixed_device(const DTab64<D>& T, int64_t R, const double* tree_size, MixedDev<D>& M, cudaStream_t s);

}  // namespace lsg
