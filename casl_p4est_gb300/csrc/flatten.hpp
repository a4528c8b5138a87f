// Device flattener (flatten.cu): the FP64 and mixed tables built on the GPU from the grid, with the
// same contents as the host flattener (tables.cpp, tables32.cpp) up to the numbering of the irregular
// geometry classes (and so the order of the irregular nodes), which no result depends on.
#pragma once
#include <stdint.h>

#include "devbuf.hpp"
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
