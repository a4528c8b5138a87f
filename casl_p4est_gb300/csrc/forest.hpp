// Host forest: the minimal stand-in for the p4est objects that parCASL's level-set path reads.
//
// parCASL builds its grids with p4est (brick connectivity, refinement passes, ghost layer, node
// numbering). p4est is an external library, so this file provides the pieces the hot path needs,
// for a single process:
//   - brick connectivity and tree geometry          src/my_p4est_tools.c:37-170 (my_p4est_brick_new)
//   - one refinement pass over all leaves            p4est_refine(non-recursive), as called by
//                                                    examples/reinitialization/main_2d.cpp:169-173
//   - node numbering where every leaf corner is an independent node, owned by the lowest tree
//     that touches it, clamped inside that tree, sorted by (tree, Morton)
//                                                    src/my_p4est_nodes.h:55-63, src/my_p4est_nodes.c:606-627
//   - local_nodes: corner node of each leaf          p4est_nodes_t::local_nodes
//   - point location of the leaf containing a logical point
//                                                    src/my_p4est_hierarchy.cpp:569-600
// Leaves are kept in tree-major Morton order (p4est's linear order), so locating the leaf that
// contains a point is a binary search over sorted keys instead of a walk down a cell tree.
#pragma once
#include <stdint.h>

#include <functional>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "lsg_common.h"

namespace lsg {

struct Brick {
  int dim = 2;
  int n[3] = {1, 1, 1};
  double xyz_min[3] = {0, 0, 0};
  double xyz_max[3] = {1, 1, 1};
  int periodic[3] = {0, 0, 0};
  int num_trees = 1;
  std::vector<int32_t> ijk_to_tree;  // n0*n1*k + n0*j + i -> tree id
  std::vector<int32_t> tree_ijk;     // 3 per tree
  std::vector<double> tmin, tmax;    // 3 per tree: vertex coordinates of the tree's corners 0 and last

  void init(int dim, const int* n, const double* xyz_min, const double* xyz_max, const int* periodic);
  int32_t tree_at(const int* ijk) const { return ijk_to_tree[(size_t)n[0] * n[1] * ijk[2] + (size_t)n[0] * ijk[1] + ijk[0]]; }
};

struct Quad {
  int32_t x[3];
  int32_t tree;
  int32_t level;
};

// An array that is replaced whole and never edited in place, so copies of its owner share it.
template <typename T>
class SharedArray {
 public:
  SharedArray() : p_(std::make_shared<const std::vector<T>>()) {}
  size_t size() const { return p_->size(); }
  bool empty() const { return p_->empty(); }
  const T& operator[](size_t i) const { return (*p_)[i]; }
  const T* data() const { return p_->data(); }
  typename std::vector<T>::const_iterator begin() const { return p_->begin(); }
  typename std::vector<T>::const_iterator end() const { return p_->end(); }
  const std::vector<T>& vec() const { return *p_; }
  void replace(std::vector<T>&& v) { p_ = std::make_shared<const std::vector<T>>(std::move(v)); }

 private:
  std::shared_ptr<const std::vector<T>> p_;
};

// Node numbering of a forest. Built whole and never changed afterwards, so copies of a forest share
// one instance (a forest copied before a regrid pays nothing for nodes that the regrid replaces).
// A numbering made on the device stays there until host code first reads the arrays: host() copies
// them down once (fetch), so a regrid loop that only feeds device kernels never downloads them.
struct NodeArrays {
  size_t count = 0;                  // number of nodes
  std::vector<int32_t> node_tree;    // owner tree
  std::vector<int32_t> node_x;       // D per node, clamped logical coordinates in the owner tree
  std::vector<uint64_t> node_key;
  std::vector<int32_t> local_nodes;  // CHILDREN per leaf, corner c = xbit + 2 ybit + 4 zbit
  std::function<void(NodeArrays&)> fetch;  // fills the vectors from the device copy (device numbering)

  const NodeArrays& host() const {
    if (fetch) std::call_once(fetched_, [this] { fetch(const_cast<NodeArrays&>(*this)); });
    return *this;
  }

 private:
  mutable std::once_flag fetched_;
};

template <int D>
struct Forest {
  using DD = Dim<D>;
  Brick brick;
  SharedArray<Quad> leaves;          // tree-major Morton order; replaced whole, shared by copies
  SharedArray<uint64_t> leaf_key;    // (tree << D*MAXLEVEL) | morton(x)
  // node numbering (valid once build_nodes() ran); replaced as a whole, shared by copies
  std::shared_ptr<const NodeArrays> nd = std::make_shared<const NodeArrays>();
  bool nodes_built = false;
  // device copy of the leaves and nodes (ForestDevice, flatten.hpp), set by the device node numbering
  // or on first device use, dropped whenever the leaves or the nodes change
  std::shared_ptr<void> device;

  void init(const int* n, const double* xyz_min, const double* xyz_max, const int* periodic);
  // One refinement pass: every leaf with tags[i] != 0 is replaced by its CHILDREN children.
  void refine(const uint8_t* tags);
  // Coarsening pass: each complete family of CHILDREN sibling leaves with all tags set is merged.
  void coarsen(const uint8_t* tags);
  void build_nodes();
  // the leaves changed: the node numbering and the device copy no longer hold
  void drop_nodes() {
    nodes_built = false;
    nd = std::make_shared<const NodeArrays>();
    device.reset();
  }
  // Replace the leaves with a caller-supplied complete linear forest (tree-major Morton order,
  // every tree covered exactly once); throws std::invalid_argument otherwise.
  void set_leaves(size_t n, const int32_t* tree, const int32_t* level, const int32_t* xyz);
  // splitting_criteria_tag_t::refine_and_coarsen after tagging (src/my_p4est_refine_coarsen.cpp:1170-1205):
  // one coarsening pass over complete families whose leaves are all tagged -1, then one refinement
  // pass over the surviving leaves tagged +1 (a parent made by coarsening is not refined).
  // Returns true if any leaf was created.
  bool coarsen_then_refine(const int8_t* tag);
  // splitting_criteria_tag_t::tag_quadrant (src/my_p4est_refine_coarsen.cpp:422-479,
  // finest_in_negative_flag = false) from the node values phi (nodes must be built):
  // +1 refine, -1 coarsen, 0 keep.
  void tag_refine_coarsen(int min_lvl, int max_lvl, double lip, double band, const double* phi, int8_t* tag) const;

  size_t num_leaves() const { return leaves.size(); }
  size_t num_nodes() const { return nd->count; }

  // Leaf containing the logical point x (0 <= x < ROOT_LEN) of tree `tree`; -1 if none.
  int32_t find_leaf(int32_t tree, const int32_t* x) const;
  // Map global logical coordinates (tree_ijk*ROOT_LEN + local) to (tree, local); false if outside.
  bool global_to_tree(const int64_t* G, int32_t& tree, int32_t* x) const;
  // Node coordinates, as node_x_fr_n / node_xyz_fr_n (src/my_p4est_utils.h:1346-1405).
  void node_xyz(int32_t n, double* xyz) const;
  // Unclamped logical coordinates of a node (p4est_node_unclamp).
  void node_unclamped(int32_t n, int32_t* x) const {
    for (int a = 0; a < D; ++a) {
      int32_t v = nd->host().node_x[(size_t)D * n + a];
      x[a] = (v == DD::ROOT_LEN - 1) ? DD::ROOT_LEN : v;
    }
  }
  // Leaves i..i+CHILDREN-1 form a complete family with every tag set.
  bool family_at(size_t i, const uint8_t* tags) const;
  // Finest leaf level present (for dx_min reporting).
  int max_level() const;
  int min_level() const;
  // Smallest cell size along each axis (get_dxyz_min, src/my_p4est_utils.cpp).
  void dxyz_min(double* dxyz) const;
};

// Parallel sort of 64-bit keys (OpenMP when available).
void sort_u64(std::vector<uint64_t>& v);

}  // namespace lsg
