// On-disk formats (io.cpp): VTK output of a forest with node and cell fields, PETSc binary vectors
// as VecDump writes them, and this library's forest leaf-list file.
#pragma once
#include <stdint.h>

#include <string>
#include <vector>

#include "forest.hpp"

namespace lsg {

template <int D>
void vtk_write_all(const Forest<D>& F, const std::string& filename, bool write_tree, const std::vector<std::string>& point_names,
                   const std::vector<const double*>& point_values, const std::vector<std::string>& cell_names,
                   const std::vector<const double*>& cell_values, bool binary);
void vec_dump(const std::string& fname, const std::vector<const double*>& vecs, int64_t n, bool int64_index);
void vec_load(const std::string& fname, const std::vector<double*>& vecs, int64_t n, bool int64_index);
template <int D>
void forest_save(const Forest<D>& F, const std::string& fname);
void forest_header(const std::string& fname, int* dim, int* n, double* lo, double* hi, int64_t* nleaves);
template <int D>
void forest_load_leaves(Forest<D>& F, const std::string& fname);

}  // namespace lsg
