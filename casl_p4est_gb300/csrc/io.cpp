// On-disk formats of the grid and its node fields, for checks and restarts:
//
//   VTK       my_p4est_vtk_write_all (src/my_p4est_vtk.cpp:440-940, 1074-1872): an XML unstructured
//             grid written as <name>.pvtu plus the single piece <name>.vtu/0000.vtu (one process),
//             points = the nodes ("Position", Float64, z = 0 in 2D), cells = the leaves as VTK_PIXEL /
//             VTK_VOXEL with the corner nodes in p4est corner order, cell arrays proc_rank and
//             tree_idx, then the caller's node and cell scalars; ascii (the reference's default
//             build) or inline base64 binary.
//   PETSc     VecDump (src/my_p4est_save_load.cpp:77-98) as one process writes it: per vector the
//             PETSc binary Vec record, big-endian: int32 VEC_FILE_CLASSID (1211214), the global size
//             as PetscInt (int32, or int64 for a 64-bit-index PETSc), then the values as doubles.
//             Node vectors are in single-process node order, the order VecDump writes them in.
//   forest    a leaf list of this library's own (p4est's binary forest format belongs to p4est, a
//             dependency outside the reference tree, and is not restated here): magic, dimension,
//             brick, then tree, level and logical corner of every leaf, little-endian.
#include <stdint.h>
#include <stdio.h>
#include <string.h>
#include <sys/stat.h>

#include <algorithm>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "io.hpp"

namespace lsg {

namespace {

struct File {
  FILE* f = nullptr;
  File(const std::string& name, const char* mode) : f(fopen(name.c_str(), mode)) {
    if (!f) throw std::runtime_error("cannot open " + name);
  }
  ~File() {
    if (f) fclose(f);
  }
  void write(const void* p, size_t n) {
    if (n && fwrite(p, 1, n, f) != n) throw std::runtime_error("write failed");
  }
  void read(void* p, size_t n) {
    if (n && fread(p, 1, n, f) != n) throw std::runtime_error("read failed: file too short");
  }
  void close() {
    if (f && fclose(f) != 0) {
      f = nullptr;
      throw std::runtime_error("close failed");
    }
    f = nullptr;
  }
};

bool host_little_endian() {
  const uint16_t probe = 1;
  unsigned char b;
  memcpy(&b, &probe, 1);
  return b == 1;
}

// big-endian encoding, independent of the host's byte order
template <typename T>
void put_be(std::vector<unsigned char>& out, T v) {
  unsigned char b[sizeof(T)];
  memcpy(b, &v, sizeof(T));
  if (host_little_endian()) std::reverse(b, b + sizeof(T));
  out.insert(out.end(), b, b + sizeof(T));
}

template <typename T>
T get_be(const unsigned char* p) {
  unsigned char b[sizeof(T)];
  memcpy(b, p, sizeof(T));
  if (host_little_endian()) std::reverse(b, b + sizeof(T));
  T v;
  memcpy(&v, b, sizeof(T));
  return v;
}

const int32_t VEC_FILE_CLASSID = 1211214;

std::string base64(const unsigned char* p, size_t n) {
  static const char* tab = "ABCDEFGHIJKLMNOPQRSTUVWXYZabcdefghijklmnopqrstuvwxyz0123456789+/";
  std::string s;
  s.reserve((n + 2) / 3 * 4);
  for (size_t i = 0; i < n; i += 3) {
    const uint32_t a = p[i], b = i + 1 < n ? p[i + 1] : 0, c = i + 2 < n ? p[i + 2] : 0;
    const uint32_t t = (a << 16) | (b << 8) | c;
    s.push_back(tab[(t >> 18) & 63]);
    s.push_back(tab[(t >> 12) & 63]);
    s.push_back(i + 1 < n ? tab[(t >> 6) & 63] : '=');
    s.push_back(i + 2 < n ? tab[t & 63] : '=');
  }
  return s;
}

// one DataArray body: ascii values, or VTK's inline binary (base64 of a UInt32 byte count + the bytes)
template <typename T>
void data_array(File& f, const char* type, const char* name, int ncomp, const std::vector<T>& v, bool binary) {
  std::string head = std::string("        <DataArray type=\"") + type + "\" Name=\"" + name + "\"";
  if (ncomp > 1) head += " NumberOfComponents=\"" + std::to_string(ncomp) + "\"";
  head += std::string(" format=\"") + (binary ? "binary" : "ascii") + "\">\n";
  f.write(head.data(), head.size());
  if (binary) {
    std::vector<unsigned char> bytes(sizeof(uint32_t) + v.size() * sizeof(T));
    const uint32_t nb = (uint32_t)(v.size() * sizeof(T));
    memcpy(bytes.data(), &nb, sizeof(uint32_t));
    if (!v.empty()) memcpy(bytes.data() + sizeof(uint32_t), v.data(), v.size() * sizeof(T));
    const std::string s = "          " + base64(bytes.data(), bytes.size()) + "\n";
    f.write(s.data(), s.size());
  } else {
    std::string s;
    char buf[64];
    const size_t per_line = ncomp > 1 ? (size_t)ncomp : 8;
    for (size_t i = 0; i < v.size(); ++i) {
      if (i % per_line == 0) s += "         ";
      if (std::is_floating_point<T>::value)
        snprintf(buf, sizeof buf, " %24.16e", (double)v[i]);
      else
        snprintf(buf, sizeof buf, " %lld", (long long)v[i]);
      s += buf;
      if (i % per_line == per_line - 1 || i + 1 == v.size()) s += "\n";
    }
    f.write(s.data(), s.size());
  }
  const char* tail = "        </DataArray>\n";
  f.write(tail, strlen(tail));
}

std::string base_name(const std::string& path) {
  const size_t p = path.find_last_of('/');
  return p == std::string::npos ? path : path.substr(p + 1);
}

}  // namespace

template <int D>
void vtk_write_all(const Forest<D>& F, const std::string& filename, bool write_tree, const std::vector<std::string>& point_names,
                   const std::vector<const double*>& point_values, const std::vector<std::string>& cell_names,
                   const std::vector<const double*>& cell_values, bool binary) {
  constexpr int CH = Dim<D>::CHILDREN;
  const size_t nn = F.num_nodes(), nc = F.num_leaves();
  const std::string folder = filename + ".vtu";
  mkdir(folder.c_str(), 0755);
  {
    File f(folder + "/0000.vtu", "wb");
    std::string s = "<?xml version=\"1.0\"?>\n<VTKFile type=\"UnstructuredGrid\" version=\"0.1\"";
    s += binary ? " header_type=\"UInt32\"" : "";
    s += " byte_order=\"LittleEndian\">\n  <UnstructuredGrid>\n";
    s += "    <Piece NumberOfPoints=\"" + std::to_string(nn) + "\" NumberOfCells=\"" + std::to_string(nc) + "\">\n";
    s += "      <Points>\n";
    f.write(s.data(), s.size());
    std::vector<double> pos(3 * nn, 0.0);
    for (size_t n = 0; n < nn; ++n) F.node_xyz((int32_t)n, &pos[3 * n]);
    data_array(f, "Float64", "Position", 3, pos, binary);
    s = "      </Points>\n      <Cells>\n";
    f.write(s.data(), s.size());
    std::vector<int32_t> conn(F.nd->host().local_nodes.begin(), F.nd->host().local_nodes.end()), offs(nc);
    for (size_t c = 0; c < nc; ++c) offs[c] = (int32_t)(CH * (c + 1));
    std::vector<uint8_t> types(nc, (uint8_t)(D == 3 ? 11 : 8));  // VTK_VOXEL / VTK_PIXEL
    data_array(f, "Int32", "connectivity", 1, conn, binary);
    data_array(f, "Int32", "offsets", 1, offs, binary);
    data_array(f, "UInt8", "types", 1, types, binary);
    s = "      </Cells>\n";
    std::string plist, clist = write_tree ? "proc_rank, tree_idx" : "proc_rank";
    for (size_t k = 0; k < point_names.size(); ++k) plist += (k ? ", " : "") + point_names[k];
    for (const auto& c : cell_names) clist += ", " + c;
    s += "      <PointData Scalars=\"" + plist + "\">\n";
    f.write(s.data(), s.size());
    for (size_t k = 0; k < point_names.size(); ++k)
      data_array(f, "Float64", point_names[k].c_str(), 1, std::vector<double>(point_values[k], point_values[k] + nn), binary);
    s = "      </PointData>\n      <CellData Scalars=\"" + clist + "\">\n";
    f.write(s.data(), s.size());
    data_array(f, "Int32", "proc_rank", 1, std::vector<int32_t>(nc, 0), binary);
    if (write_tree) {
      std::vector<int32_t> tree(nc);
      for (size_t c = 0; c < nc; ++c) tree[c] = F.leaves[c].tree;
      data_array(f, "Int32", "tree_idx", 1, tree, binary);
    }
    for (size_t k = 0; k < cell_names.size(); ++k)
      data_array(f, "Float64", cell_names[k].c_str(), 1, std::vector<double>(cell_values[k], cell_values[k] + nc), binary);
    s = "      </CellData>\n    </Piece>\n  </UnstructuredGrid>\n</VTKFile>\n";
    f.write(s.data(), s.size());
    f.close();
  }
  File p(filename + ".pvtu", "wb");
  const char* fmt = binary ? "binary" : "ascii";
  std::string s = "<?xml version=\"1.0\"?>\n<VTKFile type=\"PUnstructuredGrid\" version=\"0.1\"";
  s += binary ? " header_type=\"UInt32\"" : "";
  s += " byte_order=\"LittleEndian\">\n  <PUnstructuredGrid GhostLevel=\"0\">\n    <PPoints>\n";
  s += std::string("      <PDataArray type=\"Float64\" Name=\"Position\" NumberOfComponents=\"3\" format=\"") + fmt + "\"/>\n";
  s += "    </PPoints>\n    <PPointData>\n";
  for (const auto& nme : point_names) s += "      <PDataArray type=\"Float64\" Name=\"" + nme + "\" format=\"" + fmt + "\"/>\n";
  s += "    </PPointData>\n    <PCellData>\n";
  s += std::string("      <PDataArray type=\"Int32\" Name=\"proc_rank\" format=\"") + fmt + "\"/>\n";
  if (write_tree) s += std::string("      <PDataArray type=\"Int32\" Name=\"tree_idx\" format=\"") + fmt + "\"/>\n";
  for (const auto& nme : cell_names) s += "      <PDataArray type=\"Float64\" Name=\"" + nme + "\" format=\"" + fmt + "\"/>\n";
  s += "    </PCellData>\n    <Piece Source=\"" + base_name(filename) + ".vtu/0000.vtu\"/>\n  </PUnstructuredGrid>\n</VTKFile>\n";
  p.write(s.data(), s.size());
  p.close();
}

void vec_dump(const std::string& fname, const std::vector<const double*>& vecs, int64_t n, bool int64_index) {
  File f(fname, "wb");
  for (const double* v : vecs) {
    std::vector<unsigned char> out;
    out.reserve(16 + (size_t)n * 8);
    put_be<int32_t>(out, VEC_FILE_CLASSID);
    if (int64_index)
      put_be<int64_t>(out, n);
    else
      put_be<int32_t>(out, (int32_t)n);
    for (int64_t i = 0; i < n; ++i) put_be<double>(out, v[i]);
    f.write(out.data(), out.size());
  }
  f.close();
}

void vec_load(const std::string& fname, const std::vector<double*>& vecs, int64_t n, bool int64_index) {
  File f(fname, "rb");
  for (double* v : vecs) {
    unsigned char h[12];
    const size_t hn = int64_index ? 12 : 8;
    f.read(h, hn);
    if (get_be<int32_t>(h) != VEC_FILE_CLASSID) throw std::invalid_argument("VecLoad: not a PETSc binary Vec record");
    const int64_t size = int64_index ? get_be<int64_t>(h + 4) : (int64_t)get_be<int32_t>(h + 4);
    if (size != n) throw std::invalid_argument("VecLoad: the stored vector has " + std::to_string(size) + " entries, expected " +
                                               std::to_string(n));
    std::vector<unsigned char> buf((size_t)n * 8);
    f.read(buf.data(), buf.size());
    for (int64_t i = 0; i < n; ++i) v[i] = get_be<double>(&buf[(size_t)i * 8]);
  }
}

static const char FOREST_MAGIC[8] = {'L', 'S', 'G', 'F', 'R', 'S', 'T', '1'};

template <int D>
void forest_save(const Forest<D>& F, const std::string& fname) {
  File f(fname, "wb");
  f.write(FOREST_MAGIC, 8);
  const int32_t dim = D;
  f.write(&dim, 4);
  f.write(F.brick.n, sizeof(int32_t) * 3);
  f.write(F.brick.xyz_min, sizeof(double) * 3);
  f.write(F.brick.xyz_max, sizeof(double) * 3);
  const int64_t nl = (int64_t)F.num_leaves();
  f.write(&nl, 8);
  std::vector<int32_t> rec((size_t)nl * 5);
  for (int64_t i = 0; i < nl; ++i) {
    const Quad& q = F.leaves[(size_t)i];
    rec[(size_t)i * 5 + 0] = q.tree;
    rec[(size_t)i * 5 + 1] = q.level;
    for (int a = 0; a < 3; ++a) rec[(size_t)i * 5 + 2 + a] = q.x[a];
  }
  f.write(rec.data(), rec.size() * 4);
  f.close();
}

// header of a forest file: dimension and brick
void forest_header(const std::string& fname, int* dim, int* n, double* lo, double* hi, int64_t* nleaves) {
  File f(fname, "rb");
  char magic[8];
  f.read(magic, 8);
  if (memcmp(magic, FOREST_MAGIC, 8) != 0) throw std::invalid_argument("not a forest file of this library: " + fname);
  int32_t d = 0;
  f.read(&d, 4);
  if (d != 2 && d != 3) throw std::invalid_argument("forest file: bad dimension");
  *dim = d;
  int32_t nn[3];
  f.read(nn, 12);
  for (int a = 0; a < 3; ++a) n[a] = nn[a];
  f.read(lo, 24);
  f.read(hi, 24);
  f.read(nleaves, 8);
}

template <int D>
void forest_load_leaves(Forest<D>& F, const std::string& fname) {
  int dim, n[3];
  double lo[3], hi[3];
  int64_t nl = 0;
  forest_header(fname, &dim, n, lo, hi, &nl);
  if (dim != D) throw std::invalid_argument("forest file: dimension mismatch");
  File f(fname, "rb");
  std::vector<unsigned char> skip(8 + 4 + 12 + 48 + 8);
  f.read(skip.data(), skip.size());
  std::vector<int32_t> rec((size_t)nl * 5);
  f.read(rec.data(), rec.size() * 4);
  std::vector<int32_t> tree((size_t)nl), level((size_t)nl), xyz((size_t)nl * 3);
  for (int64_t i = 0; i < nl; ++i) {
    tree[(size_t)i] = rec[(size_t)i * 5];
    level[(size_t)i] = rec[(size_t)i * 5 + 1];
    for (int a = 0; a < 3; ++a) xyz[(size_t)i * 3 + a] = rec[(size_t)i * 5 + 2 + a];
  }
  F.set_leaves((size_t)nl, tree.data(), level.data(), xyz.data());
}

#define LSG_INST(D)                                                                                                        \
  template void vtk_write_all<D>(const Forest<D>&, const std::string&, bool, const std::vector<std::string>&,              \
                                 const std::vector<const double*>&, const std::vector<std::string>&,                       \
                                 const std::vector<const double*>&, bool);                                                 \
  template void forest_save<D>(const Forest<D>&, const std::string&);                                                      \
  template void forest_load_leaves<D>(Forest<D>&, const std::string&);
LSG_INST(2)
LSG_INST(3)
#undef LSG_INST

}  // namespace lsg
