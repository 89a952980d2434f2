// meshio.cpp -- GiD mesh files (".msh"), the format of the reference's input
// meshes, read into the node / element arrays the library takes.
//
// Follows the reference's readers: Msh::CMesher2D::ReadFromFile_GiDMsh
// (src/msh/mesher2d.cpp:2463-2600) for triangles and
// Msh::CMesh3D::ReadFromFile_GiDMsh (src/msh/mesh3d.cpp:601-720) for
// tetrahedra.  Layout: a header line "MESH dimension <d> ElemType <type>
// Nnode <k>", "Coordinates", one "<id> <x> <y> [<z>]" line per node (ids
// 1..n in order), "end coordinates", "Elements", one "<id> <v1> .. <vk>" line
// per element (1-based node ids), "end elements".  Triangles given with three
// coordinates must lie in a coordinate plane: like the 2D reader, the axis of
// smallest variance is dropped (a mesh whose smallest variance exceeds 1e-4
// of the total is rejected) and the other two kept in the reader's cyclic
// order.  Only the P1 simplices of the hot path (Triangle, Tetrahedra) are
// accepted.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/dfg.h"

namespace dfg {
void set_noctx_error(const std::string& msg);
}

namespace {

struct GidMesh {
  int ndim = 0, nnoel = 0;
  std::vector<double> coords;  // nnode * ndim
  std::vector<int> conn;       // nelem * nnoel, 0-based
};

bool starts_with(const char* line, const char* word) {
  while (*line == ' ' || *line == '\t') ++line;
  return std::strncmp(line, word, std::strlen(word)) == 0;
}

bool blank(const char* line) {
  for (; *line; ++line)
    if (*line != ' ' && *line != '\t' && *line != '\r' && *line != '\n') return false;
  return true;
}

// Returns an empty string on success, the reason otherwise.
std::string read_gid(const char* path, GidMesh& M) {
  FILE* fp = std::fopen(path, "r");
  if (!fp) return std::string("cannot open ") + path;
  struct Closer {
    FILE* f;
    ~Closer() { std::fclose(f); }
  } closer{fp};
  char line[1024];
  if (!std::fgets(line, sizeof(line), fp)) return "empty file";
  char w1[64] = {0}, w2[64] = {0}, w3[64] = {0}, type[64] = {0}, w5[64] = {0};
  int fdim = 0, nnoel = 0;
  if (std::sscanf(line, "%63s %63s %d %63s %63s %63s %d", w1, w2, &fdim, w3, type, w5, &nnoel) != 7 ||
      std::strcmp(w1, "MESH") != 0)
    return "not a GiD mesh header";
  const bool tri = std::strcmp(type, "Triangle") == 0, tet = std::strcmp(type, "Tetrahedra") == 0;
  if (!tri && !tet) return std::string("element type ") + type + " is not a P1 triangle or tetrahedron";
  if ((tri && nnoel != 3) || (tet && nnoel != 4)) return "node count per element does not match the type";
  if (fdim != 2 && fdim != 3) return "dimension must be 2 or 3";
  if (tet && fdim != 3) return "tetrahedra need three coordinates";
  // nodes
  do {
    if (!std::fgets(line, sizeof(line), fp)) return "missing Coordinates";
  } while (blank(line));
  if (!starts_with(line, "Coordinates")) return "missing Coordinates";
  std::vector<double> xyz;
  for (long long id = 1;; ++id) {
    if (!std::fgets(line, sizeof(line), fp)) return "unterminated coordinates";
    if (starts_with(line, "end coordinates")) break;
    if (blank(line)) { --id; continue; }
    char* p = line;
    const long long got = std::strtoll(p, &p, 10);
    if (got != id) return "node ids must run 1..n in order";
    for (int d = 0; d < fdim; ++d) {
      char* q = p;
      xyz.push_back(std::strtod(p, &q));
      if (q == p) return "bad coordinate line";
      p = q;
    }
  }
  const long long nnode = (long long)xyz.size() / fdim;
  if (nnode == 0) return "no nodes";
  // elements
  do {
    if (!std::fgets(line, sizeof(line), fp)) return "missing Elements";
  } while (blank(line));
  if (!starts_with(line, "Elements")) return "missing Elements";
  for (long long id = 1;; ++id) {
    if (!std::fgets(line, sizeof(line), fp)) return "unterminated elements";
    if (starts_with(line, "end elements")) break;
    if (blank(line)) { --id; continue; }
    char* p = line;
    const long long got = std::strtoll(p, &p, 10);
    if (got != id) return "element ids must run 1..n in order";
    for (int k = 0; k < nnoel; ++k) {
      char* q = p;
      const long long v = std::strtoll(p, &q, 10);
      if (q == p || v < 1 || v > nnode) return "element node id out of range";
      M.conn.push_back((int)(v - 1));
      p = q;
    }
  }
  if (M.conn.empty()) return "no elements";
  M.nnoel = nnoel;
  if (tet || fdim == 2) {
    M.ndim = fdim;
    M.coords = std::move(xyz);
    return "";
  }
  // planar triangles in 3D: drop the axis of smallest variance (mesher2d.cpp:2497-2530)
  double a[3] = {0, 0, 0}, v[3] = {0, 0, 0};
  for (long long i = 0; i < nnode; ++i)
    for (int d = 0; d < 3; ++d) {
      const double c = xyz[(size_t)i * 3 + d];
      a[d] += c;
      v[d] += c * c;
    }
  for (int d = 0; d < 3; ++d) {
    v[d] /= (double)nnode;
    a[d] /= (double)nnode;
    v[d] -= a[d] * a[d];
  }
  int dmin = 0;
  double vmin = v[0];
  if (v[1] < vmin) { vmin = v[1]; dmin = 1; }
  if (v[2] < vmin) { vmin = v[2]; dmin = 2; }
  if (vmin > (v[0] + v[1] + v[2]) * 0.0001) return "triangle mesh is not planar in a coordinate plane";
  const int d0 = (dmin + 1) % 3, d1 = (dmin + 2) % 3;
  M.ndim = 2;
  M.coords.resize((size_t)nnode * 2);
  for (long long i = 0; i < nnode; ++i) {
    M.coords[(size_t)i * 2] = xyz[(size_t)i * 3 + d0];
    M.coords[(size_t)i * 2 + 1] = xyz[(size_t)i * 3 + d1];
  }
  return "";
}

}  // namespace

extern "C" int dfg_mesh_read_gid(const char* path, int* ndim, int* nnoel, int* nnode, int* nelem, double* coords,
                                 int* conn) {
  if (!path || !ndim || !nnoel || !nnode || !nelem) return DFG_INVALID_ARGUMENT;
  GidMesh M;
  const std::string err = read_gid(path, M);
  if (!err.empty()) {
    dfg::set_noctx_error("dfg_mesh_read_gid: " + err);
    return DFG_INVALID_ARGUMENT;
  }
  const long long nn = (long long)M.coords.size() / M.ndim, ne = (long long)M.conn.size() / M.nnoel;
  if (nn > 0x7fffffffLL || ne > 0x7fffffffLL) {
    dfg::set_noctx_error("dfg_mesh_read_gid: more than 2^31 nodes or elements");
    return DFG_INVALID_ARGUMENT;
  }
  *ndim = M.ndim;
  *nnoel = M.nnoel;
  *nnode = (int)nn;
  *nelem = (int)ne;
  if (coords) std::memcpy(coords, M.coords.data(), M.coords.size() * sizeof(double));
  if (conn) std::memcpy(conn, M.conn.data(), M.conn.size() * sizeof(int));
  return DFG_OK;
}
