/*
 * ref_nastran.cpp — the reference's Nastran reader (src/NastranReader.cpp),
 * compiled for the CPU to pin the library's reader.
 *
 * TEST INFRASTRUCTURE ONLY (oracle/_ref).  The parser is the reference's,
 * included from its source tree; this file only exposes its result.
 */
#include <cstdint>
#include <cstring>

#include "Vector.cpp"          /* Vector, used for the coordinate bounds */
#include "NastranReader.cpp"

namespace {
/* the parsed arrays are protected members; a derived class may read them */
struct Reader : SPH::NastranReader {
  explicit Reader(char* path) { read(path); }
  int nodes() const { return node_count; }
  int elems() const { return elem_count; }
  const double* node_xyz() const { return node; }
  const int* conn() const { return elcon; }
};
}  // namespace

extern "C" int64_t wfr_read_nastran(const char* path, double* nodes, int32_t* tris,
                                    int64_t* n_nodes) {
  std::string p(path);
  Reader r(&p[0]);
  if (n_nodes) *n_nodes = r.nodes();
  if (nodes) memcpy(nodes, r.node_xyz(), sizeof(double) * 3 * (size_t)r.nodes());
  if (tris)
    for (int64_t k = 0; k < 3 * (int64_t)r.elems(); k++) tris[k] = r.conn()[k];
  return r.elems();
}
