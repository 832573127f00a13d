// wf_setup.cpp — host domain set-up: the reference's particle generators and
// zone assignment (src/Domain.cpp), used by the JSON driver and the C ABI.
//
// The generators reproduce the reference's floating-point sequence (running
// sums, not products) so that particle positions are bit-identical.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <array>
#include <map>
#include <string>
#include <vector>

#include "../../include/weldform_gb300.h"
#include "wf_setup.h"

namespace {
constexpr double kPi = 3.14159265358979323846;

// calcHalfPartCount (src/Domain.cpp:473-488): particles on one quadrant row
int half_count(double r, double R, int xinc) {
  int cnt = -1;
  if (xinc > 0) {
    cnt = 1;
    double yp = r;
    double xp = r + (double)(xinc - 1) * 2. * r;
    double rad = std::sqrt(yp * yp + xp * xp);
    while (rad <= R - r) {
      yp += 2. * r;
      rad = std::sqrt(yp * yp + xp * xp);
      cnt++;
    }
    cnt -= 1;
  }
  return cnt;
}

uint64_t splitmix64(uint64_t* s) {
  uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
double uniform01(uint64_t* s) { return (double)(splitmix64(s) >> 11) * (1.0 / 9007199254740992.0); }
}  // namespace

extern "C" {

// Domain::AddCylinderLength (src/Domain.cpp:490-573): layers of 2r pitch,
// each layer built row by row from the quadrant counts; mass = pi R^2 L rho / N.
int64_t wf_gen_cylinder(double x0, double y0, double z0, double Rxy, double Lz, double r,
                        double density, double* x, double* mass) {
  int64_t cnt = 0;
  const int nxy = half_count(r, Rxy, 1);
  double zp = z0 + r;
  while (zp <= (z0 + Lz - r)) {
    double yp = y0 - r - (2. * r * (nxy - 1));
    const int nyp = 2 * nxy;
    int yinc = nxy, sign = -1;
    for (int j = 0; j < nyp; j++) {
      const int nxp = half_count(r, Rxy, yinc);
      double xp = x0 - r - (2. * r * (nxp - 1));
      for (int i = 0; i < 2 * nxp; i++) {
        if (x) { x[3 * cnt] = xp; x[3 * cnt + 1] = yp; x[3 * cnt + 2] = zp; }
        cnt++;
        xp += 2. * r;
      }
      yp += 2. * r;
      yinc += sign;
      if (yinc < 1) { yinc = 1; sign = 1; }
    }
    zp += 2. * r;
  }
  const double vol = kPi * Rxy * Rxy * Lz;
  if (mass && cnt > 0) *mass = vol * density / (double)cnt;
  return cnt;
}

// Domain::AddBoxLength, cubic packing (src/Domain.cpp:296-338): mass from
// the bounding box of the generated centres grown by r.
int64_t wf_gen_box(double x0, double y0, double z0, double Lx, double Ly, double Lz, double r,
                   double density, double* x, double* mass) {
  int64_t cnt = 0;
  double mx[3] = {x0, y0, z0};
  size_t k = 0;
  double zp = z0;
  while (zp <= (z0 + Lz - r)) {
    size_t j = 0;
    double yp = y0;
    while (yp <= (y0 + Ly - r)) {
      size_t i = 0;
      double xp = x0;
      while (xp <= (x0 + Lx - r)) {
        const double px = x0 + (2.0 * i + 1) * r, py = y0 + (2.0 * j + 1) * r,
                     pz = z0 + (2.0 * k + 1) * r;
        if (x) { x[3 * cnt] = px; x[3 * cnt + 1] = py; x[3 * cnt + 2] = pz; }
        if (px > mx[0]) mx[0] = px;
        if (py > mx[1]) mx[1] = py;
        if (pz > mx[2]) mx[2] = pz;
        cnt++;
        i++;
        xp = x0 + (2 * i + 1) * r;
      }
      j++;
      yp = y0 + (2.0 * j + 1) * r;
    }
    k++;
    zp = z0 + (2.0 * k + 1) * r;
  }
  const double t0 = (mx[0] + r) - x0, t1 = (mx[1] + r) - y0, t2 = (mx[2] + r) - z0;
  if (mass && cnt > 0) *mass = t0 * t1 * t2 * density / (double)cnt;
  return cnt;
}

// Cubic lattice (spacing dx) clipped to a cylinder of radius R and height H
// (axis z, base z = 0), each coordinate jittered by U[-jitter, jitter]*dx
// from a splitmix64 stream seeded with `seed`.  The synthetic workload of
// the compression benchmarks.
int64_t wf_gen_cylinder_lattice(double R, double H, double dx, double jitter, uint64_t seed,
                                double* x) {
  int64_t cnt = 0;
  const int nxy = (int)std::floor(2.0 * R / dx + 0.5);
  const int nz = (int)std::floor(H / dx + 0.5);
  uint64_t st = seed;
  for (int k = 0; k < nz; k++)
    for (int j = 0; j < nxy; j++)
      for (int i = 0; i < nxy; i++) {
        const double px = (i + 0.5) * dx - R, py = (j + 0.5) * dx - R, pz = (k + 0.5) * dx;
        if (px * px + py * py > R * R) continue;
        if (x) {
          const double jx = (2.0 * uniform01(&st) - 1.0) * jitter * dx;
          const double jy = (2.0 * uniform01(&st) - 1.0) * jitter * dx;
          const double jz = (2.0 * uniform01(&st) - 1.0) * jitter * dx;
          x[3 * cnt] = px + jx; x[3 * cnt + 1] = py + jy; x[3 * cnt + 2] = pz + jz;
        }
        cnt++;
      }
  return cnt;
}

// Domain::AddCylUniformLength (src/Domain.cpp:1071-1192): rows at z = r,
// 3r, ... up to Lz - r; in each row, rings at radius r_i, r_i + 2r, ... < Rxy
// (running sums) of ceil(ang ri / 2r) particles ang / count apart (one at
// ri = 0).  Ids: `tag`; 2 / 3 on the first / last `rows` of a partial slice
// (ang < 2 pi); 4 within r/10 of the axis.  Every particle's mass is
// pi Rxy^2 Lz density / count.  Two-call protocol as wf_gen_cylinder.
int64_t wf_gen_cylinder_uniform(double Rxy, double Lz, double r, double density, double ang,
                                int rows, double r_i, int32_t tag, double* x, int32_t* ids,
                                double* mass) {
  if (!(r > 0.0) || !(Rxy > 0.0) || !(Lz > 0.0) || !(ang > 0.0)) return -1;
  const double z0 = r;
  int64_t cnt = 0;
  for (double zp = z0; zp <= z0 + Lz - r; zp += 2.0 * r) {
    for (double ri = r_i; ri < Rxy; ri += 2. * r) {
      int tg;
      double dalpha;
      if (ri == 0.) {
        tg = 1;
        dalpha = 0.;
      } else {
        tg = (int)ceil((ang * ri) / (2. * r));
        dalpha = ang / tg;
      }
      for (int a = 0; a < tg; a++) {
        int32_t id = tag;
        if (ang < 2.0 * kPi) {
          if (a < rows) id = 2;
          else if (a > tg - 1 - rows) id = 3;
        }
        const double xp = ri * cos(a * dalpha), yp = ri * sin(a * dalpha);
        if (std::fabs(xp) < r / 10 && std::fabs(yp) < r / 10) id = 4;
        if (x) { x[3 * cnt] = xp; x[3 * cnt + 1] = yp; x[3 * cnt + 2] = zp; }
        if (ids) ids[cnt] = id;
        cnt++;
      }
    }
  }
  if (mass && cnt > 0) *mass = kPi * Rxy * Rxy * Lz * density / (double)cnt;
  return cnt;
}

// Icosphere tool of radius R about `center` (the rigid indenter of the
// 2M-particle contact benchmark: the lower half of a ~10k-triangle sphere).
// The icosahedron's 20 faces are split `level` times into 4 (edge midpoints
// pushed to the sphere; shared midpoints created once, keyed by the edge's
// node pair); faces are ordered for outward normals.  lower_half keeps the
// faces whose centroid lies at or below center[2], and their nodes (renumbered
// in order of first use).  Two-call protocol: returns the face count and
// *n_nodes; fills nodes (3 n_nodes) and tris (3 per face) when not NULL.
int64_t wf_gen_icosphere(double R, const double* center, int level, int lower_half,
                         double* nodes, int32_t* tris, int64_t* n_nodes) {
  if (!(R > 0.0) || !center || level < 0 || level > 8) return -1;
  const double t = (1.0 + std::sqrt(5.0)) / 2.0;
  std::vector<double> v = {-1, t, 0, 1, t, 0, -1, -t, 0, 1, -t, 0, 0, -1, t, 0, 1, t,
                           0, -1, -t, 0, 1, -t, t, 0, -1, t, 0, 1, -t, 0, -1, -t, 0, 1};
  for (size_t k = 0; k < v.size(); k += 3) {
    const double s = 1.0 / std::sqrt(v[k] * v[k] + v[k + 1] * v[k + 1] + v[k + 2] * v[k + 2]);
    v[k] *= s; v[k + 1] *= s; v[k + 2] *= s;
  }
  std::vector<int32_t> f = {0, 11, 5, 0, 5, 1, 0, 1, 7, 0, 7, 10, 0, 10, 11, 1, 5, 9, 5, 11, 4,
                            11, 10, 2, 10, 7, 6, 7, 1, 8, 3, 9, 4, 3, 4, 2, 3, 2, 6, 3, 6, 8,
                            3, 8, 9, 4, 9, 5, 2, 4, 11, 6, 2, 10, 8, 6, 7, 9, 8, 1};
  for (int l = 0; l < level; l++) {
    std::map<std::pair<int32_t, int32_t>, int32_t> mid;
    auto midpoint = [&](int32_t a, int32_t b) {
      const std::pair<int32_t, int32_t> key(std::min(a, b), std::max(a, b));
      auto it = mid.find(key);
      if (it != mid.end()) return it->second;
      double p[3] = {0.5 * (v[3 * a] + v[3 * b]), 0.5 * (v[3 * a + 1] + v[3 * b + 1]),
                     0.5 * (v[3 * a + 2] + v[3 * b + 2])};
      const double s = 1.0 / std::sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
      const int32_t id = (int32_t)(v.size() / 3);
      v.push_back(p[0] * s); v.push_back(p[1] * s); v.push_back(p[2] * s);
      mid[key] = id;
      return id;
    };
    std::vector<int32_t> g;
    g.reserve(f.size() * 4);
    for (size_t k = 0; k < f.size(); k += 3) {
      const int32_t a = f[k], b = f[k + 1], c = f[k + 2];
      const int32_t ab = midpoint(a, b), bc = midpoint(b, c), ca = midpoint(c, a);
      const int32_t nf[12] = {a, ab, ca, b, bc, ab, c, ca, bc, ab, bc, ca};
      g.insert(g.end(), nf, nf + 12);
    }
    f.swap(g);
  }
  std::vector<int32_t> keep, remap(v.size() / 3, -1);
  int32_t nn = 0;
  for (size_t k = 0; k < f.size(); k += 3) {
    const double cz = (v[3 * f[k] + 2] + v[3 * f[k + 1] + 2] + v[3 * f[k + 2] + 2]) / 3.0;
    if (lower_half && cz > 0.0) continue;
    for (int q = 0; q < 3; q++) {
      if (remap[f[k + q]] < 0) remap[f[k + q]] = nn++;
      keep.push_back(remap[f[k + q]]);
    }
  }
  if (n_nodes) *n_nodes = nn;
  if (nodes)
    for (size_t q = 0; q < remap.size(); q++)
      if (remap[q] >= 0)
        for (int k = 0; k < 3; k++) nodes[3 * remap[q] + k] = center[k] + R * v[3 * q + k];
  if (tris) std::copy(keep.begin(), keep.end(), tris);
  return (int64_t)(keep.size() / 3);
}

// Domain::AssignZone (src/Domain.cpp:989-1005): inclusive box test.
int64_t wf_assign_zone(const double* x, int64_t n, const double* start, const double* end,
                       int32_t zone_id, int32_t* id, uint8_t* not_write) {
  int64_t cnt = 0;
  for (int64_t a = 0; a < n; a++) {
    bool inc = true;
    for (int c = 0; c < 3; c++)
      if (x[3 * a + c] < start[c] || x[3 * a + c] > end[c]) inc = false;
    if (inc) {
      id[a] = zone_id;
      if (not_write) not_write[a] = 1;
      cnt++;
    }
  }
  return cnt;
}

// NastranReader::read (src/NastranReader.cpp:5-150): fixed-field (8-character)
// GRID and CTRIA cards.  Nodes are the consecutive lines from the first GRID
// card (id in field 2, x y z in fields 4-6, implicit exponents); elements are
// the consecutive lines from the first CTRIA / CBEAM / CBAR card (node ids in
// fields 4-6, mapped to node positions).  Two-call protocol: NULL buffers
// return the element count and *n_nodes only.  Negative return: WF_ERR_IO
// (file), WF_ERR_ARG (beam elements, unknown node id).
int64_t wf_read_nastran(const char* path, double* nodes, int32_t* tris, int64_t* n_nodes) {
  if (!path) return WF_ERR_ARG;
  std::ifstream f(path);
  if (!f) return WF_ERR_IO;
  std::vector<std::string> lines;
  for (std::string l; std::getline(f, l);) lines.push_back(l);
  int64_t nn = 0, ne = 0, first_node = -1, first_elem = -1;
  bool beams = false;
  for (int64_t l = 0; l < (int64_t)lines.size(); l++) {
    const std::string& s = lines[l];
    if (s.compare(0, 4, "GRID") == 0) {
      if (first_node < 0) first_node = l;
      nn++;
    } else if (s.compare(0, 5, "CTRIA") == 0 || s.compare(0, 5, "CBEAM") == 0 ||
               s.compare(0, 4, "CBAR") == 0) {
      if (first_elem < 0) first_elem = l;
      if (s.compare(0, 5, "CTRIA") != 0) beams = true;
      ne++;
    }
  }
  if (beams) return WF_ERR_ARG;                       // dim = 2: not a triangle mesh
  if (n_nodes) *n_nodes = nn;
  if (!nodes && !tris) return ne;
  auto field = [](const std::string& s, int k) {
    const size_t p = 8 * (size_t)k;
    return p < s.size() ? s.substr(p, 8) : std::string();
  };
  // "0.7354-03" is 0.7354E-03: an exponent sign is the first '+', or the
  // first '-' that is not the field's leading sign
  auto real = [](std::string t) {
    size_t s = t.find('+');
    if (s != std::string::npos) {
      t.insert(s, "E");
    } else if ((s = t.find('-')) != std::string::npos) {
      if (s != 0) t.insert(s, "E");
      else if ((s = t.find('-', 1)) != std::string::npos) t.insert(s, "E");
    }
    return strtod(t.c_str(), nullptr);
  };
  std::map<int, int32_t> pos;
  for (int64_t q = 0; q < nn; q++) {
    const std::string& s = lines[first_node + q];
    pos[atoi(field(s, 1).c_str())] = (int32_t)q;
    for (int i = 0; i < 3; i++) {
      const double v = real(field(s, 3 + i));
      if (nodes) nodes[3 * q + i] = v;
    }
  }
  for (int64_t e = 0; e < ne; e++) {
    const std::string& s = lines[first_elem + e];
    for (int k = 0; k < 3; k++) {
      auto it = pos.find(atoi(field(s, 3 + k).c_str()));
      if (it == pos.end()) return WF_ERR_ARG;
      if (tris) tris[3 * e + k] = it->second;
    }
  }
  return ne;
}

// LS-DYNA keyword deck with SPH particles: Domain_d::ReadFromLSdyna
// (src/cuda/Domain_d.cu:236-281) reads it through the LSDynaReader submodule,
// which the reference tree does not carry; this reader follows the public
// keyword format.  One particle per *ELEMENT_SPH card, in card order, at its
// node's *NODE position, with the card's mass; a particle whose node is in a
// *SET_NODE_LIST takes that set's id (a later set wins), else 0.
namespace {
std::string trim(const std::string& t) {
  size_t a = t.find_first_not_of(" \t\r"), b = t.find_last_not_of(" \t\r");
  return a == std::string::npos ? std::string() : t.substr(a, b - a + 1);
}
// the fields of a data card: comma-separated (free format), else fixed widths
std::vector<std::string> card_fields(const std::string& line, const std::vector<int>& widths) {
  std::vector<std::string> f;
  if (line.find(',') != std::string::npos) {
    std::string cur;
    for (char c : line) {
      if (c == ',') { f.push_back(trim(cur)); cur.clear(); }
      else cur += c;
    }
    f.push_back(trim(cur));
    return f;
  }
  size_t p = 0;
  for (int w : widths) {
    f.push_back(p < line.size() ? trim(line.substr(p, (size_t)w)) : std::string());
    p += (size_t)w;
  }
  return f;
}
bool to_num(const std::string& t, double* v) {
  if (t.empty()) { *v = 0.0; return true; }
  char* e = nullptr;
  *v = strtod(t.c_str(), &e);
  return e && *e == '\0';
}
}  // namespace

int64_t wf_read_lsdyna(const char* path, double* x, double* mass, int32_t* ids) {
  if (!path) return WF_ERR_ARG;
  std::ifstream f(path);
  if (!f) return WF_ERR_IO;
  std::map<long long, std::array<double, 3>> node;
  std::vector<std::pair<long long, double>> sph;   // (node id, mass), card order
  std::vector<std::pair<long long, std::vector<long long>>> sets;
  enum { NONE, NODE, SPH, SET_CARD1, SET_NODES, SET_TITLE } sec = NONE;
  for (std::string line; std::getline(f, line);) {
    if (!line.empty() && line.back() == '\r') line.pop_back();
    if (line.empty() || line[0] == '$') continue;
    if (line[0] == '*') {
      std::string k = trim(line);
      for (char& c : k) c = (char)toupper((unsigned char)c);
      if (k == "*NODE") sec = NODE;
      else if (k == "*ELEMENT_SPH") sec = SPH;
      else if (k == "*SET_NODE_LIST") sec = SET_CARD1;
      else if (k == "*SET_NODE_LIST_TITLE") sec = SET_TITLE;
      else sec = NONE;
      continue;
    }
    double v[4];
    if (sec == NODE) {
      const auto fl = card_fields(line, {8, 16, 16, 16});
      if (fl.size() < 4 || !to_num(fl[0], &v[0]) || !to_num(fl[1], &v[1]) ||
          !to_num(fl[2], &v[2]) || !to_num(fl[3], &v[3]))
        return WF_ERR_IO;
      node[(long long)v[0]] = {v[1], v[2], v[3]};
    } else if (sec == SPH) {
      const auto fl = card_fields(line, {8, 8, 16});
      if (fl.size() < 3 || !to_num(fl[0], &v[0]) || !to_num(fl[2], &v[2])) return WF_ERR_IO;
      sph.push_back({(long long)v[0], v[2]});
    } else if (sec == SET_TITLE) {
      sec = SET_CARD1;                       // the title line
    } else if (sec == SET_CARD1) {
      const auto fl = card_fields(line, {10, 10, 10, 10, 10, 10});
      if (fl.empty() || !to_num(fl[0], &v[0])) return WF_ERR_IO;
      sets.push_back({(long long)v[0], {}});
      sec = SET_NODES;
    } else if (sec == SET_NODES) {
      const auto fl = card_fields(line, {10, 10, 10, 10, 10, 10, 10, 10});
      for (const std::string& t : fl) {
        if (t.empty()) continue;
        if (!to_num(t, &v[0])) return WF_ERR_IO;
        if (v[0] != 0.0) sets.back().second.push_back((long long)v[0]);
      }
    }
  }
  if (sph.empty()) return WF_ERR_ARG;
  const int64_t n = (int64_t)sph.size();
  for (const auto& e : sph)
    if (node.find(e.first) == node.end()) return WF_ERR_ARG;
  if (!x && !mass && !ids) return n;
  std::map<long long, int64_t> particle_of;    // node id -> particle index
  for (int64_t p = 0; p < n; p++) {
    auto it = node.find(sph[p].first);
    particle_of[sph[p].first] = p;
    if (x) for (int k = 0; k < 3; k++) x[3 * p + k] = it->second[k];
    if (mass) mass[p] = sph[p].second;
    if (ids) ids[p] = 0;
  }
  if (ids)
    for (const auto& st : sets)
      for (long long nid : st.second) {
        auto it = particle_of.find(nid);
        if (it != particle_of.end()) ids[it->second] = (int32_t)st.first;
      }
  return n;
}

// TriMesh_d::AxisPlaneMesh (src/cuda/Mesh.cu:48-194), the rigid plane main
// builds for a "Plane" body (src/WeldFormGPU.cu:545-552).  The reference
// steps both in-plane directions by dl = (p2.x - p1.x) / dens from p1 (x
// inner, y outer, running sums) at z = p1.z whatever the axis; the two
// triangles of a cell are ordered for an outward normal along +axis when
// `positive`, and the normals are set on the axis.
int64_t wf_gen_plane_mesh(int axis, int positive, const double* p1, const double* p2, int dens,
                          double* nodes, int32_t* tris, double* normals) {
  if (dens < 1 || axis < 0 || axis > 2 || !p1 || !p2) return -1;
  const int64_t ne = 2 * (int64_t)dens * dens;
  if (!nodes && !tris && !normals) return ne;
  const double dl = (p2[0] - p1[0]) / dens;
  const double z = p1[2];
  double y = p1[1];
  int64_t vi = 0;
  for (int j = 0; j <= dens; j++, y += dl) {
    double x = p1[0];
    for (int i = 0; i <= dens; i++, vi++, x += dl)
      if (nodes) { nodes[3 * vi] = x; nodes[3 * vi + 1] = y; nodes[3 * vi + 2] = z; }
  }
  int64_t el = 0;
  for (int j = 0; j < dens; j++)
    for (int i = 0; i < dens; i++) {
      const int32_t a = (dens + 1) * j + i, b = a + 1, c = (dens + 1) * (j + 1) + i, e = c + 1;
      const int32_t tri[2][3] = {{a, positive ? b : c, positive ? c : b},
                                 {b, positive ? e : c, positive ? c : e}};
      for (int t = 0; t < 2; t++, el++)
        if (tris) for (int q = 0; q < 3; q++) tris[3 * el + q] = tri[t][q];
    }
  if (normals)
    for (int64_t k = 0; k < ne; k++) {
      normals[3 * k] = normals[3 * k + 1] = normals[3 * k + 2] = 0.0;
      normals[3 * k + axis] = positive ? 1.0 : -1.0;
    }
  return ne;
}

}  // extern "C"
