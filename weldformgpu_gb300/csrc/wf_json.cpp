// wf_json.cpp — the reference's input-file driver (src/WeldFormGPU.cu:142-926)
// on the library's C ABI: reads the same JSON keys, builds the particle
// domain with the reference's generators, sets it up as main does and runs
// MechFraserSolve, writing out_<time>.csv at the output times and test.csv at
// the end (the reference's column set, Domain_d::WriteCSV).
//
// A small JSON reader is included (objects, arrays, numbers, strings, true /
// false / null), enough for the reference's input files.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <utility>
#include <vector>

#include "../../include/weldform_gb300.h"

namespace {

struct Json {
  enum Kind { NUL, BOOL, NUM, STR, ARR, OBJ } kind = NUL;
  bool b = false;
  double num = 0.0;
  std::string str;
  std::vector<Json> arr;
  std::vector<std::pair<std::string, Json>> obj;

  const Json* get(const char* key) const {
    if (kind != OBJ) return nullptr;
    for (const auto& kv : obj)
      if (kv.first == key) return &kv.second;
    return nullptr;
  }
  const Json* at(size_t i) const { return kind == ARR && i < arr.size() ? &arr[i] : nullptr; }
};

class Parser {
 public:
  explicit Parser(const std::string& t) : s_(t) {}
  bool parse(Json& out, std::string& err) {
    if (!value(out) || (ws(), p_ != s_.size())) {
      err = "JSON syntax error near offset " + std::to_string(p_);
      return false;
    }
    return true;
  }

 private:
  const std::string& s_;
  size_t p_ = 0;
  void ws() {
    while (p_ < s_.size() && (s_[p_] == ' ' || s_[p_] == '\t' || s_[p_] == '\n' || s_[p_] == '\r'))
      p_++;
  }
  bool lit(const char* w) {
    const size_t n = strlen(w);
    if (s_.compare(p_, n, w) != 0) return false;
    p_ += n;
    return true;
  }
  bool string(std::string& out) {
    if (p_ >= s_.size() || s_[p_] != '"') return false;
    p_++;
    while (p_ < s_.size() && s_[p_] != '"') {
      char c = s_[p_++];
      if (c == '\\' && p_ < s_.size()) {
        const char e = s_[p_++];
        c = e == 'n' ? '\n' : e == 't' ? '\t' : e;
      }
      out.push_back(c);
    }
    if (p_ >= s_.size()) return false;
    p_++;
    return true;
  }
  bool value(Json& v) {
    ws();
    if (p_ >= s_.size()) return false;
    const char c = s_[p_];
    if (c == '{') {
      v.kind = Json::OBJ;
      p_++;
      ws();
      if (p_ < s_.size() && s_[p_] == '}') { p_++; return true; }
      while (true) {
        ws();
        std::string key;
        if (!string(key)) return false;
        ws();
        if (p_ >= s_.size() || s_[p_] != ':') return false;
        p_++;
        Json item;
        if (!value(item)) return false;
        v.obj.emplace_back(std::move(key), std::move(item));
        ws();
        if (p_ < s_.size() && s_[p_] == ',') { p_++; continue; }
        if (p_ < s_.size() && s_[p_] == '}') { p_++; return true; }
        return false;
      }
    }
    if (c == '[') {
      v.kind = Json::ARR;
      p_++;
      ws();
      if (p_ < s_.size() && s_[p_] == ']') { p_++; return true; }
      while (true) {
        Json item;
        if (!value(item)) return false;
        v.arr.push_back(std::move(item));
        ws();
        if (p_ < s_.size() && s_[p_] == ',') { p_++; continue; }
        if (p_ < s_.size() && s_[p_] == ']') { p_++; return true; }
        return false;
      }
    }
    if (c == '"') { v.kind = Json::STR; return string(v.str); }
    if (lit("true")) { v.kind = Json::BOOL; v.b = true; return true; }
    if (lit("false")) { v.kind = Json::BOOL; v.b = false; return true; }
    if (lit("null")) { v.kind = Json::NUL; return true; }
    const char* b = s_.c_str() + p_;
    char* e = nullptr;
    v.num = strtod(b, &e);
    if (e == b) return false;
    v.kind = Json::NUM;
    p_ += (size_t)(e - b);
    return true;
  }
};

// readValue / readVector / readArray of the reference (src/WeldFormGPU.cu:20-50):
// a missing key keeps the default
bool read_num(const Json* o, const char* k, double& out) {
  const Json* v = o ? o->get(k) : nullptr;
  if (!v) return false;
  if (v->kind == Json::NUM) { out = v->num; return true; }
  if (v->kind == Json::BOOL) { out = v->b ? 1.0 : 0.0; return true; }
  return false;
}
bool read_int(const Json* o, const char* k, int& out) {
  double d;
  if (!read_num(o, k, d)) return false;
  out = (int)d;
  return true;
}
bool read_str(const Json* o, const char* k, std::string& out) {
  const Json* v = o ? o->get(k) : nullptr;
  if (!v || v->kind != Json::STR) return false;
  out = v->str;
  return true;
}
bool read_vec3(const Json* o, const char* k, double out[3]) {
  const Json* v = o ? o->get(k) : nullptr;
  if (!v || v->kind != Json::ARR || v->arr.size() < 3) return false;
  for (int i = 0; i < 3; i++) out[i] = v->arr[i].kind == Json::NUM ? v->arr[i].num : 0.0;
  return true;
}
std::vector<double> read_array(const Json* o, const char* k) {
  std::vector<double> r;
  const Json* v = o ? o->get(k) : nullptr;
  if (v && v->kind == Json::ARR)
    for (const Json& x : v->arr) r.push_back(x.kind == Json::NUM ? x.num : 0.0);
  return r;
}

}  // namespace

namespace {

struct Run {
  std::string err;
  int code = WF_OK;
  bool fail(int c, const std::string& m) {
    code = c;
    err = m;
    return false;
  }
};

bool read_file(const char* path, std::string& out) {
  std::ifstream f(path, std::ios::binary);
  if (!f) return false;
  std::ostringstream ss;
  ss << f.rdbuf();
  out = ss.str();
  return true;
}

// one ABI call; on failure records the library's message
bool ok(Run& run, wf_domain* d, int rc, const char* what) {
  if (rc == WF_OK) return true;
  return run.fail(rc, std::string(what) + ": " + (d ? wf_last_error(d) : "failed"));
}

struct Bc {
  int zone;
  double v[3];
};

bool run_input(const Json& root, const std::string& out_dir, const std::string& json_dir,
               Run& run) {
  const Json* config = root.get("Configuration");
  const Json* materials = root.get("Materials");
  const Json* domblock = root.get("DomainBlocks");
  const Json* zones = root.get("DomainZones");
  const Json* rigid = root.get("RigidBodies");
  const Json* contact = root.get("Contact");
  const Json* bcs = root.get("BoundaryConditions");
  const Json* ics = root.get("InitialConditions");
  // Configuration (src/WeldFormGPU.cu:205-270)
  double r = 0.0, hfactor = 0.0, sim_time = 0.0, out_time = 0.0;
  read_num(config, "particleRadius", r);
  read_num(config, "hFactor", hfactor);
  read_num(config, "simTime", sim_time);
  read_num(config, "outTime", out_time);
  if (!(r > 0.0) || !(hfactor > 0.0) || !(sim_time > 0.0) || !(out_time > 0.0))
    return run.fail(WF_ERR_ARG, "Configuration needs particleRadius, hFactor, simTime, outTime > 0");
  // Materials[0] (:215-240, :749-800)
  const Json* mat0 = materials ? materials->at(0) : nullptr;
  if (!mat0) return run.fail(WF_ERR_ARG, "no Materials entry");
  std::string mattype = "Bilinear";
  read_str(mat0, "type", mattype);
  double rho = 0.0, E = 0.0, nu = 0.0, Fy = 0.0;
  const bool has_fy = read_num(mat0, "yieldStress0", Fy);
  read_num(mat0, "density0", rho);
  read_num(mat0, "youngsModulus", E);
  read_num(mat0, "poissonsRatio", nu);
  const std::vector<double> c = read_array(mat0, "const");
  if (!(rho > 0.0) || !(E > 0.0)) return run.fail(WF_ERR_ARG, "material density0 / youngsModulus");
  const double K = E / (3. * (1. - 2 * nu));
  const double G = E / (2. * (1. + nu));
  const double dx = 2. * r;
  const double h = dx * hfactor;
  const double Cs = std::sqrt(K / rho);
  wf_material mat{};
  mat.E = E;
  mat.nu = nu;
  if (mattype == "Bilinear") {
    if (c.empty()) return run.fail(WF_ERR_ARG, "Bilinear needs const[0] = tangent modulus");
    mat.model = WF_BILINEAR;
    mat.Et = c[0];
    mat.sy0 = Fy;
  } else if (mattype == "JohnsonCook") {
    if (c.size() < 8) return run.fail(WF_ERR_ARG, "JohnsonCook needs const[0..7]");
    mat.model = WF_JOHNSON_COOK;
    mat.A = c[0]; mat.B = c[1]; mat.n = c[2]; mat.C = c[3];
    mat.eps0 = c[4]; mat.m = c[5]; mat.Tm = c[6]; mat.Tt = c[7];
    // the reference evaluates the JC law at T = 0 here (:792), which is NaN
    // for T_t > 0; the initial yield stress is yieldStress0, else A
    if (!has_fy) Fy = mat.A;
    mat.sy0 = Fy;
  } else if (mattype == "Hollomon") {
    if (c.size() < 2) return run.fail(WF_ERR_ARG, "Hollomon needs const[0..1]");
    mat.model = WF_HOLLOMON;
    mat.K_hol = c[0];
    mat.m_hol = c[1];
    mat.sy0 = Fy;
  } else {
    return run.fail(WF_ERR_ARG, "material type must be Bilinear, JohnsonCook or Hollomon");
  }
  // DomainBlocks[0] (:300-395)
  const Json* db = domblock ? domblock->at(0) : nullptr;
  if (!db) return run.fail(WF_ERR_ARG, "no DomainBlocks entry");
  std::string domtype = "Box", grid = "Cartesian";
  double start[3] = {0, 0, 0}, L[3] = {0, 0, 0};
  read_str(db, "type", domtype);
  read_str(db, "gridCoordSys", grid);
  read_vec3(db, "start", start);
  read_vec3(db, "dim", L);
  std::vector<double> x;
  std::vector<int32_t> gen_ids;
  std::vector<double> masses;              // per particle (a particle file), else `mass`
  double mass = 0.0;
  int64_t ns = 0;
  double slice = 2.0000001 * 3.14159265358979323846;   // the reference's default (:307)
  read_num(db, "sliceAngle", slice);
  if (domtype == "Cylinder" && grid == "Cylindrical") {
    // AddCylUniformLength (:336-349): the full cylinder when sliceAngle is
    // exactly 2 pi; any other angle is main's axisymmetric slice, not built
    if (slice != 2.0 * 3.14159265358979323846)
      return run.fail(WF_ERR_ARG, "axisymmetric slices (sliceAngle != 2 pi) are not supported");
    ns = wf_gen_cylinder_uniform(L[0] / 2.0, L[2], r, rho, slice, 1, 0.0, 0, nullptr, nullptr,
                                 &mass);
    if (ns <= 0) return run.fail(WF_ERR_ARG, "the domain block holds no particles");
    x.resize(3 * (size_t)ns);
    gen_ids.resize((size_t)ns);
    wf_gen_cylinder_uniform(L[0] / 2.0, L[2], r, rho, slice, 1, 0.0, 0, x.data(), gen_ids.data(),
                            &mass);
  } else if (domtype == "Cylinder") {
    if (grid != "Cartesian") return run.fail(WF_ERR_ARG, "gridCoordSys must be Cartesian or Cylindrical");
    ns = wf_gen_cylinder(start[0], start[1], start[2], L[0] / 2., L[2], r, rho, nullptr, &mass);
    x.resize(3 * (size_t)ns);
    wf_gen_cylinder(start[0], start[1], start[2], L[0] / 2., L[2], r, rho, x.data(), &mass);
  } else if (domtype == "Box") {
    ns = wf_gen_box(start[0], start[1], start[2], L[0], L[1], L[2], r, rho, nullptr, &mass);
    x.resize(3 * (size_t)ns);
    wf_gen_box(start[0], start[1], start[2], L[0], L[1], L[2], r, rho, x.data(), &mass);
  } else if (domtype == "File") {
    // particles from an LS-DYNA keyword deck (:378-398, Domain_d::ReadFromLSdyna)
    std::string fname;
    read_str(db, "fileName", fname);
    if (fname.empty()) return run.fail(WF_ERR_ARG, "a File domain block needs fileName");
    std::string path = fname;               // as given, else beside the input file
    if (!std::ifstream(path) && !json_dir.empty()) path = json_dir + "/" + fname;
    ns = wf_read_lsdyna(path.c_str(), nullptr, nullptr, nullptr);
    if (ns == WF_ERR_IO) return run.fail(WF_ERR_IO, "cannot read particle file " + path);
    if (ns <= 0) return run.fail(WF_ERR_ARG, "no SPH particles (or an unknown node) in " + path);
    x.resize(3 * (size_t)ns);
    masses.resize((size_t)ns);
    gen_ids.resize((size_t)ns);
    wf_read_lsdyna(path.c_str(), x.data(), masses.data(), gen_ids.data());
  } else {
    return run.fail(WF_ERR_ARG, "domain type must be Box, Cylinder or File");
  }
  if (ns <= 0) return run.fail(WF_ERR_ARG, "the domain block holds no particles");
  // DomainZones (:396-412); main then protects every zoned particle (:851-858)
  std::vector<int32_t> ids = gen_ids.empty() ? std::vector<int32_t>((size_t)ns, 0) : gen_ids;
  std::vector<uint8_t> nw((size_t)ns, 0);
  if (zones && zones->kind == Json::ARR)
    for (const Json& z : zones->arr) {
      int zid = 0;
      double zs[3] = {0, 0, 0}, ze[3] = {0, 0, 0};
      read_int(&z, "id", zid);
      read_vec3(&z, "start", zs);
      read_vec3(&z, "end", ze);
      wf_assign_zone(x.data(), ns, zs, ze, zid, ids.data(), nullptr);
    }
  for (int64_t i = 0; i < ns; i++) nw[i] = ids[i] != 0;
  // BoundaryConditions (:457-485): constant velocities
  std::vector<Bc> bclist;
  if (bcs && bcs->kind == Json::ARR)
    for (const Json& b : bcs->arr) {
      Bc bc{0, {0, 0, 0}};
      int vt = 0;
      read_int(&b, "zoneId", bc.zone);
      read_int(&b, "valueType", vt);
      if (vt != 0) return run.fail(WF_ERR_ARG, "amplitude boundary conditions are not supported");
      read_vec3(&b, "value", bc.v);
      bclist.push_back(bc);
    }
  // RigidBodies[0] + Contact[0] (:417-440, :498-645)
  const Json* rb = rigid ? rigid->at(0) : nullptr;
  std::string rbtype;
  const bool has_contact = read_str(rb, "type", rbtype);
  std::vector<double> nodes, normals;
  std::vector<int32_t> tris;
  int64_t ne = 0;
  int rzone = 0;
  double mu_s = 0.0, mu_d = 0.0, contact_law = 0.0;
  if (has_contact) {
    double rs[3] = {0, 0, 0}, rd[3] = {0, 0, 0};
    int dens = 10;
    read_vec3(rb, "start", rs);
    read_vec3(rb, "dim", rd);
    read_int(rb, "partSide", dens);
    read_int(rb, "zoneId", rzone);
    if (rbtype == "Plane") {
      const double p2[3] = {rs[0] + rd[0], rs[1] + rd[1], rs[2]};
      ne = wf_gen_plane_mesh(2, 0, rs, p2, dens, nullptr, nullptr, nullptr);
      if (ne <= 0) return run.fail(WF_ERR_ARG, "rigid plane partSide");
      nodes.resize(3 * (size_t)(dens + 1) * (dens + 1));
      tris.resize(3 * (size_t)ne);
      normals.resize(3 * (size_t)ne);
      wf_gen_plane_mesh(2, 0, rs, p2, dens, nodes.data(), tris.data(), normals.data());
    } else if (rbtype == "File") {
      // Nastran mesh (:553-566); the file is looked up as given, then beside
      // the input file.  moveDir moves the mesh (the reference moves only its
      // host copy, so its rigid particles and contact geometry disagree).
      std::string fname;
      read_str(rb, "fileName", fname);
      std::string path = fname;
      if (!std::ifstream(path) && !json_dir.empty()) path = json_dir + "/" + fname;
      double md[3] = {0, 0, 0};
      read_vec3(rb, "moveDir", md);
      int64_t nn = 0;
      ne = wf_read_nastran(path.c_str(), nullptr, nullptr, &nn);
      if (ne <= 0) return run.fail(ne < 0 ? (int)ne : WF_ERR_ARG, "cannot read mesh " + fname);
      nodes.resize(3 * (size_t)nn);
      tris.resize(3 * (size_t)ne);
      wf_read_nastran(path.c_str(), nodes.data(), tris.data(), &nn);
      for (int64_t q = 0; q < nn; q++)
        for (int k = 0; k < 3; k++) nodes[3 * q + k] += md[k];
    } else {
      return run.fail(WF_ERR_ARG, "rigid body type must be Plane or File");
    }
    const Json* ct = contact ? contact->at(0) : nullptr;
    read_num(ct, "fricCoeffStatic", mu_s);
    read_num(ct, "fricCoeffDynamic", mu_d);
    // extension: "law": 1 selects the binned nearest-triangle law (contact_dx =
    // the particle spacing 2 r)
    read_num(ct, "law", contact_law);
    if (contact_law != 0.0 && contact_law != 1.0)
      return run.fail(WF_ERR_ARG, "Contact law must be 0 or 1");
  }
  const int64_t n = ns + ne;
  // initial temperature (InitialConditions[0].Temp; main leaves T unset)
  double T0 = 20.0;
  read_num(ics ? ics->at(0) : nullptr, "Temp", T0);
  // set-up through the C ABI, in main's order (:689-870)
  wf_domain* d = nullptr;
  if (!ok(run, nullptr, wf_create(&d, n), "wf_create")) return false;
  struct Guard { wf_domain* d; ~Guard() { wf_destroy(d); } } guard{d};
  std::vector<double> xa(3 * (size_t)n, 0.0), ma((size_t)n, 0.0), cs((size_t)n, Cs),
      Ta((size_t)n, T0);
  std::vector<int32_t> ida((size_t)n, rzone);
  std::vector<uint8_t> nwa((size_t)n, 0), fr((size_t)n, 1);
  for (int64_t i = 0; i < ns; i++) {
    for (int k = 0; k < 3; k++) xa[3 * i + k] = x[3 * i + k];
    ma[i] = masses.empty() ? mass : masses[i];
    ida[i] = ids[i];
    nwa[i] = nw[i];
  }
  const double dt = 0.4 * h / (Cs + 10.0);           // VMAX = 10, :906
  if (!ok(run, d, wf_set_solid_count(d, ns), "solid count") ||
      !ok(run, d, wf_set_material(d, &mat), "material") ||
      !ok(run, d, wf_set_density(d, rho), "SetDensity") ||
      !ok(run, d, wf_set_h(d, h), "Set_h") ||
      !ok(run, d, wf_set_positions(d, xa.data()), "positions") ||
      !ok(run, d, wf_set_mass(d, ma.data()), "masses") ||
      !ok(run, d, wf_set_shear_modulus(d, G), "SetShearModulus") ||
      !ok(run, d, wf_set_free(d, fr.data()), "SetFreePart") ||
      !ok(run, d, wf_set_id(d, ida.data()), "SetID") ||
      !ok(run, d, wf_set_cs(d, cs.data()), "SetCs") ||
      !ok(run, d, wf_set_sigma_y(d, Fy), "SetSigmay") ||
      !ok(run, d, wf_set_not_write_surf_id(d, nwa.data()), "not_write_surf_ID") ||
      !ok(run, d, wf_set_temperature(d, Ta.data()), "temperature") ||
      !ok(run, d, wf_set_time_step(d, dt), "time step"))
    return false;
  double mesh_v[3] = {0, 0, 0};
  for (const Bc& b : bclist) {
    if (!ok(run, d, wf_add_velocity_bc(d, b.zone, b.v[0], b.v[1], b.v[2]), "BC")) return false;
    if (has_contact && b.zone == rzone)
      for (int k = 0; k < 3; k++) mesh_v[k] = b.v[k];   // SetMeshVelKernel, :598-607
  }
  if (has_contact) {
    const double w[3] = {0, 0, 0};
    if (!ok(run, d, wf_add_trimesh(d, nodes.data(), (int32_t)(nodes.size() / 3), tris.data(),
                                   (int32_t)ne, normals.empty() ? nullptr : normals.data(),
                                   rzone, ns, mesh_v, w),
            "rigid plane") ||
        !ok(run, d, wf_set_contact(d, mu_s, mu_d, (int)contact_law), "contact"))
      return false;
    if (contact_law == 1.0 && !ok(run, d, wf_set_option(d, "contact_dx", 2.0 * r), "contact law 1"))
      return false;
  }
  // options the reference has no key for (documented extensions)
  std::string s;
  if (read_str(config, "precision", s) &&
      !ok(run, d, wf_set_option(d, "precision", s == "mixed" ? 1.0 : 0.0), "precision"))
    return false;
  double rb_inc = 0.0;
  if (read_num(config, "rebuildStrainIncrement", rb_inc) &&
      !ok(run, d, wf_set_option(d, "rebuild_strain_increment", rb_inc), "rebuildStrainIncrement"))
    return false;
  if (read_str(config, "returnMap", s) &&
      !ok(run, d, wf_set_option(d, "return_map", s == "newton" ? 1.0 : 0.0), "returnMap"))
    return false;
  if (read_str(config, "solver", s) && s == "Mech-Thermal") {
    double k = 0.0, cp = 0.0, chi = 0.0;
    read_num(mat0, "thermalCond", k);
    read_num(mat0, "thermalHeatCap", cp);
    read_num(config, "taylorQuinney", chi);
    if (!ok(run, d, wf_set_conductivity(d, k), "thermalCond") ||
        !ok(run, d, wf_set_heat_cap(d, cp), "thermalHeatCap") ||
        !ok(run, d, wf_set_option(d, "thermal", 1.0), "thermal") ||
        !ok(run, d, wf_set_option(d, "taylor_quinney", chi), "taylorQuinney"))
      return false;
  }
  const std::string prefix = out_dir.empty() ? std::string() : out_dir + "/";
  if (!ok(run, d, wf_set_csv_output(d, prefix.c_str()), "CSV output") ||
      !ok(run, d, wf_mech_fraser_solve(d, sim_time, out_time), "MechFraserSolve") ||
      !ok(run, d, wf_write_csv(d, (prefix + "test.csv").c_str()), "WriteCSV"))
    return false;
  return true;
}

}  // namespace

extern "C" int wf_run_json(const char* path, const char* out_dir, char* err, int64_t err_len) {
  Run run;
  std::string text;
  Json root;
  if (!path) {
    run.fail(WF_ERR_ARG, "no input file");
  } else if (!read_file(path, text)) {
    run.fail(WF_ERR_IO, std::string("cannot read ") + path);
  } else {
    Parser p(text);
    std::string perr;
    if (!p.parse(root, perr)) run.fail(WF_ERR_IO, perr);
    else {
      const std::string p(path);
      const size_t slash = p.find_last_of('/');
      run_input(root, out_dir ? out_dir : "", slash == std::string::npos ? "" : p.substr(0, slash),
                run);
    }
  }
  if (err && err_len > 0) snprintf(err, (size_t)err_len, "%s", run.err.c_str());
  return run.code;
}
