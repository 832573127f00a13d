/*
 * ref_domain.cpp — runs the reference's own Domain_d kernels on the CPU.
 *
 * TEST INFRASTRUCTURE ONLY: compiled by oracle/build_ref.py into
 * oracle/_ref/ from the sources under the reference tree; never shipped.
 *
 * The member functions called here (CalcDensInc, UpdateDensity,
 * CalcRateTensors, StressStrainOne, CalcAccel, ApplyBCVel, UpdatePosFraser,
 * UpdateVel, CalcIntEnergy) and the kernels PressureKernelExt,
 * ThermalSolveKernel, CalcConvHeatKernel and TempCalcLeapfrog[First] are the
 * reference's, included verbatim from src/cuda/.  This file only allocates
 * the Domain_d arrays on the host, runs each kernel as a sequential loop
 * over its thread index, and calls them in MechFraserSolve's order
 * (src/cuda/SolverFraser.cu:164-398).  Arrays the reference leaves
 * uninitialised are set to the values the oracle assumes: PresEq = P0 = 0,
 * FPMassC = 1, NoSlip = false.
 */
#include <array>
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <fcntl.h>
#include <iostream>
#include <unistd.h>
#include <vector>

#include "cuda_host_shim.h"
#include "cuda_helper.h"
#include "Domain_d.cuh"
#include "Functions.cuh"
#include "Mechanical.cu"
#include "InteractionAlt.cu"
#include "Energy.cu"   /* Mechanical.cu brings Geometry.cu, Contact.cu and Mesh.cu */
/* Thermal.cu's four kernels, extracted verbatim by oracle/build_ref.py into the
 * build directory (the file's host functions launch kernels with <<< >>>,
 * which a host compiler cannot parse) */
#include "thermal_kernels.inc"

using namespace SPH;

extern "C" int wfr_neighbors(const double* x, int64_t n, double h_glob, int32_t* counts,
                             int32_t* lists);

namespace {

struct RefDom {
  Domain_d* dom;
  Material_* mat;
  int64_t n, n_solid;
  std::vector<uint> nbc, nbo, nbl;
  std::vector<int> bc_zone;
  std::vector<double3> bc_v;
  double3* x_h;
  int ts_i, is_yielding, rebuild_every;
  double max_pl_strain, time;
};

template <class T>
T* alloc(int64_t n) {
  T* p = (T*)calloc((size_t)(n > 0 ? n : 1), sizeof(T));
  return p;
}

template <class F>
void launch_seq(int64_t n, F&& f) {
  blockDim = dim3(1, 1, 1);
  blockIdx = make_uint3(0, 0, 0);
  for (int64_t t = 0; t < n; t++) {
    threadIdx = make_uint3((unsigned)t, 0, 0);
    f();
  }
}

/* the bilinear branch printf()s per yielding particle (Mechanical.cu:523,534) */
struct Quiet {
  int saved;
  Quiet() {
    fflush(stdout);
    saved = dup(1);
    int nul = open("/dev/null", O_WRONLY);
    dup2(nul, 1);
    close(nul);
  }
  ~Quiet() {
    fflush(stdout);
    dup2(saved, 1);
    close(saved);
  }
};

void rebuild(RefDom* r, const double3* pos) {
  std::vector<int32_t> cnt(r->n), lst((size_t)r->n * 70);
  wfr_neighbors((const double*)pos, r->n, r->dom->h_glob, cnt.data(), lst.data());
  r->nbc.assign(r->n, 0);
  r->nbo.assign(r->n, 0);
  r->nbl.clear();
  for (int64_t i = 0; i < r->n; i++) {
    r->nbc[i] = (uint)cnt[i];
    r->nbo[i] = (uint)r->nbl.size();
    for (int k = 0; k < cnt[i]; k++) r->nbl.push_back((uint)lst[(size_t)i * 70 + k]);
  }
  if (r->nbl.empty()) r->nbl.push_back(0);
}

}  // namespace

thread_local uint3 threadIdx;
thread_local uint3 blockIdx;
thread_local dim3 blockDim;

extern "C" {

void* wfr_create(int64_t n) {
  RefDom* r = new RefDom();
  r->n = n;
  r->n_solid = n;
  Domain_d* d = (Domain_d*)calloc(1, sizeof(Domain_d));   /* like cudaMallocManaged: no ctor */
  r->dom = d;
  d->particle_count = (int)n;
  d->solid_part_count = (int)n;
  d->x = alloc<double3>(n); d->v = alloc<double3>(n); d->a = alloc<double3>(n);
  d->u = alloc<double3>(n); d->va = alloc<double3>(n); d->NSv = alloc<double3>(n);
  d->VXSPH = alloc<double3>(n); d->normal = alloc<double3>(n); d->contforce = alloc<double3>(n);
  d->h = alloc<double>(n); d->m = alloc<double>(n); d->rho = alloc<double>(n);
  d->rho_0 = alloc<double>(n); d->p = alloc<double>(n); d->PresEq = alloc<double>(n);
  d->Cs = alloc<double>(n); d->P0 = alloc<double>(n); d->FPMassC = alloc<double>(n);
  d->G = alloc<double>(n); d->drho = alloc<double>(n);
  d->sigma = alloc<double>(6 * n); d->strrate = alloc<double>(6 * n);
  d->rotrate = alloc<double>(6 * n); d->shearstress = alloc<double>(6 * n);
  d->strain = alloc<double>(6 * n);
  d->sigma_eq = alloc<double>(n); d->pl_strain = alloc<double>(n); d->sigma_y = alloc<double>(n);
  d->eff_strain_rate = alloc<double>(n); d->int_energy = alloc<double>(n);
  d->T = alloc<double>(n);
  d->Ta = alloc<double>(n); d->Tb = alloc<double>(n); d->dTdt = alloc<double>(n);
  d->k_T = alloc<double>(n); d->cp_T = alloc<double>(n); d->BC_T = alloc<int>(n);
  d->IsFree = alloc<bool>(n); d->NoSlip = alloc<bool>(n); d->ID = alloc<int>(n);
  /* contact arrays (WeldFormGPU.cu:503-511, Domain_d.cu:160-170) */
  d->not_write_surf_ID = alloc<bool>(n);
  d->contneib_count = alloc<int>(n); d->contneib_part = alloc<int>(20 * n + 20);
  d->mesh_id = alloc<int>(n);
  d->contact_surf_id = alloc<int>(8); d->first_fem_particle_idx = alloc<int>(8);
  d->trimesh = alloc<TriMesh_d*>(8);
  d->mat = alloc<Material_*>(n);
  for (int64_t i = 0; i < n; i++) { d->IsFree[i] = true; d->FPMassC[i] = 1.0; }
  d->Alpha = 1.0;    /* SetDimension, Domain_d.cu:191-192 */
  d->Beta = 0.0;
  d->contact = false;
  d->trimesh_count = 0;
  r->mat = new Material_(Elastic_(1.0, 0.3));
  r->mat->Material_model = BILINEAR;
  r->mat->Et = 0.0;
  d->materials = r->mat;
  for (int64_t i = 0; i < n; i++) d->mat[i] = r->mat;
  r->x_h = alloc<double3>(n);
  r->rebuild_every = 5;
  r->ts_i = 0; r->is_yielding = 0; r->max_pl_strain = 0.0; r->time = 0.0;
  return r;
}

void wfr_destroy(void* h) {
  RefDom* r = (RefDom*)h;
  if (!r) return;
  Domain_d* d = r->dom;
  void* ptrs[] = {d->x, d->v, d->a, d->u, d->va, d->NSv, d->VXSPH, d->normal, d->contforce,
                  d->h, d->m, d->rho, d->rho_0, d->p, d->PresEq, d->Cs, d->P0, d->FPMassC,
                  d->G, d->drho, d->sigma, d->strrate, d->rotrate, d->shearstress, d->strain,
                  d->sigma_eq, d->pl_strain, d->sigma_y, d->eff_strain_rate, d->int_energy, d->T,
                  d->Ta, d->Tb, d->dTdt, d->k_T, d->cp_T, d->BC_T,
                  d->IsFree, d->NoSlip, d->ID, d->mat, r->x_h, d->not_write_surf_ID,
                  d->contneib_count, d->contneib_part, d->mesh_id, d->contact_surf_id,
                  d->first_fem_particle_idx};
  for (void* p : ptrs) free(p);
  for (int mi = 0; mi < d->trimesh_count; mi++) {
    TriMesh_d* t = d->trimesh[mi];
    void* mp[] = {t->node, t->node_v, t->elnode, t->pplane, t->centroid, t->normal, t->nfar};
    for (void* p : mp) free(p);
    delete t;
  }
  free(d->trimesh);
  free(d);
  delete r->mat;
  delete r;
}

/* scalar parameters: h, rho (density and rho_0), G, sigma_y, Cs, dt, alpha, beta */
void wfr_set_scalars(void* h, double hh, double rho, double G, double sy, double Cs, double dt,
                     double alpha, double beta) {
  RefDom* r = (RefDom*)h;
  Domain_d* d = r->dom;
  for (int64_t i = 0; i < r->n; i++) {
    d->h[i] = hh; d->rho[i] = rho; d->rho_0[i] = rho; d->G[i] = G; d->sigma_y[i] = sy;
    d->Cs[i] = Cs;
  }
  d->h_glob = hh;
  d->deltat = dt;
  d->Alpha = alpha;
  d->Beta = beta;
}

void wfr_set_material(void* h, int model, double E, double nu, double Et, double A, double B,
                      double n_, double C, double eps0, double m_, double Tm, double Tt) {
  RefDom* r = (RefDom*)h;
  *r->mat = Material_(Elastic_(E, nu));
  r->mat->Material_model = model;
  r->mat->Et = Et;
  r->mat->A = A; r->mat->B = B; r->mat->n = n_; r->mat->C = C; r->mat->eps_0 = eps0;
  r->mat->m = m_; r->mat->T_m = Tm; r->mat->T_t = Tt;
}

void wfr_set_arrays(void* h, const double* x, const double* m, const int32_t* id,
                    const double* T) {
  RefDom* r = (RefDom*)h;
  Domain_d* d = r->dom;
  for (int64_t i = 0; i < r->n; i++) {
    d->x[i] = make_double3(x[3 * i], x[3 * i + 1], x[3 * i + 2]);
    d->m[i] = m[i];
    d->ID[i] = id[i];
    if (T) d->T[i] = T[i];
  }
}

/* the Hollomon power law as the reference initialises it (Material.cuh:48-63) */
void wfr_set_hollomon(void* h, double E, double nu, double sy0, double K, double m) {
  RefDom* r = (RefDom*)h;
  Quiet q;                                     /* InitHollomon printf()s */
  *r->mat = Material_(Elastic_(E, nu));
  r->mat->InitHollomon(Elastic_(E, nu), sy0, K, m);
}

void wfr_add_bc(void* h, int zone, double vx, double vy, double vz) {
  RefDom* r = (RefDom*)h;
  r->bc_zone.push_back(zone);
  r->bc_v.push_back(make_double3(vx, vy, vz));
}

void wfr_set_rebuild_every(void* h, int k) { ((RefDom*)h)->rebuild_every = k; }

void wfr_set_not_write(void* h, const uint8_t* f) {
  RefDom* r = (RefDom*)h;
  for (int64_t i = 0; i < r->n; i++) r->dom->not_write_surf_ID[i] = f[i] != 0;
}

void wfr_set_contact(void* h, double mu_s, double mu_d) {
  Domain_d* d = ((RefDom*)h)->dom;
  d->friction_sta = mu_s;
  d->friction_dyn = mu_d;
}

/* a rigid mesh as main sets it up (WeldFormGPU.cu:545-610): the device mesh
 * (nodes, connectivity, centroids by CalcCentroids, normals given or by
 * CalcNormals), AddTrimeshParticles' bookkeeping, mesh_id and the centroid
 * particles (mass 0, the zone id) of the host domain (Domain.cpp:969-990) */
void wfr_add_trimesh(void* h, const double* nodes, int nn, const int32_t* tris, int ne,
                     const double* normals, int zone, int64_t first, const double* vel,
                     const double* angvel) {
  RefDom* r = (RefDom*)h;
  Domain_d* d = r->dom;
  TriMesh_d* t = new TriMesh_d();
  t->nodecount = nn;
  t->elemcount = ne;
  t->node = alloc<double3>(nn); t->node_v = alloc<double3>(nn);
  t->elnode = alloc<int>(3 * ne); t->pplane = alloc<double>(ne);
  t->centroid = alloc<double3>(ne); t->normal = alloc<double3>(ne); t->nfar = alloc<int>(ne);
  for (int q = 0; q < nn; q++) t->node[q] = make_double3(nodes[3 * q], nodes[3 * q + 1], nodes[3 * q + 2]);
  for (int k = 0; k < 3 * ne; k++) t->elnode[k] = tris[k];
  launch_seq(ne, [&] { t->CalcCentroids(); });
  if (normals) {
    for (int e = 0; e < ne; e++) t->normal[e] = make_double3(normals[3 * e], normals[3 * e + 1], normals[3 * e + 2]);
  } else {
    launch_seq(ne, [&] { t->CalcNormals(); });
  }
  t->m_v = make_double3(vel[0], vel[1], vel[2]);
  t->m_w = make_double3(angvel[0], angvel[1], angvel[2]);
  t->id = zone;
  const int m = d->trimesh_count;
  d->first_fem_particle_idx[m] = (int)first;       /* AddTrimeshParticles, Domain_d.cu:644-655 */
  d->contact_surf_id[m] = zone;
  d->trimesh[m] = t;
  d->trimesh_count++;
  for (int e = 0; e < ne; e++) {
    const int64_t p = first + e;
    d->x[p] = t->centroid[e];
    d->m[p] = 0.0;
    d->ID[p] = zone;
    d->mesh_id[p] = m;
    d->normal[p] = t->normal[e];
  }
  d->contact = true;
  d->solid_part_count = (int)d->first_fem_particle_idx[0];
  r->n_solid = d->solid_part_count;
}

/* MechFraserSolve prologue (SolverFraser.cu:56-123) */
void wfr_begin(void* h) {
  RefDom* r = (RefDom*)h;
  Domain_d* d = r->dom;
  memcpy(r->x_h, d->x, sizeof(double3) * r->n);
  rebuild(r, r->x_h);
  launch_seq(r->n, [&] { d->SetVel(make_double3(0., 0., 0.)); });
  r->ts_i = 0; r->is_yielding = 0; r->max_pl_strain = 0.0; r->time = 0.0;
  d->isfirst_step = true;
  d->id_free_surf = 1;                               /* SolverFraser.cu:118 */
  d->totmass = 0.0;                                  /* WeldFormGPU.cu:808-820 */
  for (int64_t i = 0; i < r->n; i++) d->totmass += d->m[i];
  if (d->contact)
    for (int m = 0; m < d->trimesh_count; m++) {
      /* CalcSpheresKernel (SolverFraser.cu:129-141): its radius loop reads
       * node[3e + n], past the node array for most elements, and only leaves
       * nfar = 2; that value is set here and the plane coefficients computed */
      TriMesh_d* t = d->trimesh[m];
      for (int e = 0; e < t->elemcount; e++) t->nfar[e] = 2;
      launch_seq(t->elemcount, [&] { t->UpdatePlaneCoeff(); });
    }
}

/* one iteration of the Fraser loop body (SolverFraser.cu:164-398), no
 * contact, no thermal, no output (x_h is never refreshed). */
void wfr_step(void* h, int64_t nsteps) {
  RefDom* r = (RefDom*)h;
  Domain_d* d = r->dom;
  Quiet q;
  const int64_t N = r->n;
  for (int64_t s = 0; s < nsteps; s++) {
    if (r->ts_i == 0 && r->is_yielding) rebuild(r, r->x_h);
    const uint *c = r->nbc.data(), *o = r->nbo.data(), *l = r->nbl.data();
    launch_seq(N, [&] { d->CalcDensInc(c, o, l, 0); });
    launch_seq(N, [&] { d->UpdateDensity(d->deltat); });
    launch_seq(N, [&] { d->CalcRateTensors(c, o, l); });
    launch_seq(N, [&] { PressureKernelExt(d->p, d->PresEq, d->Cs, d->P0, d->rho, d->rho_0, d->particle_count); });
    launch_seq(N, [&] { d->StressStrainOne((int)threadIdx.x); });
    launch_seq(N, [&] { d->CalcAccel(c, o, l, 0, 0.0); });
    if (d->contact) {                                 /* SolverFraser.cu:233-257 */
      launch_seq(N, [&] { d->CalculateSurface(c, o, l, d->totmass); });
      if (r->ts_i == 0) launch_seq(N, [&] { d->CalcContactNb(c, o, l); });
      launch_seq(N, [&] { d->CalcContactForcesWang(c, o, l); });
    }
    if (!r->is_yielding) {
      for (int64_t i = 0; i < N; i++)
        if (d->pl_strain[i] > r->max_pl_strain) r->max_pl_strain = d->pl_strain[i];
      if (r->max_pl_strain > MIN_PS_FOR_NBSEARCH) r->is_yielding = 1;
    }
    for (size_t b = 0; b < r->bc_zone.size(); b++)
      launch_seq(N, [&] { d->ApplyBCVel(r->bc_zone[b], r->bc_v[b]); });
    launch_seq(N, [&] { d->UpdatePosFraser(d->deltat); });
    launch_seq(N, [&] { d->UpdateVel(d->deltat); });
    for (size_t b = 0; b < r->bc_zone.size(); b++)
      launch_seq(N, [&] { d->ApplyBCVel(r->bc_zone[b], r->bc_v[b]); });
    launch_seq(N, [&] { d->CalcIntEnergy(); });
    if (d->contact) {                                 /* SolverFraser.cu:290-316 */
      /* MeshUpdateKernel's four stages, each over the whole mesh before the
       * next (the kernel runs them without a grid barrier) */
      for (int m = 0; m < d->trimesh_count; m++) {
        TriMesh_d* t = d->trimesh[m];
        launch_seq(t->nodecount, [&] { t->Move(d->deltat); });
        launch_seq(t->elemcount, [&] { t->CalcCentroids(); });
        launch_seq(t->elemcount, [&] { t->CalcNormals(); });
        launch_seq(t->elemcount, [&] { t->UpdatePlaneCoeff(); });
      }
      for (int m = 0; m < d->trimesh_count; m++)
        launch_seq(d->trimesh[m]->elemcount, [&] { d->UpdateContactParticles(m); });
    }
    d->isfirst_step = false;
    r->time += d->deltat;
    r->ts_i++;
    if (r->ts_i > r->rebuild_every - 1) r->ts_i = 0;
  }
}

/* Domain_d::ThermalSolve (Thermal.cu:188-260) for `nsteps` steps: the
 * neighbour lists of the current positions as CSR (neib_part / neib_offs,
 * which main builds before the call), then per step the array form of
 * ThermalSolveKernel (:101-142), CalcConvHeatKernel (:36-64) with the
 * domain's T_inf and the h_conv given (ThermalSolve passes its local
 * h_conv = 100), and TempCalcLeapfrogFirst / TempCalcLeapfrog (:16-31). */
void wfr_thermal_solve(void* h, int64_t nsteps, const double* k, const double* cp,
                       const int32_t* bc_t, double h_conv, double T_inf) {
  RefDom* r = (RefDom*)h;
  Domain_d* d = r->dom;
  const int64_t N = r->n;
  for (int64_t i = 0; i < N; i++) {
    d->k_T[i] = k[i];
    d->cp_T[i] = cp[i];
    d->BC_T[i] = bc_t[i];
  }
  d->T_inf = T_inf;
  rebuild(r, d->x);
  std::vector<int> offs(N + 1), part(r->nbl.size());
  for (int64_t i = 0; i < N; i++) offs[i] = (int)r->nbo[i];
  offs[N] = (int)(r->nbo[N - 1] + r->nbc[N - 1]);
  for (size_t q = 0; q < part.size(); q++) part[q] = (int)r->nbl[q];
  d->isfirst_step = true;
  for (int64_t s = 0; s < nsteps; s++) {
    launch_seq(N, [&] { ThermalSolveKernel(d->dTdt, d->x, d->h, d->m, d->rho, d->T, d->k_T,
                                           d->cp_T, part.data(), offs.data(), (int)N); });
    launch_seq(N, [&] { CalcConvHeatKernel(d->dTdt, d->m, d->rho, d->cp_T, d->T, d->T_inf,
                                           d->BC_T, h_conv, (int)N); });
    if (d->isfirst_step) {
      launch_seq(N, [&] { TempCalcLeapfrogFirst(d->T, d->Ta, d->Tb, d->dTdt, d->deltat, (int)N); });
      d->isfirst_step = false;
    } else {
      launch_seq(N, [&] { TempCalcLeapfrog(d->T, d->Ta, d->Tb, d->dTdt, d->deltat, (int)N); });
    }
  }
}

/* copies a named field out, layout as in the product ABI */
int wfr_get(void* h, const char* name, double* out) {
  RefDom* r = (RefDom*)h;
  Domain_d* d = r->dom;
  const int64_t N = r->n;
  auto cp3 = [&](const double3* p) {
    for (int64_t i = 0; i < N; i++) { out[3 * i] = p[i].x; out[3 * i + 1] = p[i].y; out[3 * i + 2] = p[i].z; }
  };
  auto cp = [&](const double* p, int c) { memcpy(out, p, sizeof(double) * c * N); };
  std::string s(name);
  if (s == "x") cp3(d->x);
  else if (s == "v") cp3(d->v);
  else if (s == "a") cp3(d->a);
  else if (s == "u") cp3(d->u);
  else if (s == "rho") cp(d->rho, 1);
  else if (s == "drho") cp(d->drho, 1);
  else if (s == "p") cp(d->p, 1);
  else if (s == "sigma") cp(d->sigma, 6);
  else if (s == "strrate") cp(d->strrate, 6);
  else if (s == "rotrate") cp(d->rotrate, 6);
  else if (s == "shearstress") cp(d->shearstress, 6);
  else if (s == "sigma_eq") cp(d->sigma_eq, 1);
  else if (s == "pl_strain") cp(d->pl_strain, 1);
  else if (s == "sigma_y") cp(d->sigma_y, 1);
  else if (s == "eff_strain_rate") cp(d->eff_strain_rate, 1);
  else if (s == "int_energy") cp(d->int_energy, 1);
  else if (s == "normal") cp3(d->normal);
  else if (s == "contforce") cp3(d->contforce);
  else if (s == "T") cp(d->T, 1);
  else if (s == "Ta") cp(d->Ta, 1);
  else if (s == "Tb") cp(d->Tb, 1);
  else if (s == "dTdt") cp(d->dTdt, 1);
  else return -1;
  return 0;
}

int wfr_get_id(void* h, int32_t* out) {
  RefDom* r = (RefDom*)h;
  for (int64_t i = 0; i < r->n; i++) out[i] = r->dom->ID[i];
  return 0;
}

}  // extern "C"
