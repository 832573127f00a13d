/*
 * wf_oracle.c — CPU oracle (FP64) for the explicit SPH solid-mechanics step.
 *
 * TEST INFRASTRUCTURE ONLY: loaded by tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline arm, never by the product library.
 *
 * Every function restates one reference kernel, in the reference's own
 * operation order, so that results can be compared bit for bit with the
 * reference compiled for the CPU (oracle/_ref) and with the plain-FP64 GPU
 * path.  Build flags must keep IEEE semantics: -O2 -ffp-contract=off, no
 * -ffast-math (the reference builds with --fmad=false, src/CMakeLists.txt:29).
 *
 * Where the reference reads memory it never initialises, the oracle fixes
 * the value and says so at the use site:
 *   - PresEq[] and P0[] are cudaMalloc'd but never copied (the host values at
 *     src/WeldFormGPU.cu:830 stay on the host): both are taken as 0, which
 *     selects EOS case 0 with zero reference pressure.
 *   - FPMassC[] is never written: taken as 1.0, Particle's default
 *     (src/Particle.cpp:55).  It only matters for non-free particles.
 *   - StressStrainOne accumulates into an uninitialised local `Strain`
 *     (src/cuda/Mechanical.cu:472,542): the oracle accumulates into the
 *     stored strain instead.
 *
 * Neighbour order.  cuNSearch visits the 27 cells in z, y, x order and takes
 * the particles of a cell in the order an atomicAdd handed out slots
 * (src/cuNSearch/src/cuNSearchKernels.cu:104,145-175): the order inside a cell
 * is not reproducible on the reference GPU.  The oracle fixes it to ascending
 * particle index; the neighbour SET is the reference's exactly.
 */
#define _GNU_SOURCE
#include <limits.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "wf_oracle.h"

#define NBMAX WF_MAX_NEIGHBORS
#define WFO_MAX_BC 64
#define WFO_MAX_MESH 8
#define WFO_PI 3.14159265358979323846      /* M_PI */
#define MIN_PS_FOR_NBSEARCH 1.e-6           /* src/cuda/SolverFraser.cu:17 */
#define CONT_MAX_NB 20                      /* MAX_NB_COUNT, src/cuda/Contact.cu:7 */

typedef struct { double x, y, z; } d3;
typedef struct { double xx, xy, xz, yx, yy, yz, zx, zy, zz; } t3;

struct wfo_domain {
  int64_t n, n_solid;
  double h_glob, dt, alpha, beta, totmass;
  wf_material mat;
  int has_mat;
  d3 *x, *v, *a, *u, *x_h, *normal, *contforce;
  double *h, *m, *rho, *rho0, *p, *drho, *Cs, *G;
  double *sigma, *strrate, *rotrate, *shearstress, *strain;
  double *sigma_eq, *pl_strain, *sigma_y, *eff_strain_rate, *int_energy, *dep;
  int32_t *ID;
  uint8_t *is_free, *not_write;
  double *T, *Ta, *Tb, *dTdt, *k_T, *cp_T;
  int32_t *BC_T;
  double T_inf, h_conv;
  int32_t *nb_count, *nb;
  int nbc;
  int32_t bc_zone[WFO_MAX_BC];
  d3 bc_v[WFO_MAX_BC];
  /* options */
  int rebuild_every, rebuild_after_yield, rebuild_current, thermal, return_map, energy_mode;
  int newton_max_iter, mlp_on, clamp_homologous;
  double chi, newton_rtol, output_interval;
  double mlp[WFO_MLP_NPARAM];
  /* contact with rigid triangle meshes (TriMesh_d, src/cuda/Mesh.cuh:19-54) */
  int contact, trimesh_count, contact_law;
  int32_t csid[WFO_MAX_MESH];      /* contact_surf_id: the zone id of each mesh */
  struct {
    int32_t nn, ne, first;         /* nodes, elements, first rigid particle */
    d3 *node, *node_v, *centroid, *normal;
    int32_t* elnode;
    double* pplane;
    d3 m_v, m_w;
  } mesh[WFO_MAX_MESH];
  int32_t *cont_cnt, *cont_nb;     /* contneib_count / contneib_part (20 per particle) */
  double mu_s, mu_d;               /* friction_sta / friction_dyn */
  int32_t id_free_surf;            /* 1, set by MechFraserSolve (SolverFraser.cu:118) */
  /* contact law 1 (no reference counterpart): penalty kappa K dx delta, regularised
   * Coulomb friction, frictional heat */
  double c_kappa, c_dx, c_vreg, c_eta;
  double* qf;                      /* frictional heat into each particle (W) */
  /* adaptive rebuild: at a plastic-strain increment (0: off) */
  double rb_dep;
  double* eps_rb;                  /* plastic strain at the last rebuild */
  /* solver state */
  int started, ts_i, is_yielding, isfirst_step, nb_built;
  double time, t_out, dt_out, max_pl_strain, int_energy_sum;
  int64_t step, newton_calls, newton_iters, mlp_used, rebuilds, newton_capped;
  /* output rows (no reference counterpart beyond the values SolverFraser.cu:350-388
   * prints): recorded at output times, or every step with output_every_step */
  int out_every_step;
  d3* fr;                          /* m a before the BCs, BC-zone particles, on row steps */
  double* series;                  /* rows of 11 + 3 nbc values */
  int64_t series_n, series_cap, series_alloc;
  char err[256];
};

static int g_threads = 0;

/* ------------------------------------------------------------------------ */
/* small vector / tensor algebra, tensor3.cu and vector_math.h semantics     */
/* ------------------------------------------------------------------------ */
static inline d3 v3(double x, double y, double z) { d3 r = {x, y, z}; return r; }
static inline d3 d3_sub(d3 a, d3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline d3 d3_add(d3 a, d3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
/* operator*(double s, double3 a) and operator*(double3 a, double s): a.x*s */
static inline d3 d3_scale(d3 a, double s) { return v3(a.x * s, a.y * s, a.z * s); }
/* dot: a.x*b.x + a.y*b.y + a.z*b.z, left to right (vector_math.h:805) */
static inline double d3_dot(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline double d3_len(d3 a) { return sqrt(d3_dot(a, a)); }
static inline d3 d3_cross(d3 a, d3 b) {
  return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
/* operator/(double3, double): multiply by 1.0/s (vector_math.h:785) */
static inline d3 d3_div(d3 a, double s) { double inv = 1.0 / s; return d3_scale(a, inv); }

static inline t3 t3_zero(void) { t3 r; memset(&r, 0, sizeof r); return r; }
/* FromFlatSym (tensor3.cu:62) */
static inline t3 t3_from_sym(const double* f) {
  t3 r;
  r.xx = f[0]; r.yy = f[1]; r.zz = f[2];
  r.xy = r.yx = f[3];
  r.yz = r.zy = f[4];
  r.xz = r.zx = f[5];
  return r;
}
/* FromFlatAntiSym (tensor3.cu:72) */
static inline t3 t3_from_antisym(const double* f) {
  t3 r;
  r.xx = f[0]; r.yy = f[1]; r.zz = f[2];
  r.xy = f[3]; r.yz = f[4]; r.xz = f[5];
  r.yx = -f[3]; r.zy = -f[4]; r.zx = -f[5];
  return r;
}
/* ToFlatSymPtr (tensor3.cu:95): upper triangle */
static inline void t3_to_flat(t3 t, double* f) {
  f[0] = t.xx; f[1] = t.yy; f[2] = t.zz; f[3] = t.xy; f[4] = t.yz; f[5] = t.xz;
}
/* operator*(tensor3, double) / operator*(double, tensor3): m.c * f */
static inline t3 t3_scale(t3 m, double f) {
  t3 r;
  r.xx = m.xx * f; r.xy = m.xy * f; r.xz = m.xz * f;
  r.yx = m.yx * f; r.yy = m.yy * f; r.yz = m.yz * f;
  r.zx = m.zx * f; r.zy = m.zy * f; r.zz = m.zz * f;
  return r;
}
static inline t3 t3_add(t3 a, t3 b) {
  t3 r;
  r.xx = a.xx + b.xx; r.xy = a.xy + b.xy; r.xz = a.xz + b.xz;
  r.yx = a.yx + b.yx; r.yy = a.yy + b.yy; r.yz = a.yz + b.yz;
  r.zx = a.zx + b.zx; r.zy = a.zy + b.zy; r.zz = a.zz + b.zz;
  return r;
}
static inline t3 t3_sub(t3 a, t3 b) {
  t3 r;
  r.xx = a.xx - b.xx; r.xy = a.xy - b.xy; r.xz = a.xz - b.xz;
  r.yx = a.yx - b.yx; r.yy = a.yy - b.yy; r.yz = a.yz - b.yz;
  r.zx = a.zx - b.zx; r.zy = a.zy - b.zy; r.zz = a.zz - b.zz;
  return r;
}
/* f * Identity(): Identity() has 1.0 on the diagonal, 0.0 elsewhere, and the
 * product multiplies every component (tensor3.cu:102,294). */
static inline t3 t3_ident_scaled(double f) {
  t3 r;
  r.xx = r.yy = r.zz = 1.0 * f;
  r.xy = r.xz = r.yx = r.yz = r.zx = r.zy = 0.0 * f;
  return r;
}
static inline t3 t3_trans(t3 m) {
  t3 r;
  r.xx = m.xx; r.yy = m.yy; r.zz = m.zz;
  r.xy = m.yx; r.xz = m.zx;
  r.yx = m.xy; r.yz = m.zy;
  r.zx = m.xz; r.zy = m.yz;
  return r;
}
/* operator*(tensor3, tensor3) exactly as tensor3.cu:241-256: the x column is
 * (A.B) but the y and z columns are (A.B^T). */
static inline t3 t3_mul_ref(t3 a, t3 b) {
  t3 r;
  r.xx = a.xx * b.xx + a.xy * b.yx + a.xz * b.zx;
  r.xy = a.xx * b.yx + a.xy * b.yy + a.xz * b.yz;
  r.xz = a.xx * b.zx + a.xy * b.zy + a.xz * b.zz;
  r.yx = a.yx * b.xx + a.yy * b.yx + a.yz * b.zx;
  r.yy = a.yx * b.yx + a.yy * b.yy + a.yz * b.yz;
  r.yz = a.yx * b.zx + a.yy * b.zy + a.yz * b.zz;
  r.zx = a.zx * b.xx + a.zy * b.yx + a.zz * b.zx;
  r.zy = a.zx * b.yx + a.zy * b.yy + a.zz * b.yz;
  r.zz = a.zx * b.zx + a.zy * b.zy + a.zz * b.zz;
  return r;
}
/* operator*(tensor3, double3) (tensor3.cu:225) */
static inline d3 t3_matvec(t3 m, d3 v) {
  return v3(m.xx * v.x + m.xy * v.y + m.xz * v.z,
            m.yx * v.x + m.yy * v.y + m.yz * v.z,
            m.zx * v.x + m.zy * v.y + m.zz * v.z);
}

/* ------------------------------------------------------------------------ */
/* SPH kernel and EOS (src/cuda/Functions.cu)                                */
/* ------------------------------------------------------------------------ */
/* GradKernel, cubic spline, Dim 3 (Functions.cu:76-88) */
static inline double grad_kernel(double q, double h) {
  double C = 1.0 / (h * h * h * h * WFO_PI);
  if (q == 0.0) return C / h * (-3.0 + (9.0 / 2.0) * q);
  else if (q < 1.0) return C / (q * h) * (-3.0 * q + (9.0 / 4.0) * q * q);
  else if (q < 2.0) return C / (q * h) * ((-3.0 / 4.0) * (2.0 - q) * (2.0 - q));
  else return 0.0;
}
/* DensitySolid, EOS 0 with P0 = 0 (Functions.cu:259-265) */
static inline double density_solid(double Cs0, double pressure, double density0) {
  return (pressure - 0.0) / (Cs0 * Cs0) + density0;
}

/* ------------------------------------------------------------------------ */
/* material models (src/cuda/Material.cuh:257-307)                           */
/* ------------------------------------------------------------------------ */
static inline double hollomon_sy(const wf_material* mt, double strain) {
  double eps0 = mt->sy0 / mt->E;                     /* InitHollomon, Material.cuh:122 */
  double eps1 = pow(mt->sy0 / mt->K_hol, 1. / mt->m_hol);
  double sy;
  if (strain + eps0 > eps1) sy = mt->K_hol * pow(strain + eps0, mt->m_hol);
  else sy = mt->sy0;
  return sy;
}
static inline double jc_sy(const wf_material* mt, double strain, double strain_rate, double temp) {
  double T_h = (temp - mt->Tt) / (mt->Tm - mt->Tt);
  double sr = strain_rate;
  if (strain_rate == 0.0) sr = 1.e-5;
  return (mt->A + mt->B * pow(strain, mt->n)) * (1.0 + mt->C * log(sr / mt->eps0)) *
         (1.0 - pow(T_h, mt->m));
}

/* ------------------------------------------------------------------------ */
/* helpers                                                                   */
/* ------------------------------------------------------------------------ */
static int fail(wfo_domain* d, int code, const char* msg) {
  if (d) snprintf(d->err, sizeof d->err, "%s", msg);
  return code;
}

static void* xcalloc(size_t n, size_t sz) { return calloc(n ? n : 1, sz); }

/* the contact pass filter of CalcDensInc / CalcAccel (InteractionAlt.cu:47-52) */
static inline int pass_ij(const wfo_domain* d, int64_t i, int64_t j) {
  if (!d->contact) return 1;
  int pass = 0;
  for (int mc = 0; mc < d->trimesh_count; mc++)
    if (d->ID[j] != d->csid[mc] && d->ID[i] != d->csid[mc]) pass = 1;
  return pass;
}
/* CalcRateTensors tests only ID[j] (InteractionAlt.cu:286-290) */
static inline int pass_j(const wfo_domain* d, int64_t j) {
  if (!d->contact) return 1;
  int pass = 0;
  for (int mc = 0; mc < d->trimesh_count; mc++)
    if (d->ID[j] != d->csid[mc]) pass = 1;
  return pass;
}

/* di, dj, mj of the pair loops (InteractionAlt.cu:60-75) */
static inline void pair_dens(const wfo_domain* d, int64_t i, int64_t j, double* di, double* dj,
                             double* mj) {
  if (!d->is_free[i]) *di = density_solid(d->Cs[j], d->p[i], d->rho0[j]);
  else *di = d->rho[i];
  if (!d->is_free[j]) {
    *dj = density_solid(d->Cs[i], d->p[j], d->rho0[i]);
    *mj = 1.0 * d->m[i];
  } else {
    *dj = d->rho[j];
    *mj = d->m[j];
  }
}

/* ------------------------------------------------------------------------ */
/* neighbour search: cuNSearch's float32 rule                               */
/* ------------------------------------------------------------------------ */
typedef struct {
  float gmin[3], gdelta[3], r2;
  uint32_t dim[3];
} grid_t;

/* computeMinMax + computeCellInformation (cuNSearchDeviceData.cu:27-123) */
static void grid_setup(const float* pf, int64_t n, float r, grid_t* g) {
  int mn[3] = {INT_MAX, INT_MAX, INT_MAX}, mx[3] = {INT_MIN, INT_MIN, INT_MIN};
  for (int64_t i = 0; i < n; i++)
    for (int a = 0; a < 3; a++) {
      int c = (int)floorf(pf[3 * i + a] / r);         /* kComputeMinMax :54-56 */
      if (c < mn[a]) mn[a] = c;
      if (c > mx[a]) mx[a] = c;
    }
  for (int a = 0; a < 3; a++) {
    float Min = (float)mn[a] * r, Max = (float)mx[a] * r;
    float gridSize = Max - Min;
    g->dim[a] = (uint32_t)ceilf(gridSize / r) + 4u;
    g->gmin[a] = Min - r * 2.0f;
    float gs2 = (float)g->dim[a] * r;
    g->gdelta[a] = (float)g->dim[a] / gs2;
  }
  g->r2 = r * r;
}

static inline void cell_of(const grid_t* g, const float* p, int c[3]) {
  for (int a = 0; a < 3; a++) c[a] = (int)floorf((p[a] - g->gmin[a]) * g->gdelta[a]);
}

/* Rebuilds nb_count / nb from the float copy of `src` positions. */
static int nb_search_from(wfo_domain* d, const d3* src) {
  int64_t n = d->n;
  if (n <= 0) return WF_OK;
  float r = (float)(2.0 * d->h_glob);                  /* SolverFraser.cu:72-79 */
  float* pf = (float*)malloc(sizeof(float) * 3 * n);
  if (!pf) return fail(d, WF_ERR_ALLOC, "oracle: out of memory");
  for (int64_t i = 0; i < n; i++) {
    pf[3 * i] = (float)src[i].x; pf[3 * i + 1] = (float)src[i].y; pf[3 * i + 2] = (float)src[i].z;
  }
  grid_t g;
  grid_setup(pf, n, r, &g);
  uint64_t ncell = (uint64_t)g.dim[0] * g.dim[1] * g.dim[2];
  uint32_t* cstart = (uint32_t*)xcalloc(ncell + 1, sizeof(uint32_t));
  uint32_t* cid = (uint32_t*)malloc(sizeof(uint32_t) * n);
  uint32_t* order = (uint32_t*)malloc(sizeof(uint32_t) * n);
  if (!cstart || !cid || !order) {
    free(pf); free(cstart); free(cid); free(order);
    return fail(d, WF_ERR_ALLOC, "oracle: out of memory (grid)");
  }
  for (int64_t i = 0; i < n; i++) {
    int c[3];
    cell_of(&g, pf + 3 * i, c);
    cid[i] = (uint32_t)(((uint64_t)c[2] * g.dim[1] + c[1]) * g.dim[0] + c[0]);
    cstart[cid[i] + 1]++;
  }
  for (uint64_t c = 0; c < ncell; c++) cstart[c + 1] += cstart[c];
  {
    uint32_t* cur = (uint32_t*)malloc(sizeof(uint32_t) * ncell);
    memcpy(cur, cstart, sizeof(uint32_t) * ncell);
    for (int64_t i = 0; i < n; i++) order[cur[cid[i]]++] = (uint32_t)i;  /* ascending index */
    free(cur);
  }
  const float r2 = g.r2;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; i++) {
    const float* pi = pf + 3 * i;
    int c[3];
    cell_of(&g, pi, c);
    int cnt = 0;
    int32_t* out = d->nb + (size_t)i * NBMAX;
    for (int z = -1; z < 2 && cnt < NBMAX; z++)
      for (int y = -1; y < 2 && cnt < NBMAX; y++)
        for (int x = -1; x < 2 && cnt < NBMAX; x++) {
          int fc0 = c[0] + x, fc1 = c[1] + y, fc2 = c[2] + z;
          if (fc0 < 0 || fc1 < 0 || fc2 < 0 || fc0 >= (int)g.dim[0] || fc1 >= (int)g.dim[1] ||
              fc2 >= (int)g.dim[2])
            continue;
          uint32_t cc = (uint32_t)(((uint64_t)fc2 * g.dim[1] + fc1) * g.dim[0] + fc0);
          for (uint32_t s = cstart[cc]; s < cstart[cc + 1]; s++) {
            uint32_t j = order[s];
            const float* pj = pf + 3 * (size_t)j;
            float dx = pj[0] - pi[0], dy = pj[1] - pi[1], dz = pj[2] - pi[2];
            float sq = dx * dx + dy * dy + dz * dz;     /* kComputeCounts :162-164 */
            if (sq < r2 && sq > 0.0) out[cnt++] = (int32_t)j;
            if (cnt == NBMAX) break;                    /* CUDA_MAX_NEIGHBORS */
          }
        }
    d->nb_count[i] = cnt;
  }
  free(pf); free(cstart); free(cid); free(order);
  d->nb_built = 1;
  return WF_OK;
}

/* ------------------------------------------------------------------------ */
/* stages of the Fraser loop body                                            */
/* ------------------------------------------------------------------------ */
/* Domain_d::CalcDensInc (InteractionAlt.cu:166-246) */
static void stage_density(wfo_domain* d) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < d->n_solid; i++) {
    double drho = 0.0;
    const int32_t* L = d->nb + (size_t)i * NBMAX;
    for (int k = 0; k < d->nb_count[i]; k++) {
      int64_t j = L[k];
      if (!pass_ij(d, i, j)) continue;
      d3 xij = d3_sub(d->x[i], d->x[j]);
      double rij = d3_len(xij);
      double di, dj, mj;
      pair_dens(d, i, j, &di, &dj, &mj);
      d3 vij = d3_sub(d->v[i], d->v[j]);
      double h_ = (d->h[i] + d->h[j]) / 2.0;
      double GK = grad_kernel(rij / h_, h_);
      double temp1 = d3_dot(vij, d3_scale(xij, GK));
      drho += mj * (di / dj) * temp1;
    }
    d->drho[i] = drho;
  }
}

/* UpdateDensity (Mechanical.cu:198-203) */
static void stage_update_density(wfo_domain* d) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < d->n_solid; i++) d->rho[i] += d->dt * d->drho[i];
}

/* Domain_d::CalcRateTensors (InteractionAlt.cu:262-383) */
static void stage_rates(wfo_domain* d) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < d->n_solid; i++) {
    t3 SRS = t3_zero(), RRS = t3_zero();
    const int32_t* L = d->nb + (size_t)i * NBMAX;
    for (int k = 0; k < d->nb_count[i]; k++) {
      int64_t j = L[k];
      if (!pass_j(d, j)) continue;
      d3 xij = d3_sub(d->x[i], d->x[j]);
      double rij = d3_len(xij);
      double di, dj, mj;
      pair_dens(d, i, j, &di, &dj, &mj);
      d3 vab = d3_sub(d->v[i], d->v[j]);
      double h_ = (d->h[i] + d->h[j]) / 2.0;
      double GK = grad_kernel(rij / h_, h_);
      t3 S;
      S.xx = 2.0 * vab.x * xij.x;
      S.xy = vab.x * xij.y + vab.y * xij.x;
      S.xz = vab.x * xij.z + vab.z * xij.x;
      S.yx = S.xy;
      S.yy = 2.0 * vab.y * xij.y;
      S.yz = vab.y * xij.z + vab.z * xij.y;
      S.zx = S.xz;
      S.zy = S.yz;
      S.zz = 2.0 * vab.z * xij.z;
      S = t3_scale(S, (-0.5) * GK);
      t3 R = t3_zero();
      R.xy = vab.x * xij.y - vab.y * xij.x;
      R.xz = vab.x * xij.z - vab.z * xij.x;
      R.yz = vab.y * xij.z - vab.z * xij.y;
      R.yx = -R.xy;
      R.xz = -R.xz;                 /* sign flip of xz (zx stays 0), :362 */
      R.zy = -R.yz;
      R = t3_scale(R, -0.5 * GK);
      double mj_dj = mj / dj;
      SRS = t3_add(SRS, t3_scale(S, mj_dj));
      RRS = t3_add(RRS, t3_scale(R, mj_dj));
    }
    t3_to_flat(RRS, d->rotrate + 6 * i);
    t3_to_flat(SRS, d->strrate + 6 * i);
  }
}

/* PressureKernelExt + EOS case 0 (Mechanical.cu:289-298, Functions.cu:211-213) */
static void stage_pressure(wfo_domain* d) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < d->n; i++)
    d->p[i] = 0.0 + (d->Cs[i] * d->Cs[i]) * (d->rho[i] - d->rho0[i]);
}

/* ---- return maps ---- */
/* hardening curve sigma_y(eps_p) at fixed strain rate and temperature, with
 * its slope; used by the consistent Newton return map. */
typedef struct {
  int model;
  double A, B, n, R, Th, sy_cur, Ep;   /* JC: (A + B ep^n) R Th;  bilinear: sy_cur + Ep dl */
  const wf_material* mt;
} hard_t;

static inline void hard_eval(const hard_t* hc, double ep0, double dl, double* sy, double* dsy) {
  if (hc->model == WF_JOHNSON_COOK) {
    double e = ep0 + dl;
    if (e > 0.0) {
      double pw = pow(e, hc->n);
      *sy = (hc->A + hc->B * pw) * hc->R * hc->Th;
      *dsy = hc->n * hc->B * pw / e * hc->R * hc->Th;
    } else {
      *sy = hc->A * hc->R * hc->Th;
      *dsy = 1.0e300;
    }
  } else if (hc->model == WF_HOLLOMON) {
    double eps0 = hc->mt->sy0 / hc->mt->E;
    double eps1 = pow(hc->mt->sy0 / hc->mt->K_hol, 1. / hc->mt->m_hol);
    double e = ep0 + dl + eps0;
    if (e > eps1) {
      double pw = pow(e, hc->mt->m_hol);
      *sy = hc->mt->K_hol * pw;
      *dsy = hc->mt->m_hol * hc->mt->K_hol * pw / e;
    } else {
      *sy = hc->mt->sy0;
      *dsy = 0.0;
    }
  } else {
    *sy = hc->sy_cur + hc->Ep * dl;
    *dsy = hc->Ep;
  }
}

/* MLP features shared with the GPU: trial ratio, eps_p, log strain rate,
 * homologous temperature (all scaled to O(1)). */
static inline void mlp_features(double ratio, double ep, double srate, double Th, double f[4]) {
  f[0] = ratio - 1.0;
  f[1] = (log10(ep + 1.0e-6) + 3.0) / 3.0;
  f[2] = (log10(srate > 1.0e-12 ? srate : 1.0e-12) - 1.5) / 3.5;
  f[3] = Th;
}
static double mlp_eval1(const double* P, const double f[4]);

/* Consistent Newton solve of  st - 3G dl - sy(ep0 + dl) = 0  on
 * [0, (st - sy0)/3G] with bisection safeguard; relative residual tol. */
static double newton_return(const wfo_domain* d, const hard_t* hc, double st, double G3,
                            double ep0, double sy0, double dl0, int* iters) {
  double hi = (st - sy0) / G3, lo = 0.0;
  double dl = dl0;
  if (!(dl > lo && dl <= hi)) dl = hi;
  int it = 0;
  for (; it < d->newton_max_iter; it++) {
    double sy, dsy;
    hard_eval(hc, ep0, dl, &sy, &dsy);
    double f = st - G3 * dl - sy;
    if (fabs(f) <= d->newton_rtol * st) break;
    if (f > 0.0) lo = dl; else hi = dl;
    double dn = dl + f / (G3 + dsy);
    if (!(dn > lo && dn < hi)) dn = 0.5 * (lo + hi);
    dl = dn;
  }
  *iters = it;
  return dl;
}

/* Domain_d::StressStrainOne (Mechanical.cu:458-554) with the radial return of
 * the reference, or the consistent Newton return map (option return_map=1). */
static void stage_stress(wfo_domain* d) {
  const wf_material* mt = &d->mat;
  int64_t calls = 0, iters = 0, used = 0, capped = 0;
#pragma omp parallel for schedule(static) reduction(+ : calls, iters, used, capped)
  for (int64_t i = 0; i < d->n_solid; i++) {
    t3 S = t3_from_sym(d->shearstress + 6 * i);
    t3 D = t3_from_sym(d->strrate + 6 * i);
    t3 W = t3_from_antisym(d->rotrate + 6 * i);
    t3 WT = t3_trans(W);
    t3 SRT = t3_mul_ref(S, WT);
    t3 RS = t3_mul_ref(W, S);
    double G = d->G[i], dt = d->dt;
    t3 Dd = t3_sub(D, t3_ident_scaled(1.0 / 3.0 * (D.xx + D.yy + D.zz)));
    t3 T1 = t3_add(t3_add(t3_scale(Dd, 2.0 * G), SRT), RS);
    S = t3_add(t3_scale(T1, dt), S);
    double eff = sqrt(0.5 * ((D.xx - D.yy) * (D.xx - D.yy) + (D.yy - D.zz) * (D.yy - D.zz) +
                             (D.zz - D.xx) * (D.zz - D.xx)) +
                      3.0 * (D.xy * D.xy + D.yz * D.yz + D.zx * D.zx));
    d->eff_strain_rate[i] = eff;
    double J2 = 0.5 * (S.xx * S.xx + 2.0 * S.xy * S.yx + 2.0 * S.xz * S.zx + S.yy * S.yy +
                       2.0 * S.yz * S.zy + S.zz * S.zz);
    double st = sqrt(3.0 * J2);
    double dep = 0.0;
    if (d->return_map == 0) {
      /* reference one-shot radial return (Mechanical.cu:503-536) */
      if (d->sigma_y[i] < st) S = t3_scale(S, d->sigma_y[i] / st);
      if (mt->model == WF_HOLLOMON) d->sigma_y[i] = hollomon_sy(mt, d->pl_strain[i]);
      else if (mt->model == WF_JOHNSON_COOK)
        d->sigma_y[i] = jc_sy(mt, d->pl_strain[i], eff, d->T[i]);
      d->sigma_eq[i] = st;
      if (st > d->sigma_y[i]) {
        double Ep = 0.0;
        if (mt->model == WF_BILINEAR) Ep = mt->E * mt->Et / (mt->E - mt->Et);
        if (Ep < 0) Ep = 1.0 * mt->E;
        dep = (st - d->sigma_y[i]) / (3. * G);
        d->pl_strain[i] += dep;
        d->sigma_eq[i] = d->sigma_y[i];
        if (mt->model == WF_BILINEAR) d->sigma_y[i] += dep * Ep;
      }
    } else {
      /* consistent return map: yield function at the current plastic strain,
       * Newton on the plastic multiplier, stress scaled onto the new surface */
      hard_t hc;
      memset(&hc, 0, sizeof hc);
      hc.model = mt->model; hc.mt = mt;
      double Th = 0.0;
      if (mt->model == WF_JOHNSON_COOK) {
        Th = (d->T[i] - mt->Tt) / (mt->Tm - mt->Tt);
        if (d->clamp_homologous) Th = Th < 0.0 ? 0.0 : (Th > 0.999 ? 0.999 : Th);
        double sr = eff == 0.0 ? 1.e-5 : eff;
        hc.A = mt->A; hc.B = mt->B; hc.n = mt->n;
        hc.R = 1.0 + mt->C * log(sr / mt->eps0);
        hc.Th = 1.0 - pow(Th, mt->m);
      } else if (mt->model == WF_BILINEAR) {
        hc.sy_cur = d->sigma_y[i];
        hc.Ep = mt->E * mt->Et / (mt->E - mt->Et);
      }
      double sy0, dsy0;
      hard_eval(&hc, d->pl_strain[i], 0.0, &sy0, &dsy0);
      d->sigma_eq[i] = st;
      if (st > sy0) {
        double G3 = 3.0 * G;
        double dl0 = (st - sy0) / G3;
        if (d->mlp_on && mt->model == WF_JOHNSON_COOK) {
          double f[4];
          mlp_features(st / sy0, d->pl_strain[i], eff, Th, f);
          double y = mlp_eval1(d->mlp, f);
          if (y > 1.0 && y <= 1.1) y = 1.0;           /* the GPU's mlp_accept() */
          if (y > 0.0 && y <= 1.0) { dl0 = y * dl0; used++; }
        }
        int it = 0;
        dep = newton_return(d, &hc, st, G3, d->pl_strain[i], sy0, dl0, &it);
        calls++; iters += it;
        if (it >= d->newton_max_iter) capped++;   /* stopped before the tolerance */
        double sy1, dsy1;
        hard_eval(&hc, d->pl_strain[i], dep, &sy1, &dsy1);
        S = t3_scale(S, sy1 / st);
        d->pl_strain[i] += dep;
        d->sigma_y[i] = sy1;
        d->sigma_eq[i] = sy1;
      } else {
        d->sigma_y[i] = sy0;
      }
    }
    d->dep[i] = dep;
    t3 Sig = t3_add(t3_ident_scaled(-d->p[i]), S);
    t3 Str = t3_add(t3_scale(D, dt), t3_from_sym(d->strain + 6 * i));
    t3_to_flat(Sig, d->sigma + 6 * i);
    t3_to_flat(Str, d->strain + 6 * i);
    t3_to_flat(S, d->shearstress + 6 * i);
  }
  d->newton_calls += calls;
  d->newton_iters += iters;
  d->mlp_used += used;
  d->newton_capped += capped;
}

/* Domain_d::CalcAccel (InteractionAlt.cu:18-150), KernelType 0, XSPH 0 */
static void stage_accel(wfo_domain* d) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < d->n_solid; i++) {
    d3 acc = v3(0., 0., 0.);
    const int32_t* L = d->nb + (size_t)i * NBMAX;
    t3 Si = t3_from_sym(d->sigma + 6 * i);
    for (int k = 0; k < d->nb_count[i]; k++) {
      int64_t j = L[k];
      if (!pass_ij(d, i, j)) continue;
      d3 xij = d3_sub(d->x[i], d->x[j]);
      double rij = d3_len(xij);
      double di, dj, mj;
      pair_dens(d, i, j, &di, &dj, &mj);
      d3 vij = d3_sub(d->v[i], d->v[j]);
      double h_ = (d->h[i] + d->h[j]) / 2.0;
      double GK = grad_kernel(rij / h_, h_);
      t3 PIij = t3_zero();
      if (d->alpha != 0.0 || d->beta != 0.0) {
        double MUij = h_ * d3_dot(vij, xij) / (rij * rij + 0.01 * h_ * h_);
        double Ci = !d->is_free[i] ? d->Cs[j] : d->Cs[i];   /* SoundSpeed EOS 0 returns Cs0 */
        double Cj = !d->is_free[j] ? d->Cs[i] : d->Cs[j];
        double Cij = 0.5 * (Ci + Cj);
        if (d3_dot(vij, xij) < 0)
          PIij = t3_ident_scaled((d->alpha * Cij * MUij + d->beta * MUij * MUij) / (0.5 * (di + dj)));
      }
      t3 Sj = t3_from_sym(d->sigma + 6 * j);
      t3 Tm = t3_add(t3_add(t3_scale(Si, 1.0 / (di * di)), t3_scale(Sj, 1.0 / (dj * dj))), PIij);
      d3 f = t3_matvec(t3_scale(Tm, mj), d3_scale(xij, GK));
      acc = d3_add(acc, f);
    }
    d->a[i] = acc;
  }
}

/* GeneralAfter = UserAcc -> ApplyBCVelKernel per BC (WeldFormGPU.cu:103-106,
 * Mechanical.cu:572-584) */
static void stage_bc(wfo_domain* d) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < d->n; i++)
    for (int b = 0; b < d->nbc; b++)
      if (d->ID[i] == d->bc_zone[b]) {
        d->a[i] = v3(0.0, 0.0, 0.0);
        d->v[i] = d->bc_v[b];
      }
}

/* UpdatePosFraser (Mechanical.cu:179-187) */
static void stage_update_pos(wfo_domain* d) {
  double dt = d->dt;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < d->n; i++) {
    d3 u_ = d3_add(d3_scale(d->v[i], dt), d3_scale(d3_scale(d3_scale(d->a[i], 0.5), dt), dt));
    d->x[i] = d3_add(d->x[i], u_);
    d->u[i] = d3_add(d->u[i], u_);
  }
}

/* UpdateVel (Mechanical.cu:142-148) */
static void stage_update_vel(wfo_domain* d) {
  double dt = d->dt;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < d->n; i++) d->v[i] = d3_add(d->v[i], d3_scale(d->a[i], dt));
}

/* ThermalCalcs (Thermal.cu:68-99): ThermalSolveKernel (:101-142) over the
 * neighbour list, Taylor-Quinney plastic heat (option chi), CalcConvHeatKernel
 * (:36-64), TempCalcLeapfrog[First] (:16-31). */
static void thermal_rates(wfo_domain* d, double h_conv, int plastic_heat) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < d->n; i++) {
    double s = 0.0;
    const int32_t* L = d->nb + (size_t)i * NBMAX;
    for (int k = 0; k < d->nb_count[i]; k++) {
      int64_t j = L[k];
      d3 xij = d3_sub(d->x[i], d->x[j]);
      double h_ = (d->h[i] + d->h[j]) / 2.0;
      double nxij = d3_len(xij);
      double GK = grad_kernel(nxij / h_, h_);
      s += d->m[j] / d->rho[j] *
           (4.0 * d->k_T[i] * d->k_T[j] / (d->k_T[i] + d->k_T[j]) * (d->T[i] - d->T[j])) *
           d3_dot(xij, d3_scale(xij, GK)) / (nxij * nxij);
    }
    s *= 1. / (d->rho[i] * d->cp_T[i]);
    if (plastic_heat && i < d->n_solid && d->dep[i] > 0.0)
      s += d->chi * d->sigma_y[i] * d->dep[i] / (d->rho[i] * d->cp_T[i] * d->dt);
    if (d->qf[i] > 0.0) s += d->qf[i] / (d->m[i] * d->cp_T[i]);   /* frictional heat, law 1 */
    if (d->BC_T[i] == 1) {
      double dS2 = pow(d->m[i] / d->rho[i], 0.666666666);
      double q_conv = h_conv * dS2 * (d->T_inf - d->T[i]) / d->m[i];
      s += 1. / d->cp_T[i] * q_conv;
    }
    d->dTdt[i] = s;
  }
}
static void thermal_leapfrog(wfo_domain* d) {
  double dt = d->dt;
  if (d->isfirst_step) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < d->n; i++) d->Ta[i] = d->T[i] - dt / 2.0 * d->dTdt[i];
  } else {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < d->n; i++) {
      d->Tb[i] = d->Ta[i];
      d->Ta[i] += d->dTdt[i] * dt;
      d->T[i] = (d->Ta[i] + d->Tb[i]) / 2.;
    }
  }
}

/* CalcIntEnergy (Energy.cu:5-19).  energy_mode 0 reproduces the reference,
 * which reads particle 0's tensors for every particle; mode 1 uses each
 * particle's own. */
static void stage_energy(wfo_domain* d) {
  double sum = 0.0;
  const double* ss0 = d->shearstress;
  const double* sr0 = d->strrate;
#pragma omp parallel for schedule(static) reduction(+ : sum)
  for (int64_t i = 0; i < d->n; i++) {
    const double* ss = d->energy_mode ? d->shearstress + 6 * i : ss0;
    const double* sr = d->energy_mode ? d->strrate + 6 * i : sr0;
    if (d->energy_mode && i >= d->n_solid) continue;
    double de = d->m[i] / d->rho[i] *
                (ss[0] * sr[0] + ss[1] * sr[1] + ss[2] * sr[2] +
                 2.0 * (ss[3] * sr[3] + ss[4] * sr[4] + ss[5] * sr[5]));
    d->int_energy[i] += de * d->dt;
    sum += d->int_energy[i];
  }
  d->int_energy_sum = sum;
}

/* ------------------------------------------------------------------------ */
/* contact with rigid triangle meshes (src/cuda/Geometry.cu, Contact.cu,    */
/* Mesh.cu), in SolverFraser.cu:233-257 and :289-316 order                  */
/* ------------------------------------------------------------------------ */
/* mesh_id[j]: the mesh whose element centroids include particle j */
static inline int mesh_of(const wfo_domain* d, int64_t j) {
  for (int mi = 0; mi < d->trimesh_count; mi++)
    if (j >= d->mesh[mi].first && j < (int64_t)d->mesh[mi].first + d->mesh[mi].ne) return mi;
  return -1;
}

/* Domain_d::CalculateSurface (Geometry.cu:26-88): normal of every solid
 * particle from its neighbours that are not rigid particles of the first
 * mesh (the reference loops mc < 1); |n| >= 0.25 h with at most 46 such
 * neighbours makes it a free-surface particle unless its zone is protected.
 * A particle without such neighbours gets 0 * inf = NaN components, as in the
 * reference, and is never tagged. */
static void stage_surface(wfo_domain* d) {
  const double np = (double)d->n;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < d->n_solid; i++) {
    d3 nrm = v3(0., 0., 0.);
    int corr = 0;
    const int32_t* L = d->nb + (size_t)i * NBMAX;
    for (int k = 0; k < d->nb_count[i]; k++) {
      const int64_t j = L[k];
      const d3 xij = d3_sub(d->x[i], d->x[j]);
      if (d->ID[j] != d->csid[0]) {
        nrm = d3_add(nrm, d3_scale(xij, d->m[j]));
        corr++;
      }
    }
    nrm = d3_scale(nrm, np / (d->totmass * (double)corr));
    d->normal[i] = nrm;
    if (d3_len(nrm) >= 0.25 * d->h[i] && corr <= 46 && !d->not_write[i])
      d->ID[i] = d->id_free_surf;
  }
}

/* Domain_d::CalcContactNb (Contact.cu:29-62), every rebuild_every steps: the
 * rigid neighbours within 2h of each free-surface particle, in neighbour
 * order, once per mesh whose zone id matches.  The reference has no bound
 * on the 20 slots; here a full list stops growing. */
static void stage_contact_nb(wfo_domain* d) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < d->n_solid; i++) {
    int cnt = 0;
    const int32_t* L = d->nb + (size_t)i * NBMAX;
    for (int k = 0; k < d->nb_count[i]; k++) {
      const int64_t j = L[k];
      const d3 xij = d3_sub(d->x[i], d->x[j]);
      for (int mc = 0; mc < d->trimesh_count; mc++)
        if (d->ID[i] == d->id_free_surf && d->ID[j] == d->csid[mc] &&
            d3_len(xij) < 2. * d->h[i] && cnt < CONT_MAX_NB)
          d->cont_nb[i * CONT_MAX_NB + cnt++] = (int32_t)j;
    }
    d->cont_cnt[i] = cnt;
  }
}

/* Domain_d::CalcContactForcesWang (Contact.cu:134-321): penalty force of the
 * rigid triangle of each contact neighbour on the predicted position, with
 * static / dynamic friction.  The force of the last contact is kept in
 * contforce; the acceleration accumulates every contact, and the predicted
 * position of a later contact sees the earlier ones. */
static void stage_contact_forces(wfo_domain* d) {
  const double dt = d->dt;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < d->n_solid; i++) {
    d->contforce[i] = v3(0., 0., 0.);
    for (int k = 0; k < d->cont_cnt[i]; k++) {
      const int64_t j = d->cont_nb[i * CONT_MAX_NB + k];
      const int mid = mesh_of(d, j);
      const int e = (int)(j - d->mesh[mid].first);
      const d3 x_pred = d3_add(d3_add(d->x[i], d3_scale(d->v[i], dt)),
                               d3_div(d3_scale(d3_scale(d->a[i], dt), dt), 2.));
      const d3 n = d->mesh[mid].normal[e];
      const double dist = d3_dot(n, x_pred) - d->mesh[mid].pplane[e];
      if (!(dist < d->h[i])) continue;
      const d3 Qj = d3_sub(d->x[i], d3_scale(n, dist));
      int inside = 1;
      const int32_t* en = d->mesh[mid].elnode + 3 * e;
      const d3* node = d->mesh[mid].node;
      for (int l = 0; l < 3 && inside; l++) {
        const int nx = l + 1 > 2 ? 0 : l + 1;
        const double crit = d3_dot(d3_cross(d3_sub(node[en[nx]], node[en[l]]),
                                            d3_sub(Qj, node[en[l]])), n);
        if (crit < 0.0) inside = 0;
      }
      if (!inside) continue;
      const double delta = d->h[i] - dist;
      const double kij = 2.0 * d->m[i] / (dt * dt);
      d->contforce[i] = d3_scale(n, 0.4 * kij * delta);
      d->a[i] = d3_add(d->a[i], d3_div(d->contforce[i], d->m[i]));
      if (d->mu_s > 0.) {
        const d3 du = d3_sub(d3_sub(x_pred, d->x[i]), d3_scale(d->v[j], dt));
        const d3 dtg = d3_sub(du, d3_scale(n, d3_dot(du, n)));
        const d3 ft = d3_scale(dtg, kij);
        if (d3_len(ft) < d->mu_s * d3_len(d->contforce[i])) {
          d->a[i] = d3_sub(d->a[i], d3_div(ft, d->m[i]));
        } else {
          const d3 fd = d3_div(d3_scale(ft, d->mu_d * d3_len(d->contforce[i])), d3_len(ft));
          d->contforce[i] = d3_sub(d->contforce[i], fd);
          d->a[i] = d3_sub(d->a[i], d3_div(fd, d->m[i]));
        }
      }
    }
  }
}

/* Closest point of triangle abc to p (Ericson, Real-Time Collision
 * Detection, 5.1.5: Voronoi regions of the vertices, edges and face). */
static d3 closest_on_tri(d3 p, d3 a, d3 b, d3 c) {
  const d3 ab = d3_sub(b, a), ac = d3_sub(c, a), ap = d3_sub(p, a);
  const double d1 = d3_dot(ab, ap), d2 = d3_dot(ac, ap);
  if (d1 <= 0.0 && d2 <= 0.0) return a;
  const d3 bp = d3_sub(p, b);
  const double d3v = d3_dot(ab, bp), d4 = d3_dot(ac, bp);
  if (d3v >= 0.0 && d4 <= d3v) return b;
  const double vc = d1 * d4 - d3v * d2;
  if (vc <= 0.0 && d1 >= 0.0 && d3v <= 0.0) return d3_add(a, d3_scale(ab, d1 / (d1 - d3v)));
  const d3 cp = d3_sub(p, c);
  const double d5 = d3_dot(ab, cp), d6 = d3_dot(ac, cp);
  if (d6 >= 0.0 && d5 <= d6) return c;
  const double vb = d5 * d2 - d1 * d6;
  if (vb <= 0.0 && d2 >= 0.0 && d6 <= 0.0) return d3_add(a, d3_scale(ac, d2 / (d2 - d6)));
  const double va = d3v * d6 - d5 * d4;
  if (va <= 0.0 && (d4 - d3v) >= 0.0 && (d5 - d6) >= 0.0)
    return d3_add(b, d3_scale(d3_sub(c, b), (d4 - d3v) / ((d4 - d3v) + (d5 - d6))));
  const double denom = 1.0 / (va + vb + vc);
  return d3_add(d3_add(a, d3_scale(ab, vb * denom)), d3_scale(ac, vc * denom));
}

/* Contact law 1 (the 2M-particle contact workload; no reference
 * counterpart).  Each solid particle takes the nearest tool triangle whose
 * closest point lies within h (ties: the first mesh, then the lowest
 * triangle index); with the gap g = (x - q).n along the face's outward normal
 * and the penetration delta = dx/2 - g > 0, the normal force is
 * kappa K dx delta (a pressure kappa K / dx on the particle's face dx^2).
 * Friction is Coulomb, regularised below the sliding speed v_reg:
 * F_t = -mu F_n v_t / max(|v_t|, v_reg), v_t the tangential velocity
 * relative to the tool; eta of the frictional power F_t . v_t heats the
 * particle. */
static void stage_contact_law1(wfo_domain* d) {
  const double K = d->mat.E / (3.0 * (1.0 - 2.0 * d->mat.nu));
  const double hs = d->h_glob * d->h_glob;
  const double rc = 0.5 * d->c_dx;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < d->n_solid; i++) {
    d->contforce[i] = v3(0., 0., 0.);
    d->qf[i] = 0.0;
    d->cont_cnt[i] = 0;
    double best = hs;
    int bm = -1, be = -1;
    d3 bq = v3(0., 0., 0.);
    for (int mi = 0; mi < d->trimesh_count; mi++)
      for (int e = 0; e < d->mesh[mi].ne; e++) {
        const int32_t* en = d->mesh[mi].elnode + 3 * e;
        const d3* nd = d->mesh[mi].node;
        const d3 q = closest_on_tri(d->x[i], nd[en[0]], nd[en[1]], nd[en[2]]);
        const d3 dv = d3_sub(d->x[i], q);
        const double d2 = d3_dot(dv, dv);
        if (d2 < best) { best = d2; bm = mi; be = e; bq = q; }
      }
    if (bm < 0) continue;
    /* contact normal: from the nearest surface point to the particle (the
     * face normal inside a face, continuous across edges and vertices); the
     * face normal and its signed gap for a centre behind the face */
    const d3 dv = d3_sub(d->x[i], bq);
    const double dist = sqrt(best);
    const double gf = d3_dot(dv, d->mesh[bm].normal[be]);
    d3 n;
    double g;
    if (gf >= 0.0 && dist > 0.0) { n = d3_div(dv, dist); g = dist; }
    else { n = d->mesh[bm].normal[be]; g = gf; }
    const double delta = rc - g;
    if (!(delta > 0.0)) continue;
    const double fn = d->c_kappa * K * d->c_dx * delta;
    d3 f = d3_scale(n, fn);
    /* relative to the tool surface at the nearest point: m_v + m_w x q */
    const d3 vtool = d3_add(d->mesh[bm].m_v, d3_cross(d->mesh[bm].m_w, bq));
    const d3 vrel = d3_sub(d->v[i], vtool);
    const d3 vt = d3_sub(vrel, d3_scale(n, d3_dot(vrel, n)));
    const double vtl = d3_len(vt);
    if (d->mu_s > 0.0) {
      const double s = d->mu_s * fn / (vtl > d->c_vreg ? vtl : d->c_vreg);
      f = d3_sub(f, d3_scale(vt, s));
      d->qf[i] = d->c_eta * s * vtl * vtl;
    }
    d->a[i] = d3_add(d->a[i], d3_div(f, d->m[i]));
    d->contforce[i] = f;
    d->cont_cnt[i] = 1;
  }
}

/* MeshUpdateKernel (Mesh.cu:24-29): TriMesh_d::Move, CalcCentroids,
 * CalcNormals, UpdatePlaneCoeff.  The reference runs the four in one kernel
 * without a grid-wide barrier, so an element may read nodes before or after
 * they move; here each runs over the whole mesh before the next (the
 * sequential meaning).  UpdatePlaneCoeff reads node[elnode[3e] + nfar] with
 * nfar = 2, the last index CalcSpheres assigns (Mesh.cu:205-231). */
static void mesh_plane_coeff(wfo_domain* d, int mi) {
  for (int e = 0; e < d->mesh[mi].ne; e++)
    d->mesh[mi].pplane[e] = d3_dot(d->mesh[mi].node[d->mesh[mi].elnode[3 * e] + 2],
                                   d->mesh[mi].normal[e]);
}
static void mesh_update(wfo_domain* d, int mi, double dt) {
  d3* node = d->mesh[mi].node;
  for (int q = 0; q < d->mesh[mi].nn; q++) {
    const d3 vr = d3_cross(d->mesh[mi].m_w, node[q]);
    d->mesh[mi].node_v[q] = d3_add(d->mesh[mi].m_v, vr);
    node[q] = d3_add(node[q], d3_scale(d->mesh[mi].node_v[q], dt));
  }
  for (int e = 0; e < d->mesh[mi].ne; e++) {
    const int32_t* en = d->mesh[mi].elnode + 3 * e;
    d->mesh[mi].centroid[e] = d3_div(d3_add(d3_add(node[en[0]], node[en[1]]), node[en[2]]), 3.);
  }
  for (int e = 0; e < d->mesh[mi].ne; e++) {
    const int32_t* en = d->mesh[mi].elnode + 3 * e;
    const d3 u = d3_sub(node[en[1]], node[en[0]]);
    const d3 v = d3_sub(node[en[2]], node[en[0]]);
    const d3 w = d3_cross(u, v);
    d->mesh[mi].normal[e] = d3_div(w, d3_len(w));
  }
  mesh_plane_coeff(d, mi);
}

/* Domain_d::UpdateContactParticles (Contact.cu:85-112): each element's rigid
 * particle takes the mean node velocity, zero acceleration and the normal. */
static void contact_particles_update(wfo_domain* d, int mi) {
  for (int e = 0; e < d->mesh[mi].ne; e++) {
    const int32_t* en = d->mesh[mi].elnode + 3 * e;
    d3 vv = v3(0., 0., 0.);
    for (int q = 0; q < 3; q++) vv = d3_add(vv, d->mesh[mi].node_v[en[q]]);
    const int64_t p = d->mesh[mi].first + e;
    d->v[p] = d3_div(vv, 3.);
    d->a[p] = v3(0., 0., 0.);
    d->normal[p] = d->mesh[mi].normal[e];
  }
}

/* ------------------------------------------------------------------------ */
/* solve loop (SolverFraser.cu:30-409)                                       */
/* ------------------------------------------------------------------------ */
static int check_ready(wfo_domain* d) {
  if (d->h_glob <= 0.0) return fail(d, WF_ERR_STATE, "h not set");
  if (d->dt <= 0.0) return fail(d, WF_ERR_STATE, "time step not set");
  if (!d->has_mat) return fail(d, WF_ERR_STATE, "material not set");
  return WF_OK;
}

static int solve_begin(wfo_domain* d, double dt_out) {
  int rc = check_ready(d);
  if (rc) return rc;
  d->time = 0.0;
  d->isfirst_step = 1;
  d->step = 0;
  d->t_out = dt_out;
  d->dt_out = dt_out;
  memcpy(d->x_h, d->x, sizeof(d3) * d->n);             /* :56 */
  rc = nb_search_from(d, d->x_h);                      /* :109 */
  if (rc) return rc;
  memcpy(d->eps_rb, d->pl_strain, sizeof(double) * d->n);
  if (d->contact && d->contact_law == 1 && !(d->c_dx > 0.0))
    return fail(d, WF_ERR_STATE, "contact law 1 needs the option contact_dx");
  for (int64_t i = 0; i < d->n_solid; i++) d->v[i] = v3(0., 0., 0.);   /* SetVelKernel :123 */
  if (d->contact)                                      /* CalcSpheresKernel :129-141 */
    for (int mi = 0; mi < d->trimesh_count; mi++) mesh_plane_coeff(d, mi);
  d->ts_i = 0;
  d->is_yielding = 0;
  d->max_pl_strain = 0.0;
  d->series_n = 0;
  d->started = 1;
  return WF_OK;
}

/* One output row, FP64, particles in index order (SolverFraser.cu:350-388:
 * max displacement from 0, max plastic strain, the sum of |contforce| over
 * free-surface particles), plus the contact force vector sum, the internal
 * energy sum and each BC zone's load. */
static void record_row(wfo_domain* d) {
  const int64_t w = 11 + 3 * (int64_t)d->nbc;
  if (d->series_n >= d->series_cap) return;
  if (d->series_n >= d->series_alloc) {
    int64_t na = d->series_alloc ? 2 * d->series_alloc : 256;
    if (na > d->series_cap) na = d->series_cap;
    d->series = (double*)realloc(d->series, sizeof(double) * (size_t)(na * w));
    d->series_alloc = na;
  }
  double* r = d->series + d->series_n * w;
  memset(r, 0, sizeof(double) * (size_t)w);
  r[0] = d->time;
  r[1] = (double)(d->step + 1);
  for (int64_t i = 0; i < d->n; i++) {
    if (d->u[i].x > r[2]) r[2] = d->u[i].x;
    if (d->u[i].y > r[3]) r[3] = d->u[i].y;
    if (d->u[i].z > r[4]) r[4] = d->u[i].z;
    if (d->pl_strain[i] > r[5]) r[5] = d->pl_strain[i];
    if (d->contact) {
      const d3 f = d->contforce[i];
      if (d->ID[i] == d->id_free_surf) r[6] += sqrt(f.x * f.x + f.y * f.y + f.z * f.z);
      r[7] += f.x;
      r[8] += f.y;
      r[9] += f.z;
    }
    r[10] += d->int_energy[i];
  }
  for (int b = 0; b < d->nbc; b++)
    for (int64_t i = 0; i < d->n; i++)
      if (d->ID[i] == d->bc_zone[b]) {
        r[11 + 3 * b] += d->fr[i].x;
        r[12 + 3 * b] += d->fr[i].y;
        r[13 + 3 * b] += d->fr[i].z;
      }
  d->series_n++;
}

static int solve_step(wfo_domain* d) {
  int rebuild;
  if (d->rb_dep > 0.0) {    /* adaptive: a plastic-strain increment since the last rebuild */
    double mx = 0.0;
    for (int64_t i = 0; i < d->n; i++)
      if (d->pl_strain[i] - d->eps_rb[i] > mx) mx = d->pl_strain[i] - d->eps_rb[i];
    rebuild = mx > d->rb_dep;
  } else {
    rebuild = d->ts_i == 0 && (d->is_yielding || !d->rebuild_after_yield);   /* :166 */
  }
  if (rebuild) {
    int rc = nb_search_from(d, d->rebuild_current ? d->x : d->x_h);
    if (rc) return rc;
    memcpy(d->eps_rb, d->pl_strain, sizeof(double) * d->n);
    d->rebuilds++;
  }
  stage_density(d);         /* :193 */
  stage_update_density(d);  /* :201 */
  stage_rates(d);           /* :204 */
  stage_pressure(d);        /* :213 */
  stage_stress(d);          /* :217 */
  stage_accel(d);           /* :221 */
  if (d->contact && d->contact_law == 1) {
    stage_contact_law1(d);
  } else if (d->contact) {  /* :233-257 */
    stage_surface(d);
    if (d->ts_i == 0) stage_contact_nb(d);
    stage_contact_forces(d);
  }
  if (!d->is_yielding) {    /* :260-271 */
    for (int64_t i = 0; i < d->n; i++)
      if (d->pl_strain[i] > d->max_pl_strain) d->max_pl_strain = d->pl_strain[i];
    if (d->max_pl_strain > MIN_PS_FOR_NBSEARCH) d->is_yielding = 1;
  }
  const int row_due = d->out_every_step || d->time + d->dt >= d->t_out;
  if (row_due)              /* the load each BC zone carries: m a before the BC zeroes a */
    for (int64_t i = 0; i < d->n; i++)
      for (int b = 0; b < d->nbc; b++)
        if (d->ID[i] == d->bc_zone[b]) d->fr[i] = d3_scale(d->a[i], d->m[i]);
  stage_bc(d);              /* :273 */
  stage_update_pos(d);      /* :275 */
  stage_update_vel(d);      /* :278 */
  stage_bc(d);              /* :281 */
  if (d->thermal) {         /* :285 */
    thermal_rates(d, d->h_conv, d->chi > 0.0);
    thermal_leapfrog(d);
  }
  stage_energy(d);          /* :287 */
  if (d->contact) {         /* :290-316 */
    for (int mi = 0; mi < d->trimesh_count; mi++) mesh_update(d, mi, d->dt);
    for (int mi = 0; mi < d->trimesh_count; mi++) contact_particles_update(d, mi);
  }
  d->isfirst_step = 0;      /* :320 */
  d->time += d->dt;
  if (row_due) record_row(d);                          /* :350-388 */
  if (d->time >= d->t_out) {                           /* :323-368 */
    memcpy(d->x_h, d->x, sizeof(d3) * d->n);
    d->t_out += d->dt_out;
  }
  d->step++;
  d->ts_i++;
  if (d->ts_i > (d->rebuild_every - 1)) d->ts_i = 0;   /* :395-397 */
  return WF_OK;
}

int wfo_mech_fraser_solve(wfo_domain* d, double tf, double dt_out) {
  if (!d) return WF_ERR_ARG;
  int rc = solve_begin(d, dt_out);
  if (rc) return rc;
  while (d->time < tf) {
    rc = solve_step(d);
    if (rc) return rc;
  }
  return WF_OK;
}

int wfo_step(wfo_domain* d, int64_t nsteps) {
  if (!d) return WF_ERR_ARG;
  if (!d->started) {
    int rc = solve_begin(d, d->output_interval);
    if (rc) return rc;
  }
  for (int64_t s = 0; s < nsteps; s++) {
    int rc = solve_step(d);
    if (rc) return rc;
  }
  return WF_OK;
}

/* Domain_d::ThermalSolve (Thermal.cu:188-260): conduction + convection +
 * leapfrog with a fixed neighbour list. */
int wfo_thermal_solve(wfo_domain* d, double tf) {
  if (!d) return WF_ERR_ARG;
  if (d->h_glob <= 0.0 || d->dt <= 0.0) return fail(d, WF_ERR_STATE, "h or time step not set");
  d->time = 0.0;
  d->isfirst_step = 1;
  int rc = nb_search_from(d, d->x);
  if (rc) return rc;
  while (d->time < tf) {
    thermal_rates(d, d->h_conv, 0);
    thermal_leapfrog(d);
    d->isfirst_step = 0;
    d->time += d->dt;
    d->step++;
  }
  return WF_OK;
}

int wfo_find_neighbors(wfo_domain* d) {
  if (!d) return WF_ERR_ARG;
  if (d->h_glob <= 0.0) return fail(d, WF_ERR_STATE, "h not set");
  memcpy(d->x_h, d->x, sizeof(d3) * d->n);
  return nb_search_from(d, d->x_h);
}

double wfo_grad_kernel(double q, double h) { return grad_kernel(q, h); }

int wfo_run_stage(wfo_domain* d, const char* s) {
  if (!d || !s) return WF_ERR_ARG;
  if (!strcmp(s, "density")) stage_density(d);
  else if (!strcmp(s, "update_density")) stage_update_density(d);
  else if (!strcmp(s, "rates")) stage_rates(d);
  else if (!strcmp(s, "pressure")) stage_pressure(d);
  else if (!strcmp(s, "stress")) stage_stress(d);
  else if (!strcmp(s, "accel")) stage_accel(d);
  else if (!strcmp(s, "bc")) stage_bc(d);
  else if (!strcmp(s, "update_pos")) stage_update_pos(d);
  else if (!strcmp(s, "update_vel")) stage_update_vel(d);
  else if (!strcmp(s, "thermal")) { thermal_rates(d, d->h_conv, d->chi > 0.0); thermal_leapfrog(d); }
  else if (!strcmp(s, "energy")) stage_energy(d);
  else return fail(d, WF_ERR_ARG, "unknown stage");
  return WF_OK;
}

/* ------------------------------------------------------------------------ */
/* lifecycle and setters                                                    */
/* ------------------------------------------------------------------------ */
int wfo_set_threads(int nthreads) {
  g_threads = nthreads;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
  return WF_OK;
}

int wfo_create(wfo_domain** out, int64_t n) {
  if (!out || n <= 0) return WF_ERR_ARG;
  wfo_domain* d = (wfo_domain*)calloc(1, sizeof(wfo_domain));
  if (!d) return WF_ERR_ALLOC;
  d->n = n;
  d->n_solid = n;
#define A(ptr, cnt) do { d->ptr = xcalloc((size_t)(cnt), sizeof(*d->ptr)); if (!d->ptr) { wfo_destroy(d); return WF_ERR_ALLOC; } } while (0)
  A(x, n); A(v, n); A(a, n); A(u, n); A(x_h, n); A(normal, n); A(contforce, n);
  A(h, n); A(m, n); A(rho, n); A(rho0, n); A(p, n); A(drho, n); A(Cs, n); A(G, n);
  A(sigma, 6 * n); A(strrate, 6 * n); A(rotrate, 6 * n); A(shearstress, 6 * n); A(strain, 6 * n);
  A(sigma_eq, n); A(pl_strain, n); A(sigma_y, n); A(eff_strain_rate, n); A(int_energy, n);
  A(dep, n); A(ID, n); A(is_free, n); A(not_write, n);
  A(T, n); A(Ta, n); A(Tb, n); A(dTdt, n); A(k_T, n); A(cp_T, n); A(BC_T, n);
  A(nb_count, n); A(nb, (size_t)n * NBMAX);
  A(cont_cnt, n); A(cont_nb, (size_t)n * CONT_MAX_NB); A(qf, n); A(eps_rb, n); A(fr, n);
#undef A
  d->series_cap = 65536;
  d->id_free_surf = 1;
  d->c_kappa = 0.1;
  d->c_vreg = 1.0e-3;
  d->c_eta = 1.0;
  for (int64_t i = 0; i < n; i++) d->is_free[i] = 1;
  /* SetDimension resets Alpha = 1, Beta = 0 (Domain_d.cu:191-192) */
  d->alpha = 1.0;
  d->beta = 0.0;
  d->rebuild_every = 5;        /* ts_nb_inc, SolverFraser.cu:91 */
  d->rebuild_after_yield = 1;
  d->rebuild_current = 0;
  d->thermal = 0;
  d->return_map = 0;
  d->energy_mode = 0;
  d->newton_max_iter = 50;
  d->newton_rtol = 1.0e-10;
  d->chi = 0.0;
  d->clamp_homologous = 1;
  d->output_interval = 1.0e300;
  d->h_conv = 100.0;           /* ThermalSolve local h_conv, Thermal.cu:204 */
  *out = d;
  return WF_OK;
}

int wfo_destroy(wfo_domain* d) {
  if (!d) return WF_OK;
  void* ptrs[] = {d->x, d->v, d->a, d->u, d->x_h, d->normal, d->contforce, d->h, d->m, d->rho,
                  d->rho0, d->p, d->drho, d->Cs, d->G, d->sigma, d->strrate, d->rotrate,
                  d->shearstress, d->strain, d->sigma_eq, d->pl_strain, d->sigma_y,
                  d->eff_strain_rate, d->int_energy, d->dep, d->ID, d->is_free, d->not_write,
                  d->T, d->Ta, d->Tb, d->dTdt, d->k_T, d->cp_T, d->BC_T, d->nb_count, d->nb,
                  d->cont_cnt, d->cont_nb, d->qf, d->eps_rb, d->fr, d->series};
  for (size_t k = 0; k < sizeof ptrs / sizeof ptrs[0]; k++) free(ptrs[k]);
  for (int mi = 0; mi < d->trimesh_count; mi++) {
    free(d->mesh[mi].node); free(d->mesh[mi].node_v); free(d->mesh[mi].centroid);
    free(d->mesh[mi].normal); free(d->mesh[mi].elnode); free(d->mesh[mi].pplane);
  }
  free(d);
  return WF_OK;
}

const char* wfo_last_error(const wfo_domain* d) { return d ? d->err : "null handle"; }

#define FILL(arr, val) do { for (int64_t i = 0; i < d->n; i++) d->arr[i] = (val); } while (0)
int wfo_set_h(wfo_domain* d, double h) { if (!d) return WF_ERR_ARG; FILL(h, h); d->h_glob = h; return WF_OK; }
int wfo_set_density(wfo_domain* d, double r) { if (!d) return WF_ERR_ARG; FILL(rho, r); FILL(rho0, r); return WF_OK; }
int wfo_set_shear_modulus(wfo_domain* d, double G) { if (!d) return WF_ERR_ARG; FILL(G, G); return WF_OK; }
int wfo_set_sigma_y(wfo_domain* d, double s) { if (!d) return WF_ERR_ARG; FILL(sigma_y, s); return WF_OK; }
int wfo_set_conductivity(wfo_domain* d, double k) { if (!d) return WF_ERR_ARG; FILL(k_T, k); return WF_OK; }
int wfo_set_heat_cap(wfo_domain* d, double c) { if (!d) return WF_ERR_ARG; FILL(cp_T, c); return WF_OK; }
#undef FILL
int wfo_set_cs(wfo_domain* d, const double* cs) {
  if (!d || !cs) return WF_ERR_ARG;
  memcpy(d->Cs, cs, sizeof(double) * d->n);
  return WF_OK;
}
int wfo_set_free(wfo_domain* d, const uint8_t* f) {
  if (!d || !f) return WF_ERR_ARG;
  memcpy(d->is_free, f, d->n);
  return WF_OK;
}
int wfo_set_id(wfo_domain* d, const int32_t* id) {
  if (!d || !id) return WF_ERR_ARG;
  memcpy(d->ID, id, sizeof(int32_t) * d->n);
  return WF_OK;
}
int wfo_set_positions(wfo_domain* d, const double* x) {
  if (!d || !x) return WF_ERR_ARG;
  memcpy(d->x, x, sizeof(d3) * d->n);
  return WF_OK;
}
int wfo_set_velocities(wfo_domain* d, const double* v) {
  if (!d || !v) return WF_ERR_ARG;
  memcpy(d->v, v, sizeof(d3) * d->n);
  return WF_OK;
}
int wfo_set_mass(wfo_domain* d, const double* m) {
  if (!d || !m) return WF_ERR_ARG;
  memcpy(d->m, m, sizeof(double) * d->n);
  d->totmass = 0.0;
  for (int64_t i = 0; i < d->n; i++) d->totmass += m[i];
  return WF_OK;
}
int wfo_set_not_write_surf_id(wfo_domain* d, const uint8_t* f) {
  if (!d || !f) return WF_ERR_ARG;
  memcpy(d->not_write, f, d->n);
  return WF_OK;
}
int wfo_set_solid_count(wfo_domain* d, int64_t ns) {
  if (!d || ns < 0 || ns > d->n) return WF_ERR_ARG;
  d->n_solid = ns;
  return WF_OK;
}
int wfo_set_time_step(wfo_domain* d, double dt) {
  if (!d || !(dt > 0.0)) return WF_ERR_ARG;
  d->dt = dt;
  return WF_OK;
}
int wfo_set_artificial_viscosity(wfo_domain* d, double a, double b) {
  if (!d) return WF_ERR_ARG;
  d->alpha = a;
  d->beta = b;
  return WF_OK;
}
int wfo_set_material(wfo_domain* d, const wf_material* mt) {
  if (!d || !mt) return WF_ERR_ARG;
  if (mt->model < 0 || mt->model > 2) return fail(d, WF_ERR_ARG, "unknown material model");
  d->mat = *mt;
  d->has_mat = 1;
  return WF_OK;
}
int wfo_set_velocity_bc(wfo_domain* d, int32_t index, double vx, double vy, double vz) {
  if (!d || index < 0 || index >= d->nbc) return WF_ERR_ARG;
  d->bc_v[index] = v3(vx, vy, vz);
  return WF_OK;
}
int wfo_get_output_series(wfo_domain* d, double* rows, int64_t cap_rows, int64_t* n_rows,
                          int64_t* width) {
  if (!d || !n_rows || (cap_rows > 0 && !rows)) return WF_ERR_ARG;
  const int64_t w = 11 + 3 * (int64_t)d->nbc;
  if (width) *width = w;
  const int64_t m = d->series_n < cap_rows ? d->series_n : cap_rows;
  if (m > 0) memcpy(rows, d->series, sizeof(double) * (size_t)(m * w));
  *n_rows = cap_rows > 0 ? m : d->series_n;
  return WF_OK;
}
int wfo_add_velocity_bc(wfo_domain* d, int32_t zone, double vx, double vy, double vz) {
  if (!d) return WF_ERR_ARG;
  if (d->nbc >= WFO_MAX_BC) return fail(d, WF_ERR_ARG, "too many boundary conditions");
  d->bc_zone[d->nbc] = zone;
  d->bc_v[d->nbc] = v3(vx, vy, vz);
  d->nbc++;
  return WF_OK;
}
int wfo_set_temperature(wfo_domain* d, const double* T) {
  if (!d || !T) return WF_ERR_ARG;
  memcpy(d->T, T, sizeof(double) * d->n);
  return WF_OK;
}
int wfo_set_thermal_bc(wfo_domain* d, const int32_t* b) {
  if (!d || !b) return WF_ERR_ARG;
  memcpy(d->BC_T, b, sizeof(int32_t) * d->n);
  return WF_OK;
}
int wfo_set_convection(wfo_domain* d, double hc, double Tinf) {
  if (!d) return WF_ERR_ARG;
  d->h_conv = hc;
  d->T_inf = Tinf;
  return WF_OK;
}

int wfo_set_option(wfo_domain* d, const char* key, double v) {
  if (!d || !key) return WF_ERR_ARG;
  if (!strcmp(key, "rebuild_every")) { if (v < 1) return WF_ERR_ARG; d->rebuild_every = (int)v; }
  else if (!strcmp(key, "rebuild_after_yield")) d->rebuild_after_yield = v != 0.0;
  else if (!strcmp(key, "rebuild_current_positions")) d->rebuild_current = v != 0.0;
  else if (!strcmp(key, "thermal")) d->thermal = v != 0.0;
  else if (!strcmp(key, "return_map")) d->return_map = (int)v;
  else if (!strcmp(key, "energy_mode")) d->energy_mode = (int)v;
  else if (!strcmp(key, "newton_rtol")) d->newton_rtol = v;
  else if (!strcmp(key, "newton_max_iter")) {
    if (!(v >= 1.0)) return fail(d, WF_ERR_ARG, "newton_max_iter must be >= 1");
    d->newton_max_iter = (int)v;
  }
  else if (!strcmp(key, "output_every_step")) d->out_every_step = v != 0;
  else if (!strcmp(key, "output_series_cap")) {
    if (!(v >= 1.0)) return fail(d, WF_ERR_ARG, "output_series_cap must be >= 1");
    d->series_cap = (int64_t)v;
  }
  else if (!strcmp(key, "taylor_quinney")) d->chi = v;
  else if (!strcmp(key, "output_interval")) d->output_interval = v;
  else if (!strcmp(key, "clamp_homologous")) d->clamp_homologous = v != 0.0;
  else if (!strcmp(key, "mlp")) d->mlp_on = v != 0.0;
  else if (!strcmp(key, "contact_stiffness")) d->c_kappa = v;
  else if (!strcmp(key, "contact_dx")) d->c_dx = v;
  else if (!strcmp(key, "contact_vreg")) d->c_vreg = v;
  else if (!strcmp(key, "contact_heat_fraction")) d->c_eta = v;
  else if (!strcmp(key, "rebuild_strain_increment")) d->rb_dep = v;
  else if (!strcmp(key, "precision") || !strcmp(key, "profile_kernel") || !strcmp(key, "graph") ||
           !strcmp(key, "fuse_heat")) {
    /* GPU-only switches: accepted and ignored by the FP64 oracle */
  } else return fail(d, WF_ERR_ARG, "unknown option");
  return WF_OK;
}

/* friction_sta / friction_dyn (WeldFormGPU.cu:640-641) and the contact law
 * (0: the reference's penalty law, CalcContactForcesWang) */
int wfo_set_contact(wfo_domain* d, double mu_static, double mu_dynamic, int law) {
  if (!d || law < 0 || law > 1 || !(mu_static >= 0.0) || !(mu_dynamic >= 0.0)) return WF_ERR_ARG;
  d->mu_s = mu_static;
  d->mu_d = mu_dynamic;
  d->contact_law = law;
  return WF_OK;
}

/* A rigid triangle mesh and its centroid particles (AddTrimeshParticles,
 * WeldFormGPU.cu:545-610, Domain.cpp:969-990): particles first .. first+ne-1
 * become the element centroids, with mass 0 and the mesh's zone id; the mesh
 * moves with velocity v and angular velocity w (m_v, m_w).  normals == NULL:
 * computed as in TriMesh_d::CalcNormals.  Turns contact on. */
int wfo_add_trimesh(wfo_domain* d, const double* nodes, int32_t nn, const int32_t* tris,
                    int32_t ne, const double* normals, int32_t zone_id, int64_t first,
                    const double* vel, const double* angvel) {
  if (!d || !nodes || !tris || nn <= 0 || ne <= 0 || !vel || !angvel) return WF_ERR_ARG;
  if (d->trimesh_count >= WFO_MAX_MESH) return fail(d, WF_ERR_ARG, "too many meshes");
  if (first < d->n_solid || first + ne > d->n) return fail(d, WF_ERR_ARG, "rigid particle range");
  if (zone_id == d->id_free_surf) return fail(d, WF_ERR_ARG, "zone id 1 is the free-surface id");
  for (int64_t k = 0; k < 3 * (int64_t)ne; k++)
    if (tris[k] < 0 || tris[k] >= nn) return fail(d, WF_ERR_ARG, "triangle node out of range");
  const int mi = d->trimesh_count;
  d->mesh[mi].nn = nn;
  d->mesh[mi].ne = ne;
  d->mesh[mi].first = (int32_t)first;
  d->mesh[mi].node = xcalloc(nn, sizeof(d3));
  d->mesh[mi].node_v = xcalloc(nn, sizeof(d3));
  d->mesh[mi].centroid = xcalloc(ne, sizeof(d3));
  d->mesh[mi].normal = xcalloc(ne, sizeof(d3));
  d->mesh[mi].elnode = xcalloc(3 * (size_t)ne, sizeof(int32_t));
  d->mesh[mi].pplane = xcalloc(ne, sizeof(double));
  for (int q = 0; q < nn; q++) d->mesh[mi].node[q] = v3(nodes[3 * q], nodes[3 * q + 1], nodes[3 * q + 2]);
  memcpy(d->mesh[mi].elnode, tris, sizeof(int32_t) * 3 * (size_t)ne);
  const d3* node = d->mesh[mi].node;
  for (int e = 0; e < ne; e++) {
    const int32_t* en = tris + 3 * e;
    d->mesh[mi].centroid[e] = d3_div(d3_add(d3_add(node[en[0]], node[en[1]]), node[en[2]]), 3.);
    if (normals) {
      d->mesh[mi].normal[e] = v3(normals[3 * e], normals[3 * e + 1], normals[3 * e + 2]);
    } else {
      const d3 w = d3_cross(d3_sub(node[en[1]], node[en[0]]), d3_sub(node[en[2]], node[en[0]]));
      d->mesh[mi].normal[e] = d3_div(w, d3_len(w));
    }
    const int64_t p = first + e;
    d->x[p] = d->mesh[mi].centroid[e];
    d->m[p] = 0.0;
    d->ID[p] = zone_id;
    d->normal[p] = d->mesh[mi].normal[e];
  }
  d->mesh[mi].m_v = v3(vel[0], vel[1], vel[2]);
  d->mesh[mi].m_w = v3(angvel[0], angvel[1], angvel[2]);
  d->csid[mi] = zone_id;
  d->trimesh_count++;
  d->contact = 1;
  d->totmass = 0.0;                                   /* WeldFormGPU.cu:808-820 */
  for (int64_t i = 0; i < d->n; i++) d->totmass += d->m[i];
  return WF_OK;
}

/* TriMesh_d::AxisPlaneMesh (src/cuda/Mesh.cu:48-194) as main builds a
 * "Plane" rigid body: (dens+1)^2 nodes stepped by dl = (p2.x - p1.x)/dens in
 * x (inner) and y (outer) from p1, at z = p1.z whatever the axis; two
 * triangles per cell, ordered for an outward normal +axis when positive;
 * normals are set on the axis.  Returns the element count 2 dens^2; nodes
 * (3 (dens+1)^2), tris (3 per element) and normals (3 per element) are
 * written when not NULL. */
int64_t wfo_gen_plane_mesh(int axis, int positive, const double* p1, const double* p2, int dens,
                           double* nodes, int32_t* tris, double* normals) {
  if (dens < 1 || axis < 0 || axis > 2 || !p1 || !p2) return -1;
  const int64_t ne = 2 * (int64_t)dens * dens;
  if (!nodes && !tris && !normals) return ne;
  const double dl = (p2[0] - p1[0]) / dens;
  const double x3 = p1[2];
  double x2 = p1[1];
  int64_t vi = 0;
  for (int j = 0; j <= dens; j++) {
    double x1 = p1[0];
    for (int i = 0; i <= dens; i++) {
      if (nodes) { nodes[3 * vi] = x1; nodes[3 * vi + 1] = x2; nodes[3 * vi + 2] = x3; }
      vi++;
      x1 += dl;
    }
    x2 += dl;
  }
  int64_t el = 0;
  for (int j = 0; j < dens; j++)
    for (int i = 0; i < dens; i++) {
      const int32_t n0 = (dens + 1) * j + i, n1 = n0 + 1;
      const int32_t n2 = (dens + 1) * (j + 1) + i, n3 = n2 + 1;
      const int32_t c[2][3] = {{n0, positive ? n1 : n2, positive ? n2 : n1},
                               {n1, positive ? n3 : n2, positive ? n2 : n3}};
      for (int e = 0; e < 2; e++, el++)
        if (tris) for (int q = 0; q < 3; q++) tris[3 * el + q] = c[e][q];
    }
  if (normals)
    for (int64_t e = 0; e < ne; e++) {
      normals[3 * e] = normals[3 * e + 1] = normals[3 * e + 2] = 0.0;
      normals[3 * e + axis] = positive ? 1.0 : -1.0;
    }
  return ne;
}

int wfo_set_mlp_params(wfo_domain* d, const double* params) {
  if (!d || !params) return WF_ERR_ARG;
  memcpy(d->mlp, params, sizeof(double) * WFO_MLP_NPARAM);
  return WF_OK;
}

/* ------------------------------------------------------------------------ */
/* getters                                                                   */
/* ------------------------------------------------------------------------ */
static const double* field_ptr(wfo_domain* d, const char* name, int* comps) {
  *comps = 1;
  if (!strcmp(name, "x")) { *comps = 3; return (double*)d->x; }
  if (!strcmp(name, "v")) { *comps = 3; return (double*)d->v; }
  if (!strcmp(name, "a")) { *comps = 3; return (double*)d->a; }
  if (!strcmp(name, "u")) { *comps = 3; return (double*)d->u; }
  if (!strcmp(name, "normal")) { *comps = 3; return (double*)d->normal; }
  if (!strcmp(name, "contforce")) { *comps = 3; return (double*)d->contforce; }
  if (!strcmp(name, "fric_heat")) return d->qf;
  if (!strcmp(name, "sigma")) { *comps = 6; return d->sigma; }
  if (!strcmp(name, "strrate")) { *comps = 6; return d->strrate; }
  if (!strcmp(name, "rotrate")) { *comps = 6; return d->rotrate; }
  if (!strcmp(name, "shearstress")) { *comps = 6; return d->shearstress; }
  if (!strcmp(name, "strain")) { *comps = 6; return d->strain; }
  if (!strcmp(name, "rho")) return d->rho;
  if (!strcmp(name, "rho0")) return d->rho0;
  if (!strcmp(name, "m")) return d->m;
  if (!strcmp(name, "h")) return d->h;
  if (!strcmp(name, "p")) return d->p;
  if (!strcmp(name, "drho")) return d->drho;
  if (!strcmp(name, "Cs")) return d->Cs;
  if (!strcmp(name, "G")) return d->G;
  if (!strcmp(name, "sigma_eq")) return d->sigma_eq;
  if (!strcmp(name, "pl_strain")) return d->pl_strain;
  if (!strcmp(name, "sigma_y")) return d->sigma_y;
  if (!strcmp(name, "eff_strain_rate")) return d->eff_strain_rate;
  if (!strcmp(name, "int_energy")) return d->int_energy;
  if (!strcmp(name, "dep")) return d->dep;
  if (!strcmp(name, "T")) return d->T;
  if (!strcmp(name, "Ta")) return d->Ta;
  if (!strcmp(name, "Tb")) return d->Tb;
  if (!strcmp(name, "dTdt")) return d->dTdt;
  return NULL;
}

int wfo_get_field(wfo_domain* d, const char* name, double* out) {
  if (!d || !name || !out) return WF_ERR_ARG;
  int c;
  const double* p = field_ptr(d, name, &c);
  if (!p) return fail(d, WF_ERR_ARG, "unknown field");
  memcpy(out, p, sizeof(double) * c * d->n);
  return WF_OK;
}

int wfo_set_field(wfo_domain* d, const char* name, const double* in) {
  if (!d || !name || !in) return WF_ERR_ARG;
  int c;
  double* p = (double*)field_ptr(d, name, &c);
  if (!p) return fail(d, WF_ERR_ARG, "unknown field");
  memcpy(p, in, sizeof(double) * c * d->n);
  return WF_OK;
}

int wfo_get_field_i32(wfo_domain* d, const char* name, int32_t* out) {
  if (!d || !name || !out) return WF_ERR_ARG;
  if (!strcmp(name, "ID")) memcpy(out, d->ID, sizeof(int32_t) * d->n);
  else if (!strcmp(name, "nb_count")) memcpy(out, d->nb_count, sizeof(int32_t) * d->n);
  else if (!strcmp(name, "BC_T")) memcpy(out, d->BC_T, sizeof(int32_t) * d->n);
  else if (!strcmp(name, "cont_count")) memcpy(out, d->cont_cnt, sizeof(int32_t) * d->n);
  else return fail(d, WF_ERR_ARG, "unknown field");
  return WF_OK;
}

int wfo_get_neighbors(wfo_domain* d, int32_t* counts, int32_t* lists) {
  if (!d || !counts || !lists) return WF_ERR_ARG;
  if (!d->nb_built) return fail(d, WF_ERR_STATE, "no neighbour list yet");
  memcpy(counts, d->nb_count, sizeof(int32_t) * d->n);
  memcpy(lists, d->nb, sizeof(int32_t) * d->n * NBMAX);
  return WF_OK;
}

int wfo_get_scalar(wfo_domain* d, const char* name, double* out) {
  if (!d || !name || !out) return WF_ERR_ARG;
  if (!strcmp(name, "time")) *out = d->time;
  else if (!strcmp(name, "step")) *out = (double)d->step;
  else if (!strcmp(name, "int_energy_sum")) *out = d->int_energy_sum;
  else if (!strcmp(name, "is_yielding")) *out = d->is_yielding;
  else if (!strcmp(name, "newton_calls")) *out = (double)d->newton_calls;
  else if (!strcmp(name, "newton_iters")) *out = (double)d->newton_iters;
  else if (!strcmp(name, "mlp_used")) *out = (double)d->mlp_used;
  else if (!strcmp(name, "rebuilds")) *out = (double)d->rebuilds;
  else if (!strcmp(name, "newton_capped")) *out = (double)d->newton_capped;
  else if (!strcmp(name, "totmass")) *out = d->totmass;
  else return fail(d, WF_ERR_ARG, "unknown scalar");
  return WF_OK;
}

/* ------------------------------------------------------------------------ */
/* generators                                                               */
/* ------------------------------------------------------------------------ */
/* calcHalfPartCount (src/Domain.cpp:473-488) */
static int calc_half_part_count(double r, double R, int xinc) {
  int ypartcount = -1;
  if (xinc > 0) {
    ypartcount = 1;
    double yp = r;
    double xp = r + (double)(xinc - 1) * 2. * r;
    double rad = sqrt(yp * yp + xp * xp);
    while (rad <= R - r) {
      yp += 2. * r;
      rad = sqrt(yp * yp + xp * xp);
      ypartcount++;
    }
    ypartcount -= 1;
  }
  return ypartcount;
}

int64_t wfo_gen_cylinder_ref(double x0, double y0, double z0, double Rxy, double Lz, double r,
                             double density, double* x, double* mass) {
  int64_t cnt = 0;
  int numpartxy = calc_half_part_count(r, Rxy, 1);
  double zp = z0 + r;
  while (zp <= (z0 + Lz - r)) {
    double yp = y0 - r - (2. * r * (numpartxy - 1));
    int numypart = 2 * numpartxy;
    int yinc = numpartxy, yinc_sign = -1;
    for (int j = 0; j < numypart; j++) {
      int numxpart = calc_half_part_count(r, Rxy, yinc);
      double xp = x0 - r - (2. * r * (numxpart - 1));
      for (int i = 0; i < 2 * numxpart; i++) {
        if (x) { x[3 * cnt] = xp; x[3 * cnt + 1] = yp; x[3 * cnt + 2] = zp; }
        cnt++;
        xp += 2. * r;
      }
      yp += 2. * r;
      yinc += yinc_sign;
      if (yinc < 1) { yinc = 1; yinc_sign = 1; }
    }
    zp += 2. * r;
  }
  double Vol = WFO_PI * Rxy * Rxy * Lz;
  if (mass && cnt > 0) *mass = Vol * density / (double)cnt;
  return cnt;
}

int64_t wfo_gen_box_cubic(double x0, double y0, double z0, double Lx, double Ly, double Lz,
                          double r, double density, double* x, double* mass) {
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
        double px = x0 + (2.0 * i + 1) * r, py = y0 + (2.0 * j + 1) * r, pz = z0 + (2.0 * k + 1) * r;
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
  double t0 = (mx[0] + r) - x0, t1 = (mx[1] + r) - y0, t2 = (mx[2] + r) - z0;
  if (mass && cnt > 0) *mass = t0 * t1 * t2 * density / (double)cnt;
  return cnt;
}

static inline uint64_t splitmix64(uint64_t* s) {
  uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
static inline double u01(uint64_t* s) { return (double)(splitmix64(s) >> 11) * (1.0 / 9007199254740992.0); }

/* Domain::AddCylUniformLength (Domain.cpp:1071-1192): rings of ceil(ang ri/2r)
 * particles at radii r_i, r_i + 2r, ... < Rxy, rows z = r, 3r, ... <= Lz;
 * mass pi Rxy^2 Lz density / count */
int64_t wfo_gen_cylinder_uniform(double Rxy, double Lz, double r, double density, double ang,
                                 int rows, double r_i, int32_t tag, double* x, int32_t* ids,
                                 double* mass) {
  if (!(r > 0.0) || !(Rxy > 0.0) || !(Lz > 0.0) || !(ang > 0.0)) return -1;
  const double z0 = r;
  int64_t cnt = 0;
  double zp = z0;
  while (zp <= (z0 + Lz - r)) {
    for (double ri = r_i; ri < Rxy; ri += 2. * r) {
      int tgcount;
      double dalpha;
      if (ri == 0.) { tgcount = 1; dalpha = 0.; }
      else { tgcount = (int)ceil((ang * ri) / (2. * r)); dalpha = ang / (tgcount); }
      for (int alphai = 0; alphai < tgcount; alphai++) {
        int32_t id = tag;
        if (ang < 2.0 * WFO_PI) {
          if (alphai < rows) id = 2;
          else if (alphai > tgcount - 1 - rows) id = 3;
        }
        double xp = ri * cos(alphai * dalpha);
        double yp = ri * sin(alphai * dalpha);
        if ((fabs(xp) < r / 10) && (fabs(yp) < r / 10)) id = 4;
        if (x) { x[3 * cnt] = xp; x[3 * cnt + 1] = yp; x[3 * cnt + 2] = zp; }
        if (ids) ids[cnt] = id;
        cnt++;
      }
    }
    zp += 2.0 * r;
  }
  if (mass && cnt > 0) {
    double Vol = WFO_PI * Rxy * Rxy * Lz;
    *mass = Vol * density / (double)cnt;
  }
  return cnt;
}

int64_t wfo_gen_cylinder_lattice(double R, double H, double dx, double jitter, uint64_t seed,
                                 double* x) {
  int64_t cnt = 0;
  int nxy = (int)floor(2.0 * R / dx + 0.5);
  int nz = (int)floor(H / dx + 0.5);
  uint64_t st = seed;
  for (int k = 0; k < nz; k++)
    for (int j = 0; j < nxy; j++)
      for (int i = 0; i < nxy; i++) {
        double px = (i + 0.5) * dx - R, py = (j + 0.5) * dx - R, pz = (k + 0.5) * dx;
        if (px * px + py * py > R * R) continue;
        if (x) {
          double jx = (2.0 * u01(&st) - 1.0) * jitter * dx;
          double jy = (2.0 * u01(&st) - 1.0) * jitter * dx;
          double jz = (2.0 * u01(&st) - 1.0) * jitter * dx;
          x[3 * cnt] = px + jx; x[3 * cnt + 1] = py + jy; x[3 * cnt + 2] = pz + jz;
        }
        cnt++;
      }
  return cnt;
}

int64_t wfo_assign_zone(const double* x, int64_t n, const double* start, const double* end,
                        int32_t zone_id, int32_t* id, uint8_t* not_write) {
  int64_t cnt = 0;
  for (int64_t a = 0; a < n; a++) {
    int inc = 1;
    for (int c = 0; c < 3; c++)
      if (x[3 * a + c] < start[c] || x[3 * a + c] > end[c]) inc = 0;
    if (inc) {
      id[a] = zone_id;
      if (not_write) not_write[a] = 1;
      cnt++;
    }
  }
  return cnt;
}

/* ------------------------------------------------------------------------ */
/* MLP (FP64 reference of the GPU inference and training kernels)           */
/* ------------------------------------------------------------------------ */
#define H1 64
#define H2 64
static inline double silu(double z) { return z / (1.0 + exp(-z)); }
static inline double dsilu(double z) {
  double s = 1.0 / (1.0 + exp(-z));
  return s * (1.0 + z * (1.0 - s));
}

static double mlp_eval1(const double* P, const double f[4]) {
  const double *W1 = P, *b1 = W1 + H1 * 4, *W2 = b1 + H1, *b2 = W2 + H2 * H1, *W3 = b2 + H2,
               *b3 = W3 + H2;
  double h1[H1], h2[H2];
  for (int o = 0; o < H1; o++) {
    double z = b1[o];
    for (int k = 0; k < 4; k++) z += W1[o * 4 + k] * f[k];
    h1[o] = silu(z);
  }
  for (int o = 0; o < H2; o++) {
    double z = b2[o];
    for (int k = 0; k < H1; k++) z += W2[o * H1 + k] * h1[k];
    h2[o] = silu(z);
  }
  double y = b3[0];
  for (int k = 0; k < H2; k++) y += W3[k] * h2[k];
  return y;
}

int wfo_mlp_forward(const double* P, const double* xin, int64_t n, double* y) {
  if (!P || !xin || !y) return WF_ERR_ARG;
  for (int64_t s = 0; s < n; s++) y[s] = mlp_eval1(P, xin + 4 * s);
  return WF_OK;
}

int wfo_mlp_loss_grad(const double* P, const double* xin, const double* t, int64_t n,
                      double* loss, double* grad) {
  if (!P || !xin || !t || !loss || !grad || n <= 0) return WF_ERR_ARG;
  const double *W1 = P, *b1 = W1 + H1 * 4, *W2 = b1 + H1, *b2 = W2 + H2 * H1, *W3 = b2 + H2,
               *b3 = W3 + H2;
  double *gW1 = grad, *gb1 = gW1 + H1 * 4, *gW2 = gb1 + H1, *gb2 = gW2 + H2 * H1, *gW3 = gb2 + H2,
         *gb3 = gW3 + H2;
  memset(grad, 0, sizeof(double) * WFO_MLP_NPARAM);
  double L = 0.0;
  for (int64_t s = 0; s < n; s++) {
    const double* f = xin + 4 * s;
    double z1[H1], h1[H1], z2[H2], h2[H2];
    for (int o = 0; o < H1; o++) {
      double z = b1[o];
      for (int k = 0; k < 4; k++) z += W1[o * 4 + k] * f[k];
      z1[o] = z; h1[o] = silu(z);
    }
    for (int o = 0; o < H2; o++) {
      double z = b2[o];
      for (int k = 0; k < H1; k++) z += W2[o * H1 + k] * h1[k];
      z2[o] = z; h2[o] = silu(z);
    }
    double y = b3[0];
    for (int k = 0; k < H2; k++) y += W3[k] * h2[k];
    double e = y - t[s];
    L += e * e;
    double gy = 2.0 * e / (double)n;
    gb3[0] += gy;
    double g2[H2];
    for (int k = 0; k < H2; k++) { gW3[k] += gy * h2[k]; g2[k] = gy * W3[k] * dsilu(z2[k]); }
    double g1[H1];
    for (int k = 0; k < H1; k++) g1[k] = 0.0;
    for (int o = 0; o < H2; o++) {
      gb2[o] += g2[o];
      for (int k = 0; k < H1; k++) { gW2[o * H1 + k] += g2[o] * h1[k]; g1[k] += g2[o] * W2[o * H1 + k]; }
    }
    for (int o = 0; o < H1; o++) {
      double g = g1[o] * dsilu(z1[o]);
      gb1[o] += g;
      for (int k = 0; k < 4; k++) gW1[o * 4 + k] += g * f[k];
    }
  }
  *loss = L / (double)n;
  return WF_OK;
}
