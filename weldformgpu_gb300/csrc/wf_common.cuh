// wf_common.cuh — shared definitions of the GB300 SPH step kernels.
//
// Per-particle state lives in "slots": particles are sorted by neighbour-search
// cell (ties broken by original particle id) at every neighbour rebuild and
// every per-particle array is physically reordered, so the pair loops gather
// neighbours that sit close in memory.  perm[slot] = original id and
// inv[original id] = slot translate at the ABI.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/weldform_gb300.h"

#define WF_NB WF_MAX_NEIGHBORS

// Neighbour lists are stored in blocks of 8 entries, block-major:
//   entry k of slot i is nb[((k / 8) * npad + i) * 8 + k % 8].
// A thread reads the 8 entries of one block as two int4 loads (32 contiguous
// bytes) and the 32 threads of a warp read one contiguous kilobyte, so a pair
// loop meets the latency of a list load once per 8 neighbours, and the next
// block can be fetched while the current one is processed.  Entries between a
// particle's count and the end of its last block hold the particle's own slot,
// so that whole blocks may be gathered without bounds checks.
#define WF_NB_BLK 8
#define WF_NB_BLOCKS ((WF_NB + WF_NB_BLK - 1) / WF_NB_BLK)
#define WF_NB_ALLOC (WF_NB_BLOCKS * WF_NB_BLK)   // entries allocated per slot
__host__ __device__ __forceinline__ int64_t nb_at(int64_t npad, int64_t i, int k) {
  return ((int64_t)(k >> 3) * npad + i) * WF_NB_BLK + (k & 7);
}
// block b of slot i as two int4 (entries 8b .. 8b+7)
__device__ __forceinline__ void nb_block(const int32_t* __restrict__ nb, int64_t npad, int64_t i,
                                         int b, int4& lo, int4& hi) {
  const int4* q = reinterpret_cast<const int4*>(nb + ((int64_t)b * npad + i) * WF_NB_BLK);
  lo = __ldg(q);
  hi = __ldg(q + 1);
}

// L2 prefetch of list block b of slot i, two blocks ahead of its use, so
// that the list stream (read once per pass, from DRAM) meets L2 latency when
// it is loaded; it holds no registers.  One thread of every `group` issues it
// (a 128-byte line holds the blocks of four consecutive slots).
__device__ __forceinline__ void nb_prefetch(const int32_t* nb, int64_t npad, int64_t i, int b,
                                            int group) {
  if ((threadIdx.x & (group - 1)) == 0)
    asm volatile("prefetch.global.L2 [%0];" ::"l"(nb + ((int64_t)b * npad + i) * WF_NB_BLK));
}

// Brings the line holding p towards L2 (a hint: no registers held).  The
// mixed pair passes issue it for the per-particle state their tail reads
// after the pair loop, so that the tail's loads hit L2.
__device__ __forceinline__ void prefetch_l2(const void* p) {
  asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

#define WF_MAX_BC 16
#define WF_MAX_MESH 4
#define WF_PI 3.14159265358979323846

// Device status bits (d_status[0]), read by the host after a run.
#define WF_STATUS_NAN       1   // a kernel produced NaN/Inf in the stress state
#define WF_STATUS_NB_CAP    2   // some particle hit WF_MAX_NEIGHBORS (list truncated)
#define WF_STATUS_GRID      4   // a particle fell outside the search grid
#define WF_STATUS_MMA_WAIT  8   // a tensor-core completion wait ran out (result discarded)
#define WF_STATUS_NEWTON   16   // a Newton return map stopped at newton_max_iter unconverged
#define WF_STATUS_SERIES   32   // the output series was full: rows were dropped
#define WF_STATUS_CHECKS   64   // option debug_checks: a list entry out of range (repaired
                                // before use) or a non-finite position or velocity

// Status words (int d_status[WF_STATUS_WORDS]): [0] bits, [1] yield flag,
// 64-bit counters at [2] Newton iterations, [4] plastic return maps, [6]
// network starts taken, [8] return maps that hit newton_max_iter.
#define WF_STATUS_WORDS 16

// Output row (wf_get_output_series), all FP64, reduced over the particles in a
// fixed order: [time, step, max u_x, max u_y, max u_z, max pl_strain,
// contact-force sum (|contforce| over free-surface particles), contact force
// vector sum (3), internal energy sum, then per velocity BC the sum of m a
// over its zone before the BC is imposed (3 each)].
#define WF_ROW_FIXED 11

// All per-slot arrays that move with the particles at a reorder.
struct Fields {
  double4* xm;      // position xyz, mass w
  double4* vd;      // velocity xyz, density w (start of step)
  double4* u;       // displacement xyz
  double4* a;       // acceleration xyz
  double* sig6;     // Cauchy stress, flat [xx yy zz xy yz xz]
  double* ss6;      // deviatoric (shear) stress
  double* eps6;     // accumulated strain
  double* sr6;      // strain rate
  double* rr6;      // rotation rate (upper triangle of the antisymmetric tensor)
  double* p;        // pressure
  double* seq;      // sigma_eq
  double* eps_p;    // accumulated equivalent plastic strain
  double* sy;       // yield stress
  double* eff;      // effective strain rate
  double* dep;      // plastic strain increment of the last step
  double* drho;     // density rate of the last step
  double* eint;     // internal energy
  double* T;        // temperature
  double* Ta;       // temperature leapfrog half steps
  double* Tb;
  double* dTdt;
  double* kT;       // conductivity
  double* cpT;      // heat capacity
  int32_t* id;      // zone / surface id
  int32_t* bct;     // thermal BC flag (1 = convection)
  int32_t* perm;    // original particle id of the slot
  uint8_t* nw;      // not_write_surf_ID
  float4* xh;       // float positions the next neighbour rebuild reads (x_h)
  // mixed-precision mirrors (written by the integration kernel)
  float4* p32;      // position xyz, mass w
  float4* v32;      // velocity xyz, density w
  float* ss32;      // deviatoric stress FP32 state (mixed form), 6 per slot
  float2* th32;     // heat-flux mirror (mixed form): T as a float pair (hi, lo)
  float4* p32n;     // next positions of the fused acceleration + integration pass
  double* pwn;      // cached eps_p^n of the Johnson-Cook law (< 0: not cached yet)
  // contact (allocated when a rigid mesh is added)
  double4* nrm;     // surface normal (solid particles) / element normal (rigid particles)
  double4* cf;      // contact force of the last contact (contforce)
  double* qf;       // frictional heat into the particle (W), contact law 1
  double* eps_rb;   // plastic strain at the last neighbour rebuild (adaptive rebuild)
};

// A rigid triangle mesh on the device (TriMesh_d, src/cuda/Mesh.cuh:19-54);
// its element e is carried by the rigid particle of original id first + e.
struct MeshDev {
  double4* node;      // node positions
  double4* node_v;    // node velocities
  double4* centroid;  // element centroids
  double4* normal;    // element normals
  int32_t* elnode;    // 3 nodes per element
  double* pplane;     // plane coefficient n . node
  int32_t nn, ne, first, zone;
  double mv[3], mw[3];  // translational and angular velocity (m_v, m_w)
  // contact law 1: triangles binned in cells whose coordinates are relative to
  // node 0 (the tool's frame up to its rotation).  A translating tool is
  // binned once; a rotating one (mw != 0) is binned again on the GPU every
  // step in a fixed box that holds it in any orientation.
  double grel[3], cs;           // bin grid origin relative to node 0, cell size
  double inv_cs;                // 1 / cs
  double margin;                // binning margin (h and a little)
  float glo[3], ghi[3];         // grid bounds widened by one cell, relative (FP32 early-out)
  int32_t dims[3];
  int32_t rot;                  // 1: rotating, binned every step
  int64_t cap;                  // bin entries allocated (cvert holds 3 * cap float4)
  int32_t* cstart;              // [cells + 1] CSR offsets
  int32_t* ctri;                // triangle indices, ascending within a cell (translating)
  uint32_t* cursor;             // [cells] fill cursors (rotating)
  uint32_t* scan_tmp;           // scan scratch (rotating)
  float4* off32;                // node 0 in FP32, written by the mesh motion
  float4* cvert;                // per bin entry: its triangle's vertices - node[0] in FP32
                                // (fixed for a translating tool), 3 float4; .w of the
                                // first holds the triangle index
  float tol32;                  // FP32 search tolerance in distance (see k_contact_law1)
};
#define WF_CONT_NB 20     // contact neighbours per particle (MAX_NB_COUNT, src/cuda/Contact.cu:7)

// Johnson-Cook / bilinear / Hollomon constants as the kernels use them.
struct MatParams {
  int model;
  double E, Et, Ep;               // bilinear
  double K_hol, m_hol, eps0_hol, eps1_hol, sy0;
  double A, B, n, C, eps0, m, Tm, Tt;
  double bin[5];                  // binomial coefficients C(n, k), k = 1..5
};

struct StepParams {
  int64_t n;            // slots (all particles)
  int64_t n_solid;      // original ids below this are solid (solid_part_count)
  int64_t npad;         // slot stride of the neighbour-list blocks (nb_at)
  double h, gkC;        // smoothing length (uniform) and 1/(h^4 pi)
  double dt;
  double Cs, G, rho0;   // uniform sound speed, shear modulus, reference density
  double alpha, beta;   // Monaghan artificial viscosity
  double chi;           // Taylor-Quinney coefficient (0: no plastic heat)
  double h_conv, T_inf; // convection
  int return_map;       // 0 reference radial return, 1 consistent Newton
  int newton_max_iter;
  double newton_rtol;
  int clamp_homologous;
  int energy_mode;      // 0 reference (particle 0's tensors), 1 per particle
  double* e0;           // mixed form, energy_mode 0: particle 0's S:D of this step
  const int32_t* inv;   // inv[original id] = slot (particle 0's slot for energy_mode 0)
  int contact;          // contact pass filter active
  int ncsid;
  int32_t csid[WF_MAX_MESH];
  MeshDev mesh[WF_MAX_MESH];   // ncsid meshes, zone ids in csid
  double mu_s, mu_d;    // static / dynamic friction coefficients
  int contact_law;      // 0 the reference's penalty law, 1 binned triangles (kappa K / dx)
  double c_kappa, c_dx, c_vreg, c_eta, Kbulk;   // law 1 constants, bulk modulus
  double totmass;       // sum of all particle masses (WeldFormGPU.cu:808-820)
  int32_t id_free_surf; // 1, the id of free-surface particles
  int32_t* cnb;         // contact neighbours [WF_CONT_NB * npad] (slot indices)
  int32_t* ccnt;        // contact neighbour counts [npad]
  unsigned long long* cstat;  // contact law 1 counters: [0] FP32 triangle tests, [1] FP64 ones
  int nbc;
  int32_t bc_zone[WF_MAX_BC];
  double bc_v[WF_MAX_BC][3];
  double4* fr;          // when not null (an output row is due this step): m a before the
                        // BCs are imposed, written at the slots of BC-zone particles
  int mlp_on;           // MLP warm start of the Newton return map
  int nb_pf;            // L2 prefetch of the neighbour lists nb_pf blocks ahead (mixed passes; 0 off)
  int state_pf;         // L2 prefetch of the state a mixed pass reads after its pair loop
  int wave_pf;          // L2 prefetch of the prologue of the slot one resident wave later
                        // and of the first wave_pf blocks of its list (0: none)
  int64_t pf_ahead;     // that distance in slots (set per launch; 0: none)
  double wave_dist;     // the distance in resident waves (host side)
  int refresh_pow;      // recompute eps_p^n with pow() this step (bounds series drift)
  int64_t log_cap;      // return-map log (training pairs for the MLP): capacity
  unsigned long long* log_count;
  float4* log_x;
  float* log_y;
  MatParams mat;
  // FP32 constants for the mixed form, computed once on the host: on GB300 a
  // per-thread FP64 division or conversion costs as much as an FP32 pair loop
  float hf, invhf, Cf, Chf, Csf, alphaf, betaf, epsf, dtf, G2f, mlp_scale;
  float k2f;        // 2 k: the pair conductivity 4 k_i k_j / (k_i + k_j) of a uniform k
  // Johnson-Cook constants of the FP32 increment form of the Newton return map
  float G3f, jcAf, jcBf, jcnf, binf[5];
  float jcTtf, jcinvdTf, jcCf, jcinveps0f, jcmf;   // T_t, 1/(T_m - T_t), C, 1/eps_0, m
  float chif, h_convf, T_inff;                      // heat: Taylor-Quinney, convection
};

#define WF_CUDA_OK(call)                                   \
  do {                                                     \
    cudaError_t e_ = (call);                               \
    if (e_ != cudaSuccess) return wf_cuda_fail(d, e_, #call); \
  } while (0)

// Cubic-spline kernel gradient (Dim 3) with C = 1/(h^4 pi) hoisted: the
// reference recomputes C from h_ = (h_i + h_j)/2 = h for every pair
// (src/cuda/Functions.cu:76-88); with a uniform h the value is identical.
__device__ __forceinline__ double gradK64(double q, double h, double C) {
  if (q == 0.0) return C / h * (-3.0 + (9.0 / 2.0) * q);
  else if (q < 1.0) return C / (q * h) * (-3.0 * q + (9.0 / 4.0) * q * q);
  else if (q < 2.0) return C / (q * h) * ((-3.0 / 4.0) * (2.0 - q) * (2.0 - q));
  return 0.0;
}

__device__ __forceinline__ float gradK32(float q, float h, float C) {
  if (q < 1.0f) return C / h * (-3.0f + 2.25f * q);
  else if (q < 2.0f) return C / (q * h) * (-0.75f * (2.0f - q) * (2.0f - q));
  return 0.0f;
}

// The mixed form's cubic-spline gradient factor GK (Functions.cu:82-88) from
// r^2 > 0 (invh = 1/h, Ch = C/h; the q < 1 branch is C/(q h) q (-3 + 9/4 q)
// without the division): r and C/r from one reciprocal square root, the two
// branches of the spline selected without a branch.  r^2 = 0 (a particle and
// itself: the padding entries of the lists) gives exactly 0: rsqrt(+0) = +inf,
// q = 0 * inf is NaN and both comparisons fail.
__device__ __forceinline__ float gk32_r2(float r2, float invh, float Ch, float C) {
  const float ri = rsqrtf(r2);
  const float q = r2 * ri * invh;
  const float t = 2.0f - q;
  const float inner = Ch * (-3.0f + 2.25f * q);
  const float outer = C * ri * (-0.75f * t * t);
  return q < 1.0f ? inner : (q < 2.0f ? outer : 0.0f);
}

// Return-map counters (64-bit status words at 2, 4, 6: Newton iterations,
// plastic calls, MLP starts taken) and the yielding flag (word 1), summed over
// the warp's active lanes first: one atomic per warp instead of one per
// particle, which would serialise on one L2 address.
// A return map that stopped at newton_max_iter without meeting its tolerance
// (capped) adds to the counter at word 8 and sets WF_STATUS_NEWTON.
__device__ __forceinline__ void warp_count(int* status, unsigned iters, unsigned calls,
                                           unsigned mlp_used, bool capped, bool yielding) {
  const unsigned mask = __activemask();
  const unsigned si = __reduce_add_sync(mask, iters);
  const unsigned sc = __reduce_add_sync(mask, calls);
  const unsigned sm = __reduce_add_sync(mask, mlp_used);
  const unsigned sk = __reduce_add_sync(mask, capped ? 1u : 0u);
  const bool y = __any_sync(mask, yielding);
  if ((int)(threadIdx.x & 31) == __ffs(mask) - 1) {
    if (si) atomicAdd((unsigned long long*)(status + 2), (unsigned long long)si);
    if (sc) atomicAdd((unsigned long long*)(status + 4), (unsigned long long)sc);
    if (sm) atomicAdd((unsigned long long*)(status + 6), (unsigned long long)sm);
    if (sk) {
      atomicAdd((unsigned long long*)(status + 8), (unsigned long long)sk);
      atomicOr(status, WF_STATUS_NEWTON);
    }
    if (y) status[1] = 1;
  }
}

__device__ __forceinline__ bool pass_ij(const StepParams& P, int32_t idi, int32_t idj) {
  if (!P.contact) return true;
  bool pass = false;
  for (int mc = 0; mc < P.ncsid; mc++)
    if (idj != P.csid[mc] && idi != P.csid[mc]) pass = true;
  return pass;
}
__device__ __forceinline__ bool pass_j(const StepParams& P, int32_t idj) {
  if (!P.contact) return true;
  bool pass = false;
  for (int mc = 0; mc < P.ncsid; mc++)
    if (idj != P.csid[mc]) pass = true;
  return pass;
}

// Kernel launchers (defined in the .cu files, called by wf_api.cu).
struct NbBuffers {
  int32_t* nb;      // [WF_NB_ALLOC * npad], blocks of 8 (nb_at)
  int32_t* cnt;     // [npad]
};

void launch_fp64_density(const StepParams& P, const Fields& F, double4* vd2, const NbBuffers& N,
                         cudaStream_t s);
void launch_fp64_stress(const StepParams& P, const Fields& F, const double4* vd2,
                        const NbBuffers& N, int* status, cudaStream_t s);
void launch_fp64_accel(const StepParams& P, const Fields& F, const double4* vd2,
                       const NbBuffers& N, cudaStream_t s);
void launch_integrate(const StepParams& P, const Fields& F, const double4* vd2,
                      const float4* a32, cudaStream_t s);
void launch_thermal(const StepParams& P, const Fields& F, const NbBuffers& N, int first,
                    int plastic_heat, int mixed, cudaStream_t s);

// contact (wf_contact.cu): surface tagging, contact list (when `list`) and
// penalty forces after the acceleration pass; mesh motion and rigid particles
// after the integration; plane coefficients at solve start
void launch_contact_stage(const StepParams& P, const Fields& F, const NbBuffers& N, bool list,
                          float4* a32, cudaStream_t s);
void launch_mesh_update(const StepParams& P, const Fields& F, int mixed, cudaStream_t s);
void launch_mesh_plane(const StepParams& P, cudaStream_t s);
struct TileHalo;
struct List16;
// density pass alone (mixed form; a call's first step, or heat off)
void launch_fp32_density(const StepParams& P, const Fields& F, double4* vd2, float4* v32b,
                         const NbBuffers& N, const List16& L16, cudaStream_t s);
// density pass of this step with the previous step's heat pass (mixed form);
// T: tile halos (T.cap = 0: none), L16: 16-bit lists (L16.base null: none)
void launch_fp32_density_heat(const StepParams& P, const Fields& F, double4* vd2, float4* v32b,
                              const NbBuffers& N, int first, int plastic_heat, const TileHalo& T,
                              const List16& L16, cudaStream_t s);
struct MlpL1;
// mlp_packed (the tcgen05 weight image) and mlp_l1 (layer 1) together, or neither;
// T: the tiles' halos (T.cap = 0: every block gathers from global memory)
// the mixed heat pass alone (a call's last step; the mixed ThermalSolve)
void launch_fp32_heat(const StepParams& P, const Fields& F, const NbBuffers& N, int plastic_heat,
                      cudaStream_t s);
void launch_fp32_stress(const StepParams& P, const Fields& F, const float4* v32b,
                        float* sigr32, const NbBuffers& N, int* status, const void* mlp_packed,
                        const MlpL1* mlp_l1, const TileHalo& T, const List16& L16,
                        cudaStream_t s);
void launch_fp32_accel(const StepParams& P, const Fields& F, const float4* v32b,
                       const float* sigr32, float4* a32, const NbBuffers& N, cudaStream_t s);
void launch_fp32_accel_integrate(const StepParams& P, const Fields& F, const float4* v32b,
                                 const float* sigr32, const double4* vd2, const NbBuffers& N,
                                 const TileHalo& T, const List16& L16, cudaStream_t s);
