// wf_api.cu — the C ABI (include/weldform_gb300.h) over the device domain.
//
// struct wf_domain plays the role of the reference's SPH::Domain_d
// (src/cuda/Domain_d.cuh:101-426): it owns the per-particle arena, the
// neighbour lists and the solver state, and runs MechFraserSolve's loop
// (src/cuda/SolverFraser.cu:30-409) and ThermalSolve (src/cuda/Thermal.cu:188-260)
// as sequences of kernel launches on one CUDA stream.
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/weldform_gb300.h"
#include "wf_common.cuh"
#include "wf_mlp.cuh"
#include "wf_nsearch.cuh"
#include "wf_tiles.cuh"

// wf_mlp.cu
int wf_mlp_pack_device(const float* dparams, void* dpacked, cudaStream_t s);
size_t wf_mlp_packed_bytes();
// wf_outputs.cu
int wf_out_partial_words(int nbc);
void launch_output_row(const StepParams& P, const Fields& F, double* part, double time,
                       double step, double* last, double* series, int64_t cap,
                       unsigned long long* count, int append, int* status, cudaStream_t s);

#define WF_VERSION "weldform-gb300 0.1 (sm_103a)"

// kernel ids for wf_set_option("profile_kernel", id)
enum { KID_NONE = 0, KID_DENSITY = 1, KID_STRESS = 2, KID_ACCEL = 3, KID_INTEGRATE = 4,
       KID_THERMAL = 5, KID_REBUILD = 6, KID_CONTACT = 7 };
// NVTX range names of the stages (a profiler shows the host-side launch of
// each stage under its name; without a profiler attached a range costs a
// few nanoseconds)
static const char* const kStageNames[] = {"wf", "density", "stress", "accel", "integrate",
                                          "thermal", "rebuild", "contact"};

struct wf_domain {
  int64_t n = 0, n_solid = 0, npad = 0;
  cudaStream_t stream = nullptr;
  int dev = 0;                  // the device the domain was created on
  char* arena = nullptr;        // fixed-size device arrays, one allocation
  size_t arena_bytes = 0;       // bytes the layout uses
  size_t arena_alloc = 0;       // bytes of the allocation (a cached one may be larger)
  // host -> device copies of the setters: two staging buffers filled on
  // cstream, each scattered on `stream` (ev_full: copy done, ev_free: scatter done)
  cudaStream_t cstream = nullptr;
  cudaEvent_t ev_full[2] = {nullptr, nullptr}, ev_free[2] = {nullptr, nullptr};
  int stage_next = 0;
  // uniform scalars (the reference's setters fill every particle with one value)
  double h = 0, rho0 = 0, G = 0, Cs = 0, dt = 0, alpha = 1.0, beta = 0.0;
  double h_conv = 100.0, T_inf = 0.0;
  bool h_set = false, rho_set = false, G_set = false, cs_set = false, mat_set = false;
  bool x_set = false, m_set = false;
  wf_material mat{};
  std::vector<int32_t> bc_zone;
  std::vector<std::array<double, 3>> bc_v;
  // options
  int precision = 0, return_map = 0, mlp_on = 0, rebuild_every = 5, rebuild_after_yield = 1;
  int rebuild_current = 0, thermal = 0, energy_mode = 0, newton_max_iter = 50;
  int clamp_homologous = 1, profile_kernel = KID_NONE, resume = 0;
  double chi = 0.0, newton_rtol = 1.0e-10, output_interval = 1.0e300;
  // device arena
  Fields F[2]{};
  int cur = 0;
  double4* vd2 = nullptr;
  float4* v32b = nullptr;
  float4* a32 = nullptr;       // mixed-form acceleration
  float* sigr32 = nullptr;
  float* mlp_w = nullptr;      // device MLP parameters (FP32, packed layout of wf_mlp.cuh)
  void* mlp_packed = nullptr;  // BF16 tensor-core fragment image of mlp_w
  MlpL1 mlp_l1{};              // layer 1 of mlp_w (a kernel parameter of the stress pass)
  bool mlp_loaded = false;
  // return-map log: (features, converged increment) pairs from the plain form
  int64_t log_cap = 0;
  unsigned long long* log_count = nullptr;
  float4* log_x = nullptr;
  float* log_y = nullptr;
  int32_t *nb = nullptr, *nbc = nullptr, *inv = nullptr;
  float4 *pf = nullptr, *pf2 = nullptr;
  uint32_t *cellid = nullptr, *cell_count = nullptr, *cell_cursor = nullptr, *scan_tmp = nullptr;
  int64_t cell_cap = 0, scan_cap = 0;
  int32_t *s_src = nullptr, *s_orig = nullptr;
  int* d_mm = nullptr;
  int* d_status = nullptr;     // WF_STATUS_WORDS words (wf_common.cuh)
  int* h_status = nullptr;     // pinned mirror
  // FP64 output rows (wf_outputs.cu): recorded at output times, or every step
  // with option output_every_step; the series holds up to series_cap rows
  double4* fr = nullptr;       // m a before the BCs at BC-zone slots (written on row steps)
  double* e0 = nullptr;        // mixed form, energy_mode 0: particle 0's S:D (one word)
  double* out_part = nullptr;  // per-block partials of the row reduction
  double* out_last = nullptr;  // the last row recorded
  double* series = nullptr;
  int64_t series_cap = 65536, series_width = 0;
  unsigned long long* series_count = nullptr;
  bool out_every_step = false, row_recorded = false, print_outputs = false;
  bool lists_stale = false;    // positions replaced mid-run: rebuild at the next step
  // tile halos of the staged mixed pair passes (wf_tiles.cuh), rebuilt with the lists
  int32_t *t_hoff = nullptr, *t_hcnt = nullptr, *t_halo = nullptr;
  uint16_t* t_nbl = nullptr;
  int64_t t_halo_cap = 0;
  int tile_staging = 0;        // option "tile_staging" (off: measured slower, see the design notes)
  int list_prefetch = 2;       // option "list_prefetch" (blocks ahead)
  int state_prefetch = 1;      // option "state_prefetch"
  int wave_prefetch = 2;       // option "wave_prefetch"
  double wave_dist = 1.0;      // option "wave_prefetch_distance"
  // 16-bit lists of the global gather path (wf_tiles.cuh), rebuilt with the lists
  int list16 = 0;              // option "list16"
  bool l16_built = false;
  int32_t* l16_base = nullptr;
  uint16_t* l16_off = nullptr;
  int tile_cap_max = WF_TILE_HALO_MAX;   // option "tile_cap_max": largest halo staged
  int tile_cap = 0;            // halo capacity the current tiles were built for (0: none)
  int tile_hmax = 0;           // largest halo of the last build (read at the next rebuild)
  // the per-step host hook (GeneralAfter)
  wf_after_fn after_fn = nullptr;
  void* after_user = nullptr;
  bool in_callback = false;
  unsigned long long* d_cstat = nullptr;   // contact law 1 triangle-test counters
  double* d_stage = nullptr;   // staging for ABI copies (6 doubles per particle)
  double* d_stage2 = nullptr;  // the setters' second staging buffer
  // solver state
  bool started = false, nb_built = false, is_yielding = false, isfirst = true;
  // mixed form: the heat pass of the last step runs inside the next step's
  // density pass, or in finish() when the call ends first
  bool fuse_heat = true, heat_pending = false, heat_pending_first = false;
  bool fuse_integrate = true;    // mixed form without contact: integration inside the accel pass
  // contact with rigid triangle meshes
  std::vector<MeshDev> meshes;
  double mu_s = 0.0, mu_d = 0.0, totmass = 0.0;
  int contact_law = 0;
  int32_t *cnb = nullptr, *ccnt = nullptr;
  // contact law 1 constants; tool bins built at the first solve
  double c_kappa = 0.1, c_dx = 0.0, c_vreg = 1.0e-3, c_eta = 1.0;
  bool bins_built = false;
  // adaptive rebuild at a plastic-strain increment (0: the reference's cadence)
  double rb_dep = 0.0;
  double k_cond = 0.0;          // conductivity (wf_set_conductivity: uniform)
  int64_t rebuilds = 0;         // neighbour rebuilds inside the step loop
  int light_rebuilds = 0;       // rebuilds since the state was last moved into cell order
  unsigned long long* d_maxdep = nullptr;
  unsigned long long* h_maxdep = nullptr;
  // MechFraserSolve's CSV snapshots (out_<time>.csv), when a prefix is set
  bool csv_on = false;
  std::string csv_prefix;
  double time = 0, t_out = 0, dt_out = 0;
  int64_t step = 0;
  int ts_i = 0;
  GridDev grid{};
  // measurement
  int64_t launches = 0;
  std::vector<cudaEvent_t> ev_pool;
  size_t ev_used = 0;
  bool timing = false;         // inside wf_time_steps
  int debug_checks = 0;        // option "debug_checks"
  int64_t inject_list_error = -1;   // option "debug_inject_list_error" (original id), -1 off
  // step-segment graphs (segment_begin / segment_end)
  int graph = 1;                // option "graph"
  bool capturing = false;
  cudaGraphExec_t gexec = nullptr;
  int64_t graph_launches = 0, graph_instantiations = 0;
  std::string err;
};

static int wf_cuda_fail(wf_domain* d, cudaError_t e, const char* what) {
  if (d) d->err = std::string(what) + ": " + cudaGetErrorString(e);
  return WF_ERR_CUDA;
}
static int wf_fail(wf_domain* d, int code, const std::string& msg) {
  if (d) d->err = msg;
  return code;
}

// ---------------------------------------------------------------------------
// small utility kernels: scatter/gather between caller order and slot order
// ---------------------------------------------------------------------------
namespace {
// flag[0] = 1 if any of the count values is not finite
__global__ void k_any_nonfinite(int64_t count, const double* v, int* flag) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const bool bad = i < count && !isfinite(v[i]);
  if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(flag, 1);
}
__global__ void k_scatter_d(int64_t n, const int32_t* inv, const double* src, int comps,
                            double* dst, int stride, int off) {
  int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (o >= n) return;
  int64_t s = inv[o];
  for (int c = 0; c < comps; c++) dst[s * stride + off + c] = src[o * comps + c];
}
__global__ void k_gather_d(int64_t n, const int32_t* inv, const double* src, int stride, int off,
                           int comps, double* dst) {
  int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (o >= n) return;
  int64_t s = inv[o];
  for (int c = 0; c < comps; c++) dst[o * comps + c] = src[s * stride + off + c];
}
__global__ void k_gather_f(int64_t n, const int32_t* inv, const float* src, int stride, int off,
                           int comps, double* dst) {
  int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (o >= n) return;
  int64_t s = inv[o];
  for (int c = 0; c < comps; c++) dst[o * comps + c] = (double)src[s * stride + off + c];
}
// sigma = -p I + S from the FP32 deviatoric state (mixed form)
__global__ void k_gather_sigma32(int64_t n, const int32_t* inv, const float* ss32, const double* p,
                                 double* dst) {
  int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (o >= n) return;
  int64_t s = inv[o];
  for (int c = 0; c < 6; c++) dst[o * 6 + c] = (double)ss32[s * 6 + c] + (c < 3 ? -p[s] : 0.0);
}
template <class T>
__global__ void k_scatter_t(int64_t n, const int32_t* inv, const T* src, T* dst) {
  int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (o >= n) return;
  dst[inv[o]] = src[o];
}
template <class T>
__global__ void k_gather_t(int64_t n, const int32_t* inv, const T* src, T* dst) {
  int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (o >= n) return;
  dst[o] = src[inv[o]];
}
__global__ void k_fill_d(int64_t n, double v, double* dst, int stride, int off) {
  int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s < n) dst[s * stride + off] = v;
}
__global__ void k_iota(int64_t n, int32_t* a, int32_t* b) {
  int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s < n) { a[s] = (int32_t)s; b[s] = (int32_t)s; }
}
// neighbour lists in caller ids: lists[o*70+k] = perm[entry k of slot inv[o]]
__global__ void k_gather_nb(int64_t n, int64_t npad, const int32_t* inv, const int32_t* perm,
                            const int32_t* nb, const int32_t* cnt, int32_t* ocnt, int32_t* olst) {
  int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (o >= n) return;
  int64_t s = inv[o];
  int c = cnt[s];
  ocnt[o] = c;
  for (int k = 0; k < WF_NB; k++) olst[o * WF_NB + k] = k < c ? perm[nb[nb_at(npad, s, k)]] : -1;
}
// SetVelKernel (src/cuda/Mechanical.cu:154-163): v = 0 for solid particles
__global__ void k_setvel0(int64_t n, int64_t n_solid, Fields F) {
  int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= n) return;
  if (F.perm[s] < n_solid) {
    double4 v = F.vd[s];
    F.vd[s] = make_double4(0.0, 0.0, 0.0, v.w);
  }
}
// FP32 mirrors of the master state for the mixed form
__global__ void k_mixed_init(int64_t n, Fields F) {
  int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= n) return;
  double4 x = F.xm[s], v = F.vd[s];
  F.p32[s] = make_float4((float)x.x, (float)x.y, (float)x.z, (float)x.w);
  F.v32[s] = make_float4((float)v.x, (float)v.y, (float)v.z, (float)v.w);
  for (int c = 0; c < 6; c++) F.ss32[s * 6 + c] = (float)F.ss6[s * 6 + c];
  const double T = F.T[s];
  const float thi = (float)T;
  F.th32[s] = make_float2(thi, (float)(T - (double)thi));
}
// FP64 copy of the FP32 deviatoric state (mixed -> plain switch)
__global__ void k_mixed_to_fp64(int64_t n, Fields F) {
  int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= n) return;
  for (int c = 0; c < 6; c++) F.ss6[s * 6 + c] = (double)F.ss32[s * 6 + c];
}
// the rigid particles of a mesh (AddTrimeshParticles, Domain.cpp:969-990):
// at the element centroids, mass 0, the mesh's zone id, the element normal
__global__ void k_place_rigid(int32_t ne, int32_t first, const int32_t* inv,
                              const double4* centroid, const double4* normal, int32_t zone,
                              Fields F) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  const int32_t s = inv[first + e];
  const double4 c = centroid[e];
  F.xm[s] = make_double4(c.x, c.y, c.z, 0.0);
  F.id[s] = zone;
  F.nrm[s] = normal[e];
}
// the largest plastic-strain increment since the last rebuild: non-negative
// doubles order like their bit patterns.  Grid-stride over at most
// kMaxDepBlocks blocks, reduced per warp and then per block, so one 64-bit
// atomicMax per block (one per warp serialised 63k atomics on one address at
// 2M particles: 44 us).
constexpr int kMaxDepBlocks = 1024;
__global__ void __launch_bounds__(256) k_max_dep(int64_t n, const double* eps,
                                                 const double* eps_rb,
                                                 unsigned long long* out) {
  __shared__ unsigned long long wmax[8];
  unsigned long long b = 0ull;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double v = eps[i] - eps_rb[i];
    if (!(v > 0.0)) v = 0.0;
    const unsigned long long c = (unsigned long long)__double_as_longlong(v);
    b = c > b ? c : b;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long c = __shfl_xor_sync(0xffffffffu, b, o);
    b = c > b ? c : b;
  }
  if ((threadIdx.x & 31) == 0) wmax[threadIdx.x >> 5] = b;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); w++) b = wmax[w] > b ? wmax[w] : b;
    atomicMax(out, b);
  }
}
__global__ void k_copy_d(int64_t n, const double* src, double* dst) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) dst[i] = src[i];
}

// ---- debug checks (option debug_checks) ---------------------------------
// The stand-in for a bounds-checking sanitizer: after every neighbour
// rebuild each list is checked before any pair pass reads it (counts within
// [0, WF_NB], entries of other particles in [0, n), padding entries the
// particle's own slot); a bad entry is replaced by the own slot (which adds
// exact zeros) and WF_STATUS_CHECKS is set, so the passes that follow stay in
// bounds and the call reports the error.  After every step positions and
// velocities are checked for non-finite values.
__global__ void k_check_lists(int64_t n, int64_t npad, int32_t* __restrict__ nb,
                              int32_t* __restrict__ cnt, int* __restrict__ status) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  bool bad = false;
  int c = cnt[i];
  if (c < 0 || c > WF_NB) {
    bad = true;
    c = c < 0 ? 0 : WF_NB;
    cnt[i] = c;
  }
  const int cend = (c + WF_NB_BLK - 1) & ~(WF_NB_BLK - 1);
  for (int k = 0; k < cend; k++) {
    int32_t& e = nb[nb_at(npad, i, k)];
    const bool ok = k < c ? (e >= 0 && (int64_t)e < n && (int64_t)e != i) : (int64_t)e == i;
    if (!ok) {
      e = (int32_t)i;
      bad = true;
    }
  }
  if (bad) atomicOr(status, WF_STATUS_CHECKS);
}
__global__ void k_check_finite(int64_t n, const double4* __restrict__ xm,
                               const double4* __restrict__ vd, int* __restrict__ status) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double4 x = xm[i], v = vd[i];
  if (!(isfinite(x.x) && isfinite(x.y) && isfinite(x.z) && isfinite(v.x) && isfinite(v.y) &&
        isfinite(v.z) && isfinite(v.w)))
    atomicOr(status, WF_STATUS_CHECKS);
}
// fault injection for the checks' test: the first entry of one particle's
// list is set out of range, between the list build and k_check_lists
__global__ void k_inject_list_error(int64_t n, int64_t npad, int32_t slot, int32_t* nb,
                                    const int32_t* cnt) {
  if (blockIdx.x == 0 && threadIdx.x == 0 && slot >= 0 && slot < n && cnt[slot] > 0)
    nb[nb_at(npad, slot, 0)] = (int32_t)(n + 7);
}
inline int nblk(int64_t n, int t = 256) { return (int)((n + t - 1) / t); }
}  // namespace

// ---------------------------------------------------------------------------
// allocation
// ---------------------------------------------------------------------------
// Zero-filled on the domain's own stream: that stream is non-blocking, so a
// cudaMemset on the legacy default stream would not be ordered before it.
template <class T>
static cudaError_t dalloc(T** p, int64_t count, cudaStream_t s) {
  const size_t bytes = sizeof(T) * (size_t)std::max<int64_t>(count, 1);
  cudaError_t e = cudaMalloc((void**)p, bytes);
  if (e == cudaSuccess) e = cudaMemsetAsync(*p, 0, bytes, s);
  return e;
}

// One device allocation holds every fixed-size per-particle array of a domain
// (both field buffers, the mixed-form mirrors, the neighbour lists, the
// search's sort arrays): wf_create makes one cudaMalloc and one zero fill
// instead of ~90 of each, and wf_destroy one cudaFree.  Offsets are 256-byte
// aligned.  Arrays whose size is known later (contact, cell tables, logs)
// keep their own allocations.
struct Arena {
  uintptr_t base = 0;  // 0 in the sizing pass
  size_t off = 0;
  template <class T>
  void take(T** p, int64_t count) {
    off = (off + 255) & ~(size_t)255;
    *p = reinterpret_cast<T*>(base + off);
    off += sizeof(T) * (size_t)std::max<int64_t>(count, 1);
  }
};

static void layout_arena(wf_domain* d, Arena& A) {
  const int64_t n = d->npad;
  for (int k = 0; k < 2; k++) {
    Fields& F = d->F[k];
    A.take(&F.xm, n); A.take(&F.vd, n); A.take(&F.u, n); A.take(&F.a, n);
    A.take(&F.sig6, 6 * n); A.take(&F.ss6, 6 * n); A.take(&F.eps6, 6 * n);
    A.take(&F.sr6, 6 * n); A.take(&F.rr6, 6 * n);
    A.take(&F.p, n); A.take(&F.seq, n); A.take(&F.eps_p, n); A.take(&F.sy, n);
    A.take(&F.eff, n); A.take(&F.dep, n); A.take(&F.drho, n); A.take(&F.eint, n);
    A.take(&F.T, n); A.take(&F.Ta, n); A.take(&F.Tb, n); A.take(&F.dTdt, n);
    A.take(&F.kT, n); A.take(&F.cpT, n);
    A.take(&F.id, n); A.take(&F.bct, n); A.take(&F.perm, n); A.take(&F.nw, n);
    A.take(&F.xh, n); A.take(&F.p32, n); A.take(&F.v32, n); A.take(&F.ss32, 6 * n);
    A.take(&F.th32, n); A.take(&F.pwn, n); A.take(&F.p32n, n);
  }
  A.take(&d->vd2, n); A.take(&d->v32b, n); A.take(&d->a32, n); A.take(&d->sigr32, 8 * n);
  A.take(&d->nb, (int64_t)WF_NB_ALLOC * n); A.take(&d->nbc, n); A.take(&d->inv, n);
  A.take(&d->pf, n); A.take(&d->pf2, n); A.take(&d->cellid, n); A.take(&d->s_src, n);
  A.take(&d->s_orig, n); A.take(&d->d_mm, 8); A.take(&d->d_status, WF_STATUS_WORDS);
  A.take(&d->d_cstat, 2);
  A.take(&d->fr, n); A.take(&d->out_part, wf_out_partial_words(WF_MAX_BC));
  A.take(&d->e0, 1);
  d->t_halo_cap = 10 * n;      // halo entries: ~7 per slot on cell-sorted lattices
  A.take(&d->t_hoff, n / WF_TILE); A.take(&d->t_hcnt, n / WF_TILE);
  A.take(&d->t_halo, d->t_halo_cap); A.take(&d->t_nbl, (int64_t)WF_NB_ALLOC * n);
  A.take(&d->l16_base, n / WF_TILE); A.take(&d->l16_off, (int64_t)WF_NB_ALLOC * n);
  A.take(&d->out_last, WF_ROW_FIXED + 3 * WF_MAX_BC); A.take(&d->series_count, 1);
  A.take(&d->d_stage, 6 * n); A.take(&d->d_stage2, 6 * n); A.take(&d->mlp_w, WF_MLP_NPARAM);
  A.take(&d->mlp_packed, (int64_t)wf_mlp_packed_bytes());
}

// the field arrays allocated on demand (contact, adaptive rebuild)
static void free_fields(Fields& F) {
  void* ptrs[] = {F.nrm, F.cf, F.qf, F.eps_rb};
  for (void* p : ptrs) if (p) cudaFree(p);
  F = Fields{};
}

// ---------------------------------------------------------------------------
// parameters
// ---------------------------------------------------------------------------
// ---------------------------------------------------------------------------
// arena cache
// ---------------------------------------------------------------------------
// wf_destroy keeps the last domain's arena (and its page-locked status words)
// here instead of freeing them, and the next wf_create on the same device
// whose layout needs between 80 and 100 % of it takes it over (zeroed on its
// stream like a fresh one).  cudaMalloc and cudaFree of the ~1 GB arena of a
// 786k-particle domain cost ~0.5 ms each, paid by every drop-in call that
// creates and destroys its domain.  A cached block that does not fit is freed
// before the new allocation; wf_release_cache() frees the cache.
struct ArenaCache {
  char* arena = nullptr;
  size_t bytes = 0;
  int dev = -1;
  int* h_status = nullptr;
};
static std::mutex g_cache_mu;
static ArenaCache g_cache;

static void cache_free_locked() {
  if (g_cache.arena) {
    int cur = 0;
    cudaGetDevice(&cur);
    cudaSetDevice(g_cache.dev);
    cudaFree(g_cache.arena);
    cudaSetDevice(cur);
  }
  if (g_cache.h_status) cudaFreeHost(g_cache.h_status);
  g_cache = ArenaCache{};
}
static void cache_take(wf_domain* d) {
  std::lock_guard<std::mutex> lk(g_cache_mu);
  if (!g_cache.arena) return;
  if (g_cache.dev != d->dev || g_cache.bytes < d->arena_bytes ||
      g_cache.bytes > d->arena_bytes + d->arena_bytes / 4) {
    cache_free_locked();
    return;
  }
  d->arena = g_cache.arena;
  d->arena_alloc = g_cache.bytes;
  d->h_status = g_cache.h_status;
  g_cache = ArenaCache{};
}
static void cache_put(wf_domain* d) {
  if (!d->arena) return;
  std::lock_guard<std::mutex> lk(g_cache_mu);
  cache_free_locked();                       // keep the most recent one
  g_cache.arena = d->arena;
  g_cache.bytes = d->arena_alloc;
  g_cache.dev = d->dev;
  g_cache.h_status = d->h_status;
  d->arena = nullptr;
  d->h_status = nullptr;
}

static StepParams make_params(const wf_domain* d) {
  StepParams P;
  memset(&P, 0, sizeof P);
  P.n = d->n;
  P.n_solid = d->n_solid;
  P.npad = d->npad;
  P.h = d->h;
  P.gkC = 1.0 / (d->h * d->h * d->h * d->h * WF_PI);   // Functions.cu:83 with h_ = h
  P.dt = d->dt;
  P.Cs = d->Cs;
  P.G = d->G;
  P.rho0 = d->rho0;
  P.alpha = d->alpha;
  P.beta = d->beta;
  P.chi = d->chi;
  P.h_conv = d->h_conv;
  P.T_inf = d->T_inf;
  P.return_map = d->return_map;
  P.newton_max_iter = d->newton_max_iter;
  P.newton_rtol = d->newton_rtol;
  P.clamp_homologous = d->clamp_homologous;
  P.energy_mode = d->energy_mode;
  P.e0 = d->e0;
  P.inv = d->inv;
  P.contact = d->meshes.empty() ? 0 : 1;
  P.ncsid = (int)d->meshes.size();
  for (int m = 0; m < P.ncsid; m++) {
    P.mesh[m] = d->meshes[m];
    P.csid[m] = d->meshes[m].zone;
  }
  P.mu_s = d->mu_s;
  P.mu_d = d->mu_d;
  P.contact_law = d->contact_law;
  P.c_kappa = d->c_kappa;
  P.c_dx = d->c_dx;
  P.c_vreg = d->c_vreg;
  P.c_eta = d->c_eta;
  P.Kbulk = d->mat.E / (3.0 * (1.0 - 2.0 * d->mat.nu));
  P.totmass = d->totmass;
  P.id_free_surf = 1;              // MechFraserSolve, SolverFraser.cu:118
  P.cnb = d->cnb;
  P.ccnt = d->ccnt;
  P.cstat = d->d_cstat;
  P.nbc = (int)d->bc_zone.size();
  for (int b = 0; b < P.nbc; b++) {
    P.bc_zone[b] = d->bc_zone[b];
    for (int c = 0; c < 3; c++) P.bc_v[b][c] = d->bc_v[b][c];
  }
  P.mlp_on = d->mlp_on;
  P.nb_pf = d->list_prefetch;
  P.state_pf = d->state_prefetch;
  P.wave_pf = d->wave_prefetch;
  P.wave_dist = d->wave_dist;
  const wf_material& m = d->mat;
  MatParams& M = P.mat;
  M.model = m.model;
  M.E = m.E;
  M.Et = m.Et;
  M.Ep = (m.model == WF_BILINEAR) ? m.E * m.Et / (m.E - m.Et) : 0.0;   // WeldFormGPU.cu:755
  M.K_hol = m.K_hol;
  M.m_hol = m.m_hol;
  M.sy0 = m.sy0;
  if (m.model == WF_HOLLOMON) {                                       // Material.cuh:116-130
    M.eps0_hol = m.sy0 / m.E;
    M.eps1_hol = std::pow(m.sy0 / m.K_hol, 1. / m.m_hol);
  }
  M.A = m.A; M.B = m.B; M.n = m.n; M.C = m.C; M.eps0 = m.eps0; M.m = m.m; M.Tm = m.Tm; M.Tt = m.Tt;
  {  // C(n, k) for (1 + u)^n, k = 1..5
    double c = 1.0;
    for (int k = 1; k <= 5; k++) {
      c = c * (m.n - (k - 1)) / k;
      M.bin[k - 1] = c;
    }
  }
  P.refresh_pow = (d->step % 64) == 0;   // bounds the drift of the cached eps_p^n
  P.log_cap = d->log_cap;
  P.log_count = d->log_count;
  P.log_x = d->log_x;
  P.log_y = d->log_y;
  P.hf = (float)P.h;
  P.invhf = (float)(1.0 / P.h);
  P.Cf = (float)P.gkC;
  P.Chf = (float)(P.gkC / P.h);
  P.Csf = (float)P.Cs;
  P.k2f = (float)(2.0 * d->k_cond);
  P.alphaf = (float)P.alpha;
  P.betaf = (float)P.beta;
  P.epsf = (float)(0.01 * P.h * P.h);
  P.dtf = (float)P.dt;
  P.G2f = (float)(2.0 * P.G);
  P.G3f = (float)(3.0 * P.G);
  P.jcAf = (float)M.A;
  P.jcBf = (float)M.B;
  P.jcnf = (float)M.n;
  for (int k = 0; k < 5; k++) P.binf[k] = (float)M.bin[k];
  P.jcTtf = (float)M.Tt;
  P.jcinvdTf = (float)(1.0 / (M.Tm - M.Tt));
  P.jcCf = (float)M.C;
  P.jcinveps0f = (float)(1.0 / M.eps0);
  P.jcmf = (float)M.m;
  P.chif = (float)P.chi;
  P.h_convf = (float)P.h_conv;
  P.T_inff = (float)P.T_inf;
  return P;
}

// ---------------------------------------------------------------------------
// measurement helpers: optional event pairs around one kernel kind
// ---------------------------------------------------------------------------
// Step-segment graphs.  The launches of the steps between two host
// synchronisation points (a neighbour rebuild, which reads the particle
// bounds back to size the cell grid; a status read; the end of a call) are
// recorded by stream capture and replayed as one CUDA graph: capture takes
// the kernels with the arguments the steps would have launched them with
// (the position buffers that alternate from step to step included), so the
// replay does the same work in the same order.  The instantiated graph is
// kept and updated in place when the next segment has the same launches.
// Not used with the adaptive rebuild or CSV snapshots (host reads every step).
static int segment_begin(wf_domain* d) {
  if (!d->graph || d->capturing || d->rb_dep > 0.0 || d->csv_on || d->after_fn) return WF_OK;
  WF_CUDA_OK(cudaStreamBeginCapture(d->stream, cudaStreamCaptureModeRelaxed));
  d->capturing = true;
  return WF_OK;
}

static int segment_end(wf_domain* d) {
  if (!d->capturing) return WF_OK;
  d->capturing = false;
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(d->stream, &g);
  if (e != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return wf_cuda_fail(d, e, "cudaStreamEndCapture");
  }
  size_t nodes = 0;
  cudaGraphGetNodes(g, nullptr, &nodes);
  if (nodes == 0) {
    cudaGraphDestroy(g);
    return WF_OK;
  }
  bool updated = false;
  if (d->gexec) {
    cudaGraphExecUpdateResultInfo info;
    updated = cudaGraphExecUpdate(d->gexec, g, &info) == cudaSuccess;
    if (!updated) {
      cudaGetLastError();   // a failed update is not an error: instantiate anew
      cudaGraphExecDestroy(d->gexec);
      d->gexec = nullptr;
    }
  }
  if (!updated) {
    e = cudaGraphInstantiate(&d->gexec, g, 0);
    if (e != cudaSuccess) {
      d->gexec = nullptr;
      cudaGraphDestroy(g);
      return wf_cuda_fail(d, e, "cudaGraphInstantiate");
    }
    d->graph_instantiations++;
  }
  cudaGraphDestroy(g);
  WF_CUDA_OK(cudaGraphLaunch(d->gexec, d->stream));
  d->graph_launches++;
  return WF_OK;
}

// Inside a step segment the timing events become event-record nodes of the
// graph (the external flag, valid only while capturing); outside, plain records.
static void record(wf_domain* d, cudaEvent_t e) {
  if (d->capturing) cudaEventRecordWithFlags(e, d->stream, cudaEventRecordExternal);
  else cudaEventRecord(e, d->stream);
}

struct KTimer {
  wf_domain* d;
  int kid;
  bool on;
  KTimer(wf_domain* d_, int kid_)
      : d(d_), kid(kid_), on(d_->timing && d_->profile_kernel == kid_) {
    nvtxRangePushA(kStageNames[kid_]);
    if (on) {
      if (d->ev_used + 2 > d->ev_pool.size()) {
        for (int k = 0; k < 64; k++) {
          cudaEvent_t e;
          cudaEventCreate(&e);
          d->ev_pool.push_back(e);
        }
      }
      record(d, d->ev_pool[d->ev_used]);
    }
  }
  ~KTimer() {
    if (on) {
      record(d, d->ev_pool[d->ev_used + 1]);
      d->ev_used += 2;
    }
    nvtxRangePop();
  }
};

// ---------------------------------------------------------------------------
// neighbour rebuild (cuNSearch find_neighbors equivalent) + reorder
// ---------------------------------------------------------------------------
static int ensure_cells(wf_domain* d, int64_t ncell) {
  if (ncell + 1 <= d->cell_cap) return WF_OK;
  if (d->cell_count) { cudaFree(d->cell_count); cudaFree(d->cell_cursor); cudaFree(d->scan_tmp); }
  int64_t cap = (ncell + 1) + (ncell + 1) / 4 + 1024;
  WF_CUDA_OK(dalloc(&d->cell_count, cap, d->stream));
  WF_CUDA_OK(dalloc(&d->cell_cursor, cap, d->stream));
  d->scan_cap = scan_tmp_words(cap) + 16;
  WF_CUDA_OK(dalloc(&d->scan_tmp, d->scan_cap, d->stream));
  d->cell_cap = cap;
  return WF_OK;
}

constexpr int kReorderEvery = 20;   // physical reorder at every 20th rebuild of a solve

static int rebuild(wf_domain* d, bool use_current, bool light = false) {
  {
    const int rc = segment_end(d);
    if (rc) return rc;
  }
  KTimer t(d, KID_REBUILD);
  const int64_t n = d->n;
  cudaStream_t s = d->stream;
  Fields& A = d->F[d->cur];
  Fields& B = d->F[1 - d->cur];
  launch_prep_positions(n, A, use_current ? 1 : 0, d->pf, s);
  int mm_init[6] = {INT_MAX, INT_MAX, INT_MAX, INT_MIN, INT_MIN, INT_MIN};
  WF_CUDA_OK(cudaMemcpyAsync(d->d_mm, mm_init, sizeof mm_init, cudaMemcpyHostToDevice, s));
  const float r = (float)(2.0 * d->h);                // SolverFraser.cu:72-82
  launch_minmax(n, d->pf, r, d->d_mm, s);
  int mm[8];   // bounds, then the largest halo of the previous tile build
  WF_CUDA_OK(cudaMemcpyAsync(mm, d->d_mm, sizeof mm, cudaMemcpyDeviceToHost, s));
  WF_CUDA_OK(cudaStreamSynchronize(s));
  if (d->tile_cap > 0) d->tile_hmax = mm[6];
  grid_from_minmax(mm, r, &d->grid);
  const int64_t ncell = (int64_t)d->grid.dim[0] * d->grid.dim[1] * d->grid.dim[2];
  if (ncell > (int64_t)2000000000) return wf_fail(d, WF_ERR_NUMERIC, "neighbour grid too large");
  int rc = ensure_cells(d, ncell);
  if (rc) return rc;
  WF_CUDA_OK(cudaMemsetAsync(d->cell_count, 0, sizeof(uint32_t) * (ncell + 1), s));
  WF_CUDA_OK(cudaMemsetAsync(d->cell_cursor, 0, sizeof(uint32_t) * (ncell + 1), s));
  launch_cell_count(n, d->pf, d->grid, d->cellid, d->cell_count, d->d_status, s);
  device_exclusive_scan(d->cell_count, ncell + 1, d->scan_tmp, s);
  launch_cell_scatter(n, d->cellid, d->cell_count, d->cell_cursor, A.perm, d->s_src, d->s_orig, s);
  launch_cell_sort(ncell, d->cell_count, d->s_src, d->s_orig, s);
  // The lists hold the same particles in the same order whether or not the
  // state is moved into the sorted order, so the arithmetic is identical;
  // moving it keeps warps' particles close in space.  Inside the step loop
  // the state is moved at every kReorderEvery-th rebuild only (solids move
  // little in between); otherwise the lists name the particles' current slots.
  const bool full = !light || ++d->light_rebuilds >= kReorderEvery;
  if (full) {
    launch_reorder(n, d->s_src, A, B, d->pf, d->pf2, d->inv, s);
    d->cur = 1 - d->cur;
    d->light_rebuilds = 0;
  } else {
    launch_gather_pf(n, d->s_src, d->pf, d->pf2, s);
  }
  launch_nblist(n, d->npad, d->pf2, d->grid, d->cell_count, full ? nullptr : d->s_src, d->nb,
                d->nbc, d->d_status, s);
  d->launches += 8;
  if (d->debug_checks) {
    if (d->inject_list_error >= 0) {
      int32_t slot = -1;
      WF_CUDA_OK(cudaMemcpyAsync(&slot, d->inv + d->inject_list_error, sizeof slot,
                                 cudaMemcpyDeviceToHost, s));
      WF_CUDA_OK(cudaStreamSynchronize(s));
      k_inject_list_error<<<1, 32, 0, s>>>(n, d->npad, slot, d->nb, d->nbc);
      d->inject_list_error = -1;                // once
    }
    k_check_lists<<<nblk(n), 256, 0, s>>>(n, d->npad, d->nb, d->nbc, d->d_status);
    d->launches += 1;
  }
  // tile halos for the staged mixed passes, sized by the previous build's
  // largest halo (tiles with larger halos gather from global memory)
  d->l16_built = false;
  if (d->precision == 1 && d->list16) {
    launch_list16(n, d->npad, d->nb, d->nbc, d->l16_base, d->l16_off, s);
    d->l16_built = true;
    d->launches += 1;
  }
  d->tile_cap = 0;
  if (d->precision == 1 && d->tile_staging && d->meshes.empty()) {
    int cap = d->tile_hmax > 0 ? ((d->tile_hmax + 31) / 32) * 32 : 1536;
    cap = std::min(std::max(cap, std::min(256, d->tile_cap_max)), d->tile_cap_max);
    WF_CUDA_OK(cudaMemsetAsync(d->d_mm + 6, 0, 2 * sizeof(int), s));
    launch_tile_halo(n, d->npad, d->nb, d->nbc, d->t_hoff, d->t_hcnt, d->t_halo, d->t_halo_cap,
                     d->t_nbl, cap, reinterpret_cast<unsigned*>(d->d_mm + 7), d->d_mm + 6, s);
    d->tile_cap = cap;
    d->launches += 1;
  }
  if (d->F[d->cur].eps_rb) {       // adaptive rebuild: the strain this list was built at
    k_copy_d<<<nblk(n), 256, 0, s>>>(n, d->F[d->cur].eps_p, d->F[d->cur].eps_rb);
    d->launches += 1;
  }
  WF_CUDA_OK(cudaGetLastError());
  d->nb_built = true;
  return WF_OK;
}

// The triangles of each tool binned once in the tool's frame as it stands
// now (contact law 1): cells of 2h over the tool's box grown by h, each
// triangle listed in every cell its box grown by h touches (ascending
// triangle index within a cell), so every triangle within h of a point is
// listed in the point's cell.
static int build_tool_bins(wf_domain* d) {
  const double cs = 2.0 * d->h, margin = d->h * (1.0 + 1e-6) + 1e-12;
  for (MeshDev& M : d->meshes) {
    std::vector<double4> nd(M.nn);
    std::vector<int32_t> en(3 * (size_t)M.ne);
    WF_CUDA_OK(cudaMemcpyAsync(nd.data(), M.node, sizeof(double4) * M.nn, cudaMemcpyDeviceToHost, d->stream));
    WF_CUDA_OK(cudaMemcpyAsync(en.data(), M.elnode, sizeof(int32_t) * 3 * M.ne, cudaMemcpyDeviceToHost, d->stream));
    WF_CUDA_OK(cudaStreamSynchronize(d->stream));
    // node coordinates relative to node 0
    std::vector<double> rel(3 * (size_t)M.nn);
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300}, ext = 0.0, rmax = 0.0;
    for (int q = 0; q < M.nn; q++) {
      const double c[3] = {nd[q].x - nd[0].x, nd[q].y - nd[0].y, nd[q].z - nd[0].z};
      for (int k = 0; k < 3; k++) {
        rel[3 * q + k] = c[k];
        lo[k] = std::min(lo[k], c[k]);
        hi[k] = std::max(hi[k], c[k]);
        ext = std::max(ext, std::fabs(c[k]));
      }
      rmax = std::max(rmax, std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]));
    }
    M.rot = (M.mw[0] != 0.0 || M.mw[1] != 0.0 || M.mw[2] != 0.0) ? 1 : 0;
    if (M.rot) {
      // a box around node 0 that holds the tool in any orientation (the
      // distances to node 0 do not change under the rigid motion; 1 % spare)
      const double R = 1.01 * rmax;
      for (int k = 0; k < 3; k++) { lo[k] = -R; hi[k] = R; }
      ext = std::max(ext, R);
    }
    int64_t ncell = 1;
    for (int k = 0; k < 3; k++) {
      M.grel[k] = lo[k] - margin - cs;
      M.dims[k] = (int32_t)std::ceil((hi[k] + margin + cs - M.grel[k]) / cs) + 1;
      ncell *= M.dims[k];
    }
    if (ncell > (int64_t)64 << 20) return wf_fail(d, WF_ERR_ARG, "tool bin grid too large");
    M.cs = cs;
    M.inv_cs = 1.0 / cs;
    M.margin = margin;
    for (int k = 0; k < 3; k++) {
      M.glo[k] = (float)(M.grel[k] - cs);
      M.ghi[k] = (float)(M.grel[k] + (M.dims[k] + 1) * cs);
    }
    if (!M.off32 && dalloc(&M.off32, 1, d->stream) != cudaSuccess)
      return wf_fail(d, WF_ERR_ALLOC, "tool offset");
    const float4 o = make_float4((float)nd[0].x, (float)nd[0].y, (float)nd[0].z, 0.f);
    WF_CUDA_OK(cudaMemcpyAsync(M.off32, &o, sizeof(float4), cudaMemcpyHostToDevice, d->stream));
    // FP32 search tolerance: 1e-3 h plus 1e-6 of the tool's extent (16 FP32
    // ulps of the largest relative coordinate), far above the FP32 distance error
    M.tol32 = (float)(1e-3 * d->h + 1e-6 * (ext + 2.0 * d->h));
    for (void* p : {(void*)M.cstart, (void*)M.ctri, (void*)M.cvert, (void*)M.cursor, (void*)M.scan_tmp})
      if (p) cudaFree(p);
    M.cstart = nullptr; M.ctri = nullptr; M.cvert = nullptr; M.cursor = nullptr; M.scan_tmp = nullptr;
    if (M.rot) {
      // entries: a triangle's box spans at most its diameter along any axis in
      // any orientation, so it touches at most (floor((D + 2 margin)/cs) + 2)^3 cells
      int64_t cap = 0;
      for (int e = 0; e < M.ne; e++) {
        double dia = 0.0;
        for (int a1 = 0; a1 < 3; a1++)
          for (int a2 = a1 + 1; a2 < 3; a2++) {
            const double* p1 = &rel[3 * en[3 * e + a1]];
            const double* p2 = &rel[3 * en[3 * e + a2]];
            dia = std::max(dia, std::sqrt((p1[0] - p2[0]) * (p1[0] - p2[0]) + (p1[1] - p2[1]) * (p1[1] - p2[1]) +
                                          (p1[2] - p2[2]) * (p1[2] - p2[2])));
          }
        const int64_t span = (int64_t)std::floor((dia + 2.0 * margin) / cs) + 2;
        cap += span * span * span;
      }
      M.cap = cap;
      if (dalloc(&M.cstart, ncell + 1, d->stream) || dalloc(&M.cursor, ncell, d->stream) ||
          dalloc(&M.scan_tmp, scan_tmp_words(ncell + 1), d->stream) ||
          dalloc(&M.cvert, 3 * cap, d->stream))
        return wf_fail(d, WF_ERR_ALLOC, "rotating tool bins");
      continue;   // binned on the GPU before every contact stage
    }
    std::vector<int32_t> start((size_t)ncell + 1, 0), list;
    auto range = [&](int e, int r0[3], int r1[3]) {
      for (int k = 0; k < 3; k++) {
        double a = 1e300, b = -1e300;
        for (int q = 0; q < 3; q++) {
          const double c = rel[3 * en[3 * e + q] + k];
          a = std::min(a, c);
          b = std::max(b, c);
        }
        r0[k] = std::max(0, (int)std::floor((a - margin - M.grel[k]) / cs));
        r1[k] = std::min(M.dims[k] - 1, (int)std::floor((b + margin - M.grel[k]) / cs));
      }
    };
    for (int pass = 0; pass < 2; pass++) {
      std::vector<int32_t> fill;
      if (pass == 1) {
        for (int64_t c = 0; c < ncell; c++) start[c + 1] += start[c];
        list.resize(start[ncell]);
        fill.assign(start.begin(), start.end() - 1);
      }
      for (int e = 0; e < M.ne; e++) {
        int r0[3], r1[3];
        range(e, r0, r1);
        for (int z = r0[2]; z <= r1[2]; z++)
          for (int y = r0[1]; y <= r1[1]; y++)
            for (int x = r0[0]; x <= r1[0]; x++) {
              const int64_t c = ((int64_t)z * M.dims[1] + y) * M.dims[0] + x;
              if (pass == 0) start[c + 1]++;
              else list[fill[c]++] = e;
            }
      }
    }
    M.cap = (int64_t)list.size();
    if (dalloc(&M.cstart, ncell + 1, d->stream) || dalloc(&M.ctri, std::max<int64_t>(1, (int64_t)list.size()), d->stream))
      return wf_fail(d, WF_ERR_ALLOC, "tool bins");
    WF_CUDA_OK(cudaMemcpyAsync(M.cstart, start.data(), sizeof(int32_t) * (ncell + 1), cudaMemcpyHostToDevice, d->stream));
    if (!list.empty())
      WF_CUDA_OK(cudaMemcpyAsync(M.ctri, list.data(), sizeof(int32_t) * list.size(), cudaMemcpyHostToDevice, d->stream));
    // each entry carries its triangle's FP32 vertices relative to node 0
    std::vector<float4> cv(3 * std::max<size_t>(1, list.size()));
    for (size_t t = 0; t < list.size(); t++) {
      const int e = list[t];
      for (int k = 0; k < 3; k++) {
        const double* p = &rel[3 * en[3 * e + k]];
        float w = 0.f;
        if (k == 0) memcpy(&w, &e, sizeof w);   // the triangle index's bits
        cv[3 * t + k] = make_float4((float)p[0], (float)p[1], (float)p[2], w);
      }
    }
    if (dalloc(&M.cvert, (int64_t)cv.size(), d->stream) != cudaSuccess)
      return wf_fail(d, WF_ERR_ALLOC, "tool bin vertices");
    WF_CUDA_OK(cudaMemcpyAsync(M.cvert, cv.data(), sizeof(float4) * cv.size(), cudaMemcpyHostToDevice,
                               d->stream));
    WF_CUDA_OK(cudaStreamSynchronize(d->stream));
  }
  d->bins_built = true;
  return WF_OK;
}

// ---------------------------------------------------------------------------
// the Fraser loop (SolverFraser.cu:30-409)
// ---------------------------------------------------------------------------
static int check_ready(wf_domain* d) {
  if (!d->h_set) return wf_fail(d, WF_ERR_STATE, "Set_h not called");
  if (!d->x_set) return wf_fail(d, WF_ERR_STATE, "positions not set");
  if (!d->m_set) return wf_fail(d, WF_ERR_STATE, "masses not set");
  if (!d->rho_set) return wf_fail(d, WF_ERR_STATE, "SetDensity not called");
  if (!(d->dt > 0)) return wf_fail(d, WF_ERR_STATE, "time step not set");
  if (!d->mat_set) return wf_fail(d, WF_ERR_STATE, "material not set");
  if (!d->cs_set) return wf_fail(d, WF_ERR_STATE, "SetCs not called");
  if (!d->G_set) return wf_fail(d, WF_ERR_STATE, "SetShearModulus not called");
  return WF_OK;
}

static int read_status(wf_domain* d) {
  {
    const int rc = segment_end(d);
    if (rc) return rc;
  }
  WF_CUDA_OK(cudaMemcpyAsync(d->h_status, d->d_status, WF_STATUS_WORDS * sizeof(int),
                             cudaMemcpyDeviceToHost, d->stream));
  WF_CUDA_OK(cudaStreamSynchronize(d->stream));
  return WF_OK;
}

// out_<time>.csv as MechFraserSolve writes it (SolverFraser.cu:142-144, 357-360)
extern "C" int wf_write_csv(wf_domain* d, const char* path);
static void flush_heat(wf_domain* d);
static int write_snapshot(wf_domain* d) {
  flush_heat(d);
  char name[64];
  snprintf(name, sizeof name, "out_%.6f.csv", d->time);
  return wf_write_csv(d, (d->csv_prefix + name).c_str());
}

static int write_series_csv(wf_domain* d, const char* path);

// MechFraserSolve's lines at an output time (SolverFraser.cu:369-388), from
// the device-reduced row, plus each BC zone's force
static int print_output_row(wf_domain* d) {
  const int rc = segment_end(d);
  if (rc) return rc;
  const int nbc = (int)d->bc_zone.size();
  std::vector<double> r(WF_ROW_FIXED + 3 * nbc);
  WF_CUDA_OK(cudaMemcpyAsync(r.data(), d->out_last, sizeof(double) * r.size(),
                             cudaMemcpyDeviceToHost, d->stream));
  WF_CUDA_OK(cudaStreamSynchronize(d->stream));
  printf("-------------------------\nTime %g\n", r[0]);
  printf("Current step: %lld, time: %g\n", (long long)r[1], d->dt);
  printf("Max disp: %g, %g, %g\n", r[2], r[3], r[4]);
  printf("Max pl_strain: %g\n", r[5]);
  if (!d->meshes.empty()) printf("Contact Force Sum: %g\n", r[6]);
  for (int b = 0; b < nbc; b++)
    printf("BC %d (zone %d) force: %g, %g, %g\n", b, d->bc_zone[b], r[WF_ROW_FIXED + 3 * b],
           r[WF_ROW_FIXED + 3 * b + 1], r[WF_ROW_FIXED + 3 * b + 2]);
  fflush(stdout);
  return WF_OK;
}

static int solve_begin(wf_domain* d, double dt_out) {
  int rc = check_ready(d);
  if (rc) return rc;
  const bool resume = d->resume != 0;
  if (!resume) {
    d->time = 0.0;
    d->isfirst = true;
    d->step = 0;
  }
  d->t_out = d->time + dt_out;
  d->dt_out = dt_out;
  d->ts_i = 0;
  d->is_yielding = false;
  {
    const int64_t width = WF_ROW_FIXED + 3 * (int64_t)d->bc_zone.size();
    if (!d->series || width != d->series_width) {
      if (d->series) cudaFree(d->series);
      d->series = nullptr;
      if (dalloc(&d->series, d->series_cap * width, d->stream) != cudaSuccess) {
        d->series = nullptr;
        return wf_fail(d, WF_ERR_ALLOC, "output series");
      }
      d->series_width = width;
      WF_CUDA_OK(cudaMemsetAsync(d->series_count, 0, sizeof(unsigned long long), d->stream));
    }
    if (!resume) {
      WF_CUDA_OK(cudaMemsetAsync(d->series_count, 0, sizeof(unsigned long long), d->stream));
      d->row_recorded = false;
    }
  }
  WF_CUDA_OK(cudaMemsetAsync(d->d_status, 0, WF_STATUS_WORDS * sizeof(int), d->stream));
  launch_snapshot(d->n, d->F[d->cur], d->stream);               // x_h = x, :56
  rc = rebuild(d, false);                                       // :109
  if (rc) return rc;
  if (!resume) k_setvel0<<<nblk(d->n), 256, 0, d->stream>>>(d->n, d->n_solid, d->F[d->cur]);   // :123
  if (!d->meshes.empty()) {
    // WeldFormGPU.cu:808-820: the masses summed in index order (rigid particles
    // hold mass 0 since wf_add_trimesh placed them)
    std::vector<double> hm((size_t)d->n);
    rc = wf_get_field(d, "m", hm.data());
    if (rc) return rc;
    d->totmass = 0.0;
    for (double mm : hm) d->totmass += mm;
    launch_mesh_plane(make_params(d), d->stream);  // CalcSpheresKernel, :129-141
    if (d->contact_law == 1) {
      if (!(d->c_dx > 0.0)) return wf_fail(d, WF_ERR_STATE, "contact law 1 needs the option contact_dx");
      for (const MeshDev& M : d->meshes)
        if (M.ne >= (1 << 24))
          return wf_fail(d, WF_ERR_ARG, "contact law 1 takes meshes of fewer than 2^24 triangles");
      if (!d->bins_built) {
        rc = build_tool_bins(d);
        if (rc) return rc;
      }
    }
  }
  if (d->precision == 1) k_mixed_init<<<nblk(d->n), 256, 0, d->stream>>>(d->n, d->F[d->cur]);
  WF_CUDA_OK(cudaGetLastError());
  d->started = true;
  if (d->csv_on) return write_snapshot(d);
  return WF_OK;
}

static int solve_step_launches(wf_domain* d) {
  cudaStream_t s = d->stream;
  bool rb;
  if (d->rb_dep > 0.0) {
    // adaptive: rebuild once the plastic strain grew by rb_dep anywhere since
    // the last rebuild (one device reduction and a 8-byte read per step)
    const Fields& F0 = d->F[d->cur];
    WF_CUDA_OK(cudaMemsetAsync(d->d_maxdep, 0, sizeof(unsigned long long), s));
    k_max_dep<<<std::min(nblk(d->n), kMaxDepBlocks), 256, 0, s>>>(d->n, F0.eps_p, F0.eps_rb,
                                                                 d->d_maxdep);
    WF_CUDA_OK(cudaMemcpyAsync(d->h_maxdep, d->d_maxdep, sizeof(unsigned long long),
                               cudaMemcpyDeviceToHost, s));
    WF_CUDA_OK(cudaStreamSynchronize(s));
    double mx;
    memcpy(&mx, d->h_maxdep, sizeof mx);
    d->launches += 1;
    rb = mx > d->rb_dep;
  } else {
    rb = d->ts_i == 0 && (d->is_yielding || !d->rebuild_after_yield);   // :166-182
  }
  if (d->lists_stale) {
    // positions were replaced after the solve started (wf_set_positions or a
    // checkpoint restore): new lists for them before this step
    launch_snapshot(d->n, d->F[d->cur], s);
    int rc = rebuild(d, false, true);
    if (rc) return rc;
    d->lists_stale = false;
    d->rebuilds++;
  } else if (rb) {
    int rc = rebuild(d, d->rebuild_current != 0, true);
    if (rc) return rc;
    d->rebuilds++;
  }
  {
    const int rc = segment_begin(d);
    if (rc) return rc;
  }
  StepParams P = make_params(d);
  // an output row is due after this step: the integration records the BC forces
  const bool row_due = d->out_every_step || d->time + d->dt >= d->t_out;
  if (row_due) P.fr = d->fr;
  const Fields& F = d->F[d->cur];
  NbBuffers N{d->nb, d->nbc};
  const bool mixed = d->precision == 1;
  bool integrated = false;
  const TileHalo TH{d->t_hoff, d->t_hcnt, d->t_halo, d->t_nbl,
                    (mixed && d->tile_staging && !P.contact) ? d->tile_cap : 0};
  const List16 L16{(mixed && d->list16 && d->l16_built) ? d->l16_base : nullptr, d->l16_off};
  if (!mixed) {
    { KTimer t(d, KID_DENSITY); launch_fp64_density(P, F, d->vd2, N, s); }          // :193-202
    { KTimer t(d, KID_STRESS); launch_fp64_stress(P, F, d->vd2, N, d->d_status, s); }  // :204-218
    { KTimer t(d, KID_ACCEL); launch_fp64_accel(P, F, d->vd2, N, s); }               // :221
  } else {
    {
      KTimer t(d, KID_DENSITY);
      if (d->heat_pending)
        launch_fp32_density_heat(P, F, d->vd2, d->v32b, N, d->heat_pending_first ? 1 : 0,
                                 d->chi > 0.0 ? 1 : 0, TH, L16, s);
      else
        launch_fp32_density(P, F, d->vd2, d->v32b, N, L16, s);
      d->heat_pending = false;
    }
    { KTimer t(d, KID_STRESS);
      launch_fp32_stress(P, F, d->v32b, d->sigr32, N, d->d_status,
                         (d->mlp_on && d->mlp_loaded) ? d->mlp_packed : nullptr, &d->mlp_l1, TH, L16,
                         s); }
    if (!P.contact && d->fuse_integrate) {
      { KTimer t(d, KID_ACCEL);
        launch_fp32_accel_integrate(P, F, d->v32b, d->sigr32, d->vd2, N, TH, L16, s); }
      std::swap(d->F[d->cur].p32, d->F[d->cur].p32n);   // the new positions become current
      integrated = true;
    } else {
      KTimer t(d, KID_ACCEL);
      launch_fp32_accel(P, F, d->v32b, d->sigr32, d->a32, N, s);
    }
  }
  if (P.contact) {                                                                    // :233-257
    KTimer t(d, KID_CONTACT);
    launch_contact_stage(P, F, N, d->ts_i == 0, mixed ? d->a32 : nullptr, s);
    d->launches += d->ts_i == 0 ? 3 : 2;
  }
  if (!integrated) {   // :273-287
    KTimer t(d, KID_INTEGRATE);
    launch_integrate(P, F, d->vd2, mixed ? d->a32 : nullptr, s);
  }
  d->launches += integrated ? 3 : 4;
  if (d->thermal) {                                                                   // :285
    if (mixed && d->fuse_heat) {
      d->heat_pending = true;
      d->heat_pending_first = d->isfirst;
    } else {
      KTimer t(d, KID_THERMAL);
      launch_thermal(P, F, N, d->isfirst ? 1 : 0, d->chi > 0.0 ? 1 : 0, mixed ? 1 : 0, s);
      d->launches += 2;
    }
  }
  if (P.contact) {                                                                    // :289-316
    KTimer t(d, KID_CONTACT);
    launch_mesh_update(P, F, mixed ? 1 : 0, s);
    d->launches += 3 * P.ncsid;
  }
  if (d->debug_checks) {
    k_check_finite<<<nblk(d->n), 256, 0, s>>>(d->n, F.xm, F.vd, d->d_status);
    d->launches += 1;
  }
  d->isfirst = false;
  d->time += d->dt;
  if (row_due) {                                                                      // :350-388
    launch_output_row(P, F, d->out_part, d->time, (double)(d->step + 1), d->out_last, d->series,
                      d->series_cap, d->series_count, 1, d->d_status, s);
    d->launches += 2;
    d->row_recorded = true;
  }
  if (d->time >= d->t_out) {                                                          // :323-368
    launch_snapshot(d->n, F, s);
    d->launches += 1;
    d->t_out += d->dt_out;
    if (d->csv_on) {
      int rc = write_snapshot(d);
      if (rc) return rc;
    }
    if (d->print_outputs) {
      int rc = print_output_row(d);
      if (rc) return rc;
    }
  }
  d->step++;
  d->ts_i++;
  if (d->ts_i > d->rebuild_every - 1) d->ts_i = 0;
  // the yield flag matters only for the next rebuild decision
  if (!d->is_yielding && d->ts_i == 0 && d->rebuild_after_yield) {
    int rc = read_status(d);
    if (rc) return rc;
    if (d->h_status[1]) d->is_yielding = true;
  }
  return WF_OK;
}

// One Fraser step.  A failure inside a step segment ends the capture and
// drops the segment, so the stream is usable again.  Then the host hook, if
// one is set (GeneralAfter, called by the reference around the integration
// of every step, SolverFraser.cu:273-281): the step's heat pass is completed
// first, so that the hook sees the whole state of the step.
static int solve_step(wf_domain* d) {
  const int rc = solve_step_launches(d);
  if (rc && d->capturing) {
    d->capturing = false;
    cudaGraph_t g = nullptr;
    if (cudaStreamEndCapture(d->stream, &g) == cudaSuccess && g) cudaGraphDestroy(g);
    cudaGetLastError();
  }
  if (rc || !d->after_fn) return rc;
  flush_heat(d);
  d->in_callback = true;
  const int r = d->after_fn(d, d->after_user);
  d->in_callback = false;
  if (r) return wf_fail(d, WF_ERR_STATE, "step callback returned " + std::to_string(r));
  return WF_OK;
}

// the last step's heat pass (mixed form), before any result leaves a call
static void flush_heat(wf_domain* d) {
  if (!d->heat_pending) return;
  StepParams P = make_params(d);
  NbBuffers N{d->nb, d->nbc};
  KTimer t(d, KID_THERMAL);
  launch_thermal(P, d->F[d->cur], N, d->heat_pending_first ? 1 : 0, d->chi > 0.0 ? 1 : 0, 1,
                 d->stream);
  d->launches += 2;
  d->heat_pending = false;
}

static int finish(wf_domain* d) {
  flush_heat(d);
  int rc = read_status(d);
  if (rc) return rc;
  WF_CUDA_OK(cudaGetLastError());
  if (d->h_status[0] & WF_STATUS_NAN) return wf_fail(d, WF_ERR_NUMERIC, "non-finite stress detected");
  if (d->h_status[0] & WF_STATUS_CHECKS)
    return wf_fail(d, WF_ERR_STATE,
                   "debug checks: a neighbour-list entry out of range (repaired) or a non-finite "
                   "position or velocity");
  if (d->h_status[0] & WF_STATUS_MMA_WAIT)
    return wf_fail(d, WF_ERR_CUDA, "a tensor-core completion wait ran out (warm-start network)");
  if (d->h_status[0] & WF_STATUS_NEWTON) {
    unsigned long long capped;
    memcpy(&capped, d->h_status + 8, sizeof capped);
    return wf_fail(d, WF_ERR_NUMERIC,
                   "Newton return map stopped at newton_max_iter = " +
                       std::to_string(d->newton_max_iter) + " without meeting newton_rtol in " +
                       std::to_string(capped) + " return maps (state advanced with them)");
  }
  return WF_OK;
}

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

const char* wf_version(void) { return WF_VERSION; }

const char* wf_last_error(const wf_domain* d) { return d ? d->err.c_str() : "null handle"; }

int wf_create(wf_domain** out, int64_t n) {
  if (!out || n <= 0 || n > (int64_t)INT32_MAX - 256) return WF_ERR_ARG;
  *out = nullptr;
  wf_domain* d = new wf_domain();
  d->n = n;
  d->n_solid = n;
  d->npad = (n + 127) / 128 * 128;
  int rc = WF_OK;
  auto bail = [&](int code) { wf_destroy(d); return code; };
  if (cudaGetDevice(&d->dev) != cudaSuccess ||
      cudaStreamCreateWithFlags(&d->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&d->cstream, cudaStreamNonBlocking) != cudaSuccess)
    return bail(WF_ERR_CUDA);
  for (int b = 0; b < 2; b++)
    if (cudaEventCreateWithFlags(&d->ev_full[b], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&d->ev_free[b], cudaEventDisableTiming) != cudaSuccess)
      return bail(WF_ERR_CUDA);
  {
    Arena size;
    layout_arena(d, size);
    d->arena_bytes = size.off;
    cache_take(d);
    if (!d->arena) {
      if (cudaMalloc((void**)&d->arena, d->arena_bytes) != cudaSuccess) {
        d->arena = nullptr;
        return bail(WF_ERR_ALLOC);
      }
      d->arena_alloc = d->arena_bytes;
    }
    if (cudaMemsetAsync(d->arena, 0, d->arena_bytes, d->stream) != cudaSuccess)
      return bail(WF_ERR_CUDA);
    Arena place;
    place.base = reinterpret_cast<uintptr_t>(d->arena);
    layout_arena(d, place);
  }
  if (!d->h_status &&
      cudaMallocHost((void**)&d->h_status, WF_STATUS_WORDS * sizeof(int)) != cudaSuccess)
    return bail(WF_ERR_ALLOC);
  k_iota<<<nblk(n), 256, 0, d->stream>>>(n, d->F[0].perm, d->inv);
  k_fill_d<<<nblk(n), 256, 0, d->stream>>>(n, -1.0, d->F[0].pwn, 1, 0);
  if (cudaStreamSynchronize(d->stream) != cudaSuccess) return bail(WF_ERR_CUDA);
  *out = d;
  return WF_OK;
}

int wf_destroy(wf_domain* d) {
  if (!d) return WF_OK;
  if (d->cstream) cudaStreamSynchronize(d->cstream);
  if (d->stream) cudaStreamSynchronize(d->stream);
  cache_put(d);                // the arena and status words, for the next domain
  for (int k = 0; k < 2; k++) free_fields(d->F[k]);
  for (MeshDev& M : d->meshes) {
    void* mp[] = {M.node, M.node_v, M.centroid, M.normal, M.elnode, M.pplane, M.cstart, M.ctri,
                  M.off32, M.cvert, M.cursor, M.scan_tmp};
    for (void* p : mp) if (p) cudaFree(p);
  }
  if (d->d_maxdep) cudaFree(d->d_maxdep);
  if (d->h_maxdep) cudaFreeHost(d->h_maxdep);
  if (d->cnb) cudaFree(d->cnb);
  if (d->ccnt) cudaFree(d->ccnt);
  void* ptrs[] = {d->log_x, d->log_y, d->log_count, d->cell_count, d->cell_cursor,
                  d->scan_tmp, d->series, d->arena};
  for (void* p : ptrs) if (p) cudaFree(p);
  if (d->h_status) cudaFreeHost(d->h_status);
  for (cudaEvent_t e : d->ev_pool) cudaEventDestroy(e);
  if (d->capturing) {
    cudaGraph_t g = nullptr;
    if (cudaStreamEndCapture(d->stream, &g) == cudaSuccess && g) cudaGraphDestroy(g);
  }
  if (d->gexec) cudaGraphExecDestroy(d->gexec);
  for (int b = 0; b < 2; b++) {
    if (d->ev_full[b]) cudaEventDestroy(d->ev_full[b]);
    if (d->ev_free[b]) cudaEventDestroy(d->ev_free[b]);
  }
  if (d->cstream) cudaStreamDestroy(d->cstream);
  if (d->stream) cudaStreamDestroy(d->stream);
  delete d;
  return WF_OK;
}

int wf_release_cache(void) {
  std::lock_guard<std::mutex> lk(g_cache_mu);
  cache_free_locked();
  return WF_OK;
}

}  // extern "C"

// ---- scatter helpers ----------------------------------------------------
// A setter's host array goes to one of two staging buffers on the copy
// stream and is scattered into slot order on the domain's stream; the call
// returns once the copy is done (the caller may then reuse its array), while
// the scatter runs on behind it and overlaps the next setter's copy.  A copy
// into a buffer waits for the scatter that last read it.
static double* stage_copy(wf_domain* d, const void* src, size_t bytes, int* b_out) {
  const int b = d->stage_next;
  d->stage_next ^= 1;
  double* stage = b ? d->d_stage2 : d->d_stage;
  if (cudaStreamWaitEvent(d->cstream, d->ev_free[b], 0) != cudaSuccess ||
      cudaMemcpyAsync(stage, src, bytes, cudaMemcpyHostToDevice, d->cstream) != cudaSuccess ||
      cudaEventRecord(d->ev_full[b], d->cstream) != cudaSuccess ||
      cudaStreamWaitEvent(d->stream, d->ev_full[b], 0) != cudaSuccess)
    return nullptr;
  *b_out = b;
  return stage;
}
static int stage_done(wf_domain* d, int b) {
  WF_CUDA_OK(cudaEventRecord(d->ev_free[b], d->stream));
  WF_CUDA_OK(cudaEventSynchronize(d->ev_full[b]));
  return WF_OK;
}
static int upload_d(wf_domain* d, const double* src, int comps, double* dst, int stride, int off) {
  int b = 0;
  double* stage = stage_copy(d, src, sizeof(double) * comps * d->n, &b);
  if (!stage) return wf_fail(d, WF_ERR_CUDA, "host to device copy");
  k_scatter_d<<<nblk(d->n), 256, 0, d->stream>>>(d->n, d->inv, stage, comps, dst, stride, off);
  return stage_done(d, b);
}
template <class T>
static int upload_t(wf_domain* d, const T* src, T* dst) {
  int b = 0;
  double* stage = stage_copy(d, src, sizeof(T) * d->n, &b);
  if (!stage) return wf_fail(d, WF_ERR_CUDA, "host to device copy");
  k_scatter_t<T><<<nblk(d->n), 256, 0, d->stream>>>(d->n, d->inv, (const T*)stage, dst);
  return stage_done(d, b);
}
// fills need no host synchronisation: later device work and read-backs are
// ordered behind them on the domain's stream
static int fill_d(wf_domain* d, double v, double* dst, int stride, int off) {
  k_fill_d<<<nblk(d->n), 256, 0, d->stream>>>(d->n, v, dst, stride, off);
  WF_CUDA_OK(cudaGetLastError());
  return WF_OK;
}
static Fields& CF(wf_domain* d) { return d->F[d->cur]; }

extern "C" {

int wf_set_h(wf_domain* d, double h) {
  if (!d || !(h > 0)) return WF_ERR_ARG;
  d->h = h;
  d->h_set = true;
  return WF_OK;
}
int wf_set_density(wf_domain* d, double rho) {
  if (!d || !(rho > 0)) return WF_ERR_ARG;
  d->rho0 = rho;
  d->rho_set = true;
  return fill_d(d, rho, (double*)CF(d).vd, 4, 3);
}
int wf_set_shear_modulus(wf_domain* d, double G) {
  if (!d) return WF_ERR_ARG;
  d->G = G;
  d->G_set = true;
  return WF_OK;
}
int wf_set_sigma_y(wf_domain* d, double sy) {
  if (!d) return WF_ERR_ARG;
  return fill_d(d, sy, CF(d).sy, 1, 0);
}
int wf_set_conductivity(wf_domain* d, double k) {
  if (!d) return WF_ERR_ARG;
  d->k_cond = k;   // one value for every particle
  return fill_d(d, k, CF(d).kT, 1, 0);
}
int wf_set_heat_cap(wf_domain* d, double cp) {
  if (!d) return WF_ERR_ARG;
  return fill_d(d, cp, CF(d).cpT, 1, 0);
}
int wf_set_cs(wf_domain* d, const double* cs) {
  if (!d || !cs) return WF_ERR_ARG;
  const double c0 = cs[0];
  bool mixed = false;
  for (int64_t i = 1; i < d->n; i++) mixed |= cs[i] != c0;   // no early exit: vectorised
  if (mixed) return wf_fail(d, WF_ERR_ARG, "per-particle Cs must be uniform");
  d->Cs = cs[0];
  d->cs_set = true;
  return WF_OK;
}
int wf_set_free(wf_domain* d, const uint8_t* f) {
  if (!d || !f) return WF_ERR_ARG;
  for (int64_t i = 0; i < d->n; i++)
    if (!f[i]) return wf_fail(d, WF_ERR_ARG, "fixed (IsFree = false) particles are not supported");
  return WF_OK;
}
int wf_set_id(wf_domain* d, const int32_t* id) {
  if (!d || !id) return WF_ERR_ARG;
  return upload_t<int32_t>(d, id, CF(d).id);
}
int wf_set_positions(wf_domain* d, const double* x) {
  if (!d || !x) return WF_ERR_ARG;
  // staged and checked on the device before anything is written
  WF_CUDA_OK(cudaMemcpyAsync(d->d_stage, x, sizeof(double) * 3 * d->n, cudaMemcpyHostToDevice,
                             d->stream));
  WF_CUDA_OK(cudaMemsetAsync(d->d_mm, 0, sizeof(int), d->stream));
  k_any_nonfinite<<<nblk(3 * d->n), 256, 0, d->stream>>>(3 * d->n, d->d_stage, d->d_mm);
  int bad = 0;
  WF_CUDA_OK(cudaMemcpyAsync(&bad, d->d_mm, sizeof(int), cudaMemcpyDeviceToHost, d->stream));
  WF_CUDA_OK(cudaStreamSynchronize(d->stream));
  if (bad) return wf_fail(d, WF_ERR_ARG, "non-finite position");
  d->x_set = true;
  if (d->started) d->lists_stale = true;   // the lists were built for the old positions
  k_scatter_d<<<nblk(d->n), 256, 0, d->stream>>>(d->n, d->inv, d->d_stage, 3, (double*)CF(d).xm,
                                                  4, 0);
  // a later setter copy into this staging buffer waits for the scatter
  WF_CUDA_OK(cudaEventRecord(d->ev_free[0], d->stream));
  return WF_OK;
}
int wf_set_velocities(wf_domain* d, const double* v) {
  if (!d || !v) return WF_ERR_ARG;
  return upload_d(d, v, 3, (double*)CF(d).vd, 4, 0);
}
int wf_set_mass(wf_domain* d, const double* m) {
  if (!d || !m) return WF_ERR_ARG;
  d->m_set = true;
  return upload_d(d, m, 1, (double*)CF(d).xm, 4, 3);
}
int wf_set_not_write_surf_id(wf_domain* d, const uint8_t* f) {
  if (!d || !f) return WF_ERR_ARG;
  return upload_t<uint8_t>(d, f, CF(d).nw);
}
int wf_set_solid_count(wf_domain* d, int64_t ns) {
  if (!d || ns < 0 || ns > d->n) return WF_ERR_ARG;
  d->n_solid = ns;
  return WF_OK;
}
int wf_set_time_step(wf_domain* d, double dt) {
  if (!d || !(dt > 0)) return WF_ERR_ARG;
  d->dt = dt;
  return WF_OK;
}
int wf_set_artificial_viscosity(wf_domain* d, double a, double b) {
  if (!d) return WF_ERR_ARG;
  d->alpha = a;
  d->beta = b;
  return WF_OK;
}
int wf_set_material(wf_domain* d, const wf_material* m) {
  if (!d || !m) return WF_ERR_ARG;
  if (m->model < WF_BILINEAR || m->model > WF_JOHNSON_COOK)
    return wf_fail(d, WF_ERR_ARG, "unknown material model");
  d->mat = *m;
  d->mat_set = true;
  return WF_OK;
}
int wf_add_velocity_bc(wf_domain* d, int32_t zone, double vx, double vy, double vz) {
  if (!d) return WF_ERR_ARG;
  if ((int)d->bc_zone.size() >= WF_MAX_BC) return wf_fail(d, WF_ERR_ARG, "too many boundary conditions");
  d->bc_zone.push_back(zone);
  d->bc_v.push_back({vx, vy, vz});
  return WF_OK;
}
int wf_set_velocity_bc(wf_domain* d, int32_t index, double vx, double vy, double vz) {
  if (!d) return WF_ERR_ARG;
  if (index < 0 || index >= (int32_t)d->bc_zone.size())
    return wf_fail(d, WF_ERR_ARG, "no velocity BC with index " + std::to_string(index));
  if (!std::isfinite(vx) || !std::isfinite(vy) || !std::isfinite(vz))
    return wf_fail(d, WF_ERR_ARG, "non-finite BC velocity");
  d->bc_v[index] = {vx, vy, vz};
  return WF_OK;
}
int wf_set_callback(wf_domain* d, wf_after_fn fn, void* user) {
  if (!d) return WF_ERR_ARG;
  if (d->in_callback) return wf_fail(d, WF_ERR_STATE, "the callback cannot be changed from itself");
  d->after_fn = fn;
  d->after_user = fn ? user : nullptr;
  return WF_OK;
}
int wf_set_csv_output(wf_domain* d, const char* prefix) {
  if (!d) return WF_ERR_ARG;
  d->csv_on = prefix != nullptr;
  d->csv_prefix = prefix ? prefix : "";
  return WF_OK;
}

int wf_set_contact(wf_domain* d, double mu_static, double mu_dynamic, int law) {
  if (!d) return WF_ERR_ARG;
  if (law != 0 && law != 1)
    return wf_fail(d, WF_ERR_ARG, "contact law must be 0 (the reference's) or 1 (binned triangles)");
  if (!(mu_static >= 0.0) || !(mu_dynamic >= 0.0))
    return wf_fail(d, WF_ERR_ARG, "friction coefficients must be >= 0");
  if (law == 1) {
    if (!d->F[0].qf)
      for (int f = 0; f < 2; f++)
        if (dalloc(&d->F[f].qf, d->npad, d->stream)) return wf_fail(d, WF_ERR_ALLOC, "qf");
  }
  d->mu_s = mu_static;
  d->mu_d = mu_dynamic;
  d->contact_law = law;
  return WF_OK;
}

int wf_add_trimesh(wf_domain* d, const double* nodes, int32_t nn, const int32_t* tris,
                   int32_t ne, const double* normals, int32_t zone_id, int64_t first,
                   const double* vel, const double* angvel) {
  if (!d || !nodes || !tris || nn <= 0 || ne <= 0 || !vel || !angvel) return WF_ERR_ARG;
  if ((int)d->meshes.size() >= WF_MAX_MESH) return wf_fail(d, WF_ERR_ARG, "at most 4 rigid meshes");
  if (first < d->n_solid || first + ne > d->n)
    return wf_fail(d, WF_ERR_ARG, "rigid particles first .. first+ne-1 must follow the solid ones");
  for (const MeshDev& M : d->meshes)
    if (first < M.first + M.ne && M.first < first + ne)
      return wf_fail(d, WF_ERR_ARG, "rigid particle ranges of two meshes overlap");
  if (zone_id == 1) return wf_fail(d, WF_ERR_ARG, "zone id 1 is the free-surface id");
  if (!d->m_set || !d->x_set) return wf_fail(d, WF_ERR_STATE, "set positions and masses first");
  if (d->started) return wf_fail(d, WF_ERR_STATE, "meshes are added before the first solve");
  for (int64_t k = 0; k < 3 * (int64_t)ne; k++)
    if (tris[k] < 0 || tris[k] >= nn) return wf_fail(d, WF_ERR_ARG, "triangle node out of range");
  for (int64_t k = 0; k < 3 * (int64_t)nn; k++)
    if (!std::isfinite(nodes[k])) return wf_fail(d, WF_ERR_ARG, "non-finite node");
  // element centroids and normals in the reference's arithmetic (CalcCentroids,
  // CalcNormals, Mesh.cu:233-257); normals given by the caller are kept
  std::vector<double4> hn(nn), hc(ne), hnorm(ne), hv(nn);
  for (int q = 0; q < nn; q++) {
    hn[q] = make_double4(nodes[3 * q], nodes[3 * q + 1], nodes[3 * q + 2], 0.0);
    hv[q] = make_double4(0.0, 0.0, 0.0, 0.0);
  }
  for (int e = 0; e < ne; e++) {
    const double4 a = hn[tris[3 * e]], b = hn[tris[3 * e + 1]], c = hn[tris[3 * e + 2]];
    const double third = 1.0 / 3.;
    hc[e] = make_double4(((a.x + b.x) + c.x) * third, ((a.y + b.y) + c.y) * third,
                         ((a.z + b.z) + c.z) * third, 0.0);
    if (normals) {
      hnorm[e] = make_double4(normals[3 * e], normals[3 * e + 1], normals[3 * e + 2], 0.0);
    } else {
      const double ux = b.x - a.x, uy = b.y - a.y, uz = b.z - a.z;
      const double vx = c.x - a.x, vy = c.y - a.y, vz = c.z - a.z;
      const double wx = uy * vz - uz * vy, wy = uz * vx - ux * vz, wz = ux * vy - uy * vx;
      const double inv = 1.0 / std::sqrt(wx * wx + wy * wy + wz * wz);
      hnorm[e] = make_double4(wx * inv, wy * inv, wz * inv, 0.0);
    }
  }
  MeshDev M{};
  M.nn = nn; M.ne = ne; M.first = (int32_t)first; M.zone = zone_id;
  for (int k = 0; k < 3; k++) { M.mv[k] = vel[k]; M.mw[k] = angvel[k]; }
  cudaStream_t s = d->stream;
  if (dalloc(&M.node, nn, s) || dalloc(&M.node_v, nn, s) || dalloc(&M.centroid, ne, s) ||
      dalloc(&M.normal, ne, s) || dalloc(&M.elnode, 3 * (int64_t)ne, s) || dalloc(&M.pplane, ne, s)) {
    void* mp[] = {M.node, M.node_v, M.centroid, M.normal, M.elnode, M.pplane};
    for (void* p : mp) if (p) cudaFree(p);
    return wf_fail(d, WF_ERR_ALLOC, "mesh arrays");
  }
  d->meshes.push_back(M);      // freed with the domain from here on
  WF_CUDA_OK(cudaMemcpyAsync(M.node, hn.data(), sizeof(double4) * nn, cudaMemcpyHostToDevice, s));
  WF_CUDA_OK(cudaMemcpyAsync(M.node_v, hv.data(), sizeof(double4) * nn, cudaMemcpyHostToDevice, s));
  WF_CUDA_OK(cudaMemcpyAsync(M.centroid, hc.data(), sizeof(double4) * ne, cudaMemcpyHostToDevice, s));
  WF_CUDA_OK(cudaMemcpyAsync(M.normal, hnorm.data(), sizeof(double4) * ne, cudaMemcpyHostToDevice, s));
  WF_CUDA_OK(cudaMemcpyAsync(M.elnode, tris, sizeof(int32_t) * 3 * ne, cudaMemcpyHostToDevice, s));
  if (!d->cnb) {               // per-particle contact state, on the first mesh
    for (int k = 0; k < 2; k++)
      if (dalloc(&d->F[k].nrm, d->npad, s) || dalloc(&d->F[k].cf, d->npad, s))
        return wf_fail(d, WF_ERR_ALLOC, "contact fields");
    if (dalloc(&d->cnb, (int64_t)WF_CONT_NB * d->npad, s) || dalloc(&d->ccnt, d->npad, s))
      return wf_fail(d, WF_ERR_ALLOC, "contact lists");
  }
  k_place_rigid<<<nblk(ne), 256, 0, s>>>(ne, (int32_t)first, d->inv, M.centroid, M.normal,
                                          zone_id, CF(d));
  WF_CUDA_OK(cudaStreamSynchronize(s));
  WF_CUDA_OK(cudaGetLastError());
  return WF_OK;
}

int wf_set_temperature(wf_domain* d, const double* T) {
  if (!d || !T) return WF_ERR_ARG;
  return upload_d(d, T, 1, CF(d).T, 1, 0);
}
int wf_set_thermal_bc(wf_domain* d, const int32_t* b) {
  if (!d || !b) return WF_ERR_ARG;
  return upload_t<int32_t>(d, b, CF(d).bct);
}
int wf_get_return_map_log(wf_domain* d, float* X, float* Y, int64_t cap, int64_t* count) {
  if (!d || !X || !Y || !count) return WF_ERR_ARG;
  if (!d->log_cap) return wf_fail(d, WF_ERR_STATE, "option log_return_map not set");
  unsigned long long c = 0;
  WF_CUDA_OK(cudaMemcpyAsync(&c, d->log_count, sizeof c, cudaMemcpyDeviceToHost, d->stream));
  WF_CUDA_OK(cudaStreamSynchronize(d->stream));
  int64_t m = std::min<int64_t>((int64_t)std::min<unsigned long long>(c, (unsigned long long)d->log_cap), cap);
  WF_CUDA_OK(cudaMemcpy(X, d->log_x, sizeof(float4) * m, cudaMemcpyDeviceToHost));
  WF_CUDA_OK(cudaMemcpy(Y, d->log_y, sizeof(float) * m, cudaMemcpyDeviceToHost));
  *count = m;
  return WF_OK;
}

int wf_set_mlp_weights(wf_domain* d, const float* params) {
  if (!d || !params) return WF_ERR_ARG;
  WF_CUDA_OK(cudaMemcpyAsync(d->mlp_w, params, sizeof(float) * WF_MLP_NPARAM,
                             cudaMemcpyHostToDevice, d->stream));
  if (wf_mlp_pack_device(d->mlp_w, d->mlp_packed, d->stream)) return wf_fail(d, WF_ERR_CUDA, "mlp pack");
  d->mlp_l1 = mlp_l1_from(params);
  WF_CUDA_OK(cudaStreamSynchronize(d->stream));
  d->mlp_loaded = true;
  return WF_OK;
}
int wf_set_convection(wf_domain* d, double hc, double Tinf) {
  if (!d) return WF_ERR_ARG;
  d->h_conv = hc;
  d->T_inf = Tinf;
  return WF_OK;
}

int wf_set_option(wf_domain* d, const char* key, double v) {
  if (!d || !key) return WF_ERR_ARG;
  std::string k(key);
  if (k == "precision") {
    int p = (int)v;
    if (p != 0 && p != 1) return wf_fail(d, WF_ERR_ARG, "precision must be 0 (fp64) or 1 (mixed)");
    if (d->started && p != d->precision) {
      if (p == 1) k_mixed_init<<<nblk(d->n), 256, 0, d->stream>>>(d->n, CF(d));
      else k_mixed_to_fp64<<<nblk(d->n), 256, 0, d->stream>>>(d->n, CF(d));
    }
    d->precision = p;
  } else if (k == "return_map") {
    if (v != 0 && v != 1) return wf_fail(d, WF_ERR_ARG, "return_map must be 0 or 1");
    d->return_map = (int)v;
  } else if (k == "mlp") d->mlp_on = v != 0;
  else if (k == "rebuild_every") {
    if (v < 1) return WF_ERR_ARG;
    d->rebuild_every = (int)v;
  } else if (k == "rebuild_after_yield") d->rebuild_after_yield = v != 0;
  else if (k == "rebuild_current_positions") d->rebuild_current = v != 0;
  else if (k == "thermal") d->thermal = v != 0;
  else if (k == "fuse_heat") d->fuse_heat = v != 0;
  else if (k == "fuse_integrate") d->fuse_integrate = v != 0;
  else if (k == "contact_stiffness") d->c_kappa = v;
  else if (k == "contact_dx") d->c_dx = v;
  else if (k == "contact_vreg") d->c_vreg = v;
  else if (k == "contact_heat_fraction") d->c_eta = v;
  else if (k == "rebuild_strain_increment") {
    if (!(v >= 0.0)) return wf_fail(d, WF_ERR_ARG, "rebuild_strain_increment must be >= 0");
    if (v > 0.0 && !d->F[0].eps_rb) {
      for (int f = 0; f < 2; f++)
        if (dalloc(&d->F[f].eps_rb, d->npad, d->stream)) return wf_fail(d, WF_ERR_ALLOC, "eps_rb");
      if (dalloc(&d->d_maxdep, 1, d->stream) ||
          cudaMallocHost((void**)&d->h_maxdep, sizeof(unsigned long long)) != cudaSuccess)
        return wf_fail(d, WF_ERR_ALLOC, "rebuild flag");
    }
    d->rb_dep = v;
  }
  else if (k == "taylor_quinney") d->chi = v;
  else if (k == "newton_rtol") d->newton_rtol = v;
  else if (k == "newton_max_iter") {
    if (!(v >= 1.0)) return wf_fail(d, WF_ERR_ARG, "newton_max_iter must be >= 1");
    d->newton_max_iter = (int)v;
  }
  else if (k == "output_every_step") d->out_every_step = v != 0;
  else if (k == "print_outputs") d->print_outputs = v != 0;
  else if (k == "output_series_cap") {
    if (!(v >= 1.0) || v > 1.0e9) return wf_fail(d, WF_ERR_ARG, "output_series_cap must be in [1, 1e9]");
    if ((int64_t)v != d->series_cap) {
      if (d->series) cudaFree(d->series);
      d->series = nullptr;          // reallocated at the next solve start
      d->series_width = 0;
      d->series_cap = (int64_t)v;
    }
  }
  else if (k == "energy_mode") d->energy_mode = (int)v;
  else if (k == "output_interval") d->output_interval = v;
  else if (k == "clamp_homologous") d->clamp_homologous = v != 0;
  else if (k == "profile_kernel") d->profile_kernel = (int)v;
  else if (k == "resume") d->resume = v != 0;
  else if (k == "log_return_map") {
    // capacity of the (state, converged increment) log kept by the plain form
    if (v < 0) return WF_ERR_ARG;
    if (d->log_x) { cudaFree(d->log_x); cudaFree(d->log_y); cudaFree(d->log_count); }
    d->log_x = nullptr; d->log_y = nullptr; d->log_count = nullptr;
    d->log_cap = (int64_t)v;
    if (d->log_cap > 0) {
      WF_CUDA_OK(dalloc(&d->log_x, d->log_cap, d->stream));
      WF_CUDA_OK(dalloc(&d->log_y, d->log_cap, d->stream));
      WF_CUDA_OK(dalloc(&d->log_count, 1, d->stream));
    }
  }
  else if (k == "tile_staging") d->tile_staging = v != 0;   // takes effect at the next rebuild
  else if (k == "list_prefetch") d->list_prefetch = std::max(0, std::min((int)v, WF_NB_BLOCKS));
  else if (k == "state_prefetch") d->state_prefetch = v != 0;
  else if (k == "debug_checks") d->debug_checks = v != 0;
  else if (k == "debug_inject_list_error") {
    // the injected entry is repaired by the list check before any pass reads it
    if (!d->debug_checks)
      return wf_fail(d, WF_ERR_ARG, "debug_inject_list_error needs debug_checks = 1");
    if (!(v >= 0.0) || v >= (double)d->n)
      return wf_fail(d, WF_ERR_ARG, "debug_inject_list_error: a particle id in [0, n)");
    d->inject_list_error = (int64_t)v;
  }
  else if (k == "wave_prefetch") d->wave_prefetch = (int)v;
  else if (k == "wave_prefetch_distance") d->wave_dist = v;
  else if (k == "list16") d->list16 = v != 0;          // takes effect at the next rebuild
  else if (k == "tile_cap_max") {
    if (!(v >= 1.0) || v > WF_TILE_HALO_MAX)
      return wf_fail(d, WF_ERR_ARG, "tile_cap_max must be in [1, 2048]");
    d->tile_cap_max = (int)v;
  }
  else if (k == "graph") {
    if (d->capturing) return wf_fail(d, WF_ERR_STATE, "graph option changed inside a step segment");
    d->graph = v != 0;
  }
  else return wf_fail(d, WF_ERR_ARG, "unknown option: " + k);
  return WF_OK;
}

int wf_find_neighbors(wf_domain* d) {
  if (!d) return WF_ERR_ARG;
  if (d->in_callback) return wf_fail(d, WF_ERR_STATE, "solvers cannot be called from the step callback");
  if (!d->h_set || !d->x_set) return wf_fail(d, WF_ERR_STATE, "h and positions required");
  launch_snapshot(d->n, CF(d), d->stream);
  int rc = rebuild(d, false);
  if (rc) return rc;
  return finish(d);
}

int wf_step(wf_domain* d, int64_t nsteps) {
  if (!d || nsteps < 0) return WF_ERR_ARG;
  if (d->in_callback) return wf_fail(d, WF_ERR_STATE, "solvers cannot be called from the step callback");
  if (!d->started) {
    int rc = solve_begin(d, d->output_interval);
    if (rc) return rc;
  }
  for (int64_t k = 0; k < nsteps; k++) {
    int rc = solve_step(d);
    if (rc) return rc;
  }
  return finish(d);
}

int wf_mech_fraser_solve(wf_domain* d, double tf, double dt_out) {
  if (!d || !(dt_out > 0)) return WF_ERR_ARG;
  if (d->in_callback) return wf_fail(d, WF_ERR_STATE, "solvers cannot be called from the step callback");
  int rc = solve_begin(d, dt_out);
  if (rc) return rc;
  while (d->time < tf) {
    rc = solve_step(d);
    if (rc) return rc;
  }
  rc = finish(d);
  if (rc == WF_OK && d->csv_on) rc = write_series_csv(d, (d->csv_prefix + "outputs.csv").c_str());
  return rc;
}

int wf_mech_solve(wf_domain* d, double tf, double dt_out) { return wf_mech_fraser_solve(d, tf, dt_out); }

int wf_thermal_solve(wf_domain* d, double tf) {
  if (!d) return WF_ERR_ARG;
  if (d->in_callback) return wf_fail(d, WF_ERR_STATE, "solvers cannot be called from the step callback");
  if (!d->h_set || !d->x_set || !d->m_set || !d->rho_set || !(d->dt > 0))
    return wf_fail(d, WF_ERR_STATE, "h, positions, masses, density and time step required");
  d->time = 0.0;
  d->isfirst = true;
  WF_CUDA_OK(cudaMemsetAsync(d->d_status, 0, WF_STATUS_WORDS * sizeof(int), d->stream));
  int rc = rebuild(d, true);
  if (rc) return rc;
  if (d->precision == 1) k_mixed_init<<<nblk(d->n), 256, 0, d->stream>>>(d->n, CF(d));
  StepParams P = make_params(d);
  NbBuffers N{d->nb, d->nbc};
  while (d->time < tf) {
    {
      KTimer t(d, KID_THERMAL);
      launch_thermal(P, CF(d), N, d->isfirst ? 1 : 0, 0, d->precision == 1 ? 1 : 0, d->stream);
    }
    d->launches += 2;
    d->isfirst = false;
    d->time += d->dt;
    d->step++;
  }
  return finish(d);
}

}  // extern "C"

// ---- getters ---------------------------------------------------------------
static int download(wf_domain* d, double* out, int64_t count) {
  WF_CUDA_OK(cudaMemcpyAsync(out, d->d_stage, sizeof(double) * count, cudaMemcpyDeviceToHost, d->stream));
  WF_CUDA_OK(cudaStreamSynchronize(d->stream));
  return WF_OK;
}

extern "C" {

// ---- state transfer (checkpoint / restart) ---------------------------------
int wf_set_field(wf_domain* d, const char* name, const double* in) {
  if (!d || !name || !in) return WF_ERR_ARG;
  Fields& F = CF(d);
  std::string s(name);
  int rc;
  if (s == "x") rc = wf_set_positions(d, in);   // finite check; new lists at the next step
  else if (s == "m") { d->m_set = true; rc = upload_d(d, in, 1, (double*)F.xm, 4, 3); }
  else if (s == "v") rc = upload_d(d, in, 3, (double*)F.vd, 4, 0);
  else if (s == "rho") rc = upload_d(d, in, 1, (double*)F.vd, 4, 3);
  else if (s == "u") rc = upload_d(d, in, 3, (double*)F.u, 4, 0);
  else if (s == "a") rc = upload_d(d, in, 3, (double*)F.a, 4, 0);
  else if (s == "sigma") rc = upload_d(d, in, 6, F.sig6, 6, 0);
  else if (s == "shearstress") rc = upload_d(d, in, 6, F.ss6, 6, 0);
  else if (s == "strain") rc = upload_d(d, in, 6, F.eps6, 6, 0);
  else if (s == "strrate") rc = upload_d(d, in, 6, F.sr6, 6, 0);
  else if (s == "rotrate") rc = upload_d(d, in, 6, F.rr6, 6, 0);
  else if (s == "p") rc = upload_d(d, in, 1, F.p, 1, 0);
  else if (s == "sigma_eq") rc = upload_d(d, in, 1, F.seq, 1, 0);
  else if (s == "pl_strain") {
    rc = upload_d(d, in, 1, F.eps_p, 1, 0);
    if (!rc) rc = fill_d(d, -1.0, F.pwn, 1, 0);    // cached eps_p^n no longer valid
  }
  else if (s == "sigma_y") rc = upload_d(d, in, 1, F.sy, 1, 0);
  else if (s == "eff_strain_rate") rc = upload_d(d, in, 1, F.eff, 1, 0);
  else if (s == "dep") rc = upload_d(d, in, 1, F.dep, 1, 0);
  else if (s == "int_energy") rc = upload_d(d, in, 1, F.eint, 1, 0);
  else if (s == "T") rc = upload_d(d, in, 1, F.T, 1, 0);
  else if (s == "Ta") rc = upload_d(d, in, 1, F.Ta, 1, 0);
  else if (s == "Tb") rc = upload_d(d, in, 1, F.Tb, 1, 0);
  else if (s == "dTdt") rc = upload_d(d, in, 1, F.dTdt, 1, 0);
  else return wf_fail(d, WF_ERR_ARG, "unknown or read-only field: " + s);
  if (rc) return rc;
  if (d->started && d->precision == 1) {
    k_mixed_init<<<nblk(d->n), 256, 0, d->stream>>>(d->n, F);
    WF_CUDA_OK(cudaStreamSynchronize(d->stream));
  }
  return WF_OK;
}

int wf_set_scalar(wf_domain* d, const char* name, double v) {
  if (!d || !name) return WF_ERR_ARG;
  std::string s(name);
  if (s == "time") d->time = v;
  else if (s == "step") d->step = (int64_t)v;
  else if (s == "isfirst") d->isfirst = v != 0;
  else if (s == "is_yielding") d->is_yielding = v != 0;
  else return wf_fail(d, WF_ERR_ARG, "unknown scalar: " + s);
  return WF_OK;
}

int wf_get_field(wf_domain* d, const char* name, double* out) {
  if (!d || !name || !out) return WF_ERR_ARG;
  const Fields& F = CF(d);
  const int64_t n = d->n;
  std::string s(name);
  const bool mixed = d->precision == 1 && d->started;
  double* st = d->d_stage;
  auto g = [&](const double* src, int stride, int off, int comps) {
    k_gather_d<<<nblk(n), 256, 0, d->stream>>>(n, d->inv, src, stride, off, comps, st);
    return download(d, out, n * comps);
  };
  auto gf = [&](const float* src, int stride, int off, int comps) {
    k_gather_f<<<nblk(n), 256, 0, d->stream>>>(n, d->inv, src, stride, off, comps, st);
    return download(d, out, n * comps);
  };
  if (s == "x") return g((const double*)F.xm, 4, 0, 3);
  if (s == "m") return g((const double*)F.xm, 4, 3, 1);
  if (s == "v") return g((const double*)F.vd, 4, 0, 3);
  if (s == "rho") return g((const double*)F.vd, 4, 3, 1);
  if (s == "u") return g((const double*)F.u, 4, 0, 3);
  if (s == "a") return g((const double*)F.a, 4, 0, 3);
  if (s == "sigma") {
    if (mixed) {
      k_gather_sigma32<<<nblk(n), 256, 0, d->stream>>>(n, d->inv, F.ss32, F.p, st);
      return download(d, out, 6 * n);
    }
    return g(F.sig6, 6, 0, 6);
  }
  if (s == "shearstress") return mixed ? gf(F.ss32, 6, 0, 6) : g(F.ss6, 6, 0, 6);
  if (s == "strain") return g(F.eps6, 6, 0, 6);
  if (s == "strrate") return g(F.sr6, 6, 0, 6);
  if (s == "rotrate") return g(F.rr6, 6, 0, 6);
  if (s == "p") return g(F.p, 1, 0, 1);
  if (s == "sigma_eq") return g(F.seq, 1, 0, 1);
  if (s == "pl_strain") return g(F.eps_p, 1, 0, 1);
  if (s == "sigma_y") return g(F.sy, 1, 0, 1);
  if (s == "eff_strain_rate") return g(F.eff, 1, 0, 1);
  if (s == "dep") return g(F.dep, 1, 0, 1);
  if (s == "drho") return g(F.drho, 1, 0, 1);
  if (s == "int_energy") return g(F.eint, 1, 0, 1);
  if (s == "T") return g(F.T, 1, 0, 1);
  if (s == "Ta") return g(F.Ta, 1, 0, 1);
  if (s == "Tb") return g(F.Tb, 1, 0, 1);
  if (s == "dTdt") return g(F.dTdt, 1, 0, 1);
  if (s == "fric_heat") {                          // zero unless contact law 1
    if (!F.qf) {
      std::fill(out, out + n, 0.0);
      return WF_OK;
    }
    return g(F.qf, 1, 0, 1);
  }
  if (s == "normal" || s == "contforce") {         // zero until a rigid mesh is added
    const double4* src = s == "normal" ? F.nrm : F.cf;
    if (!src) {
      std::fill(out, out + 3 * n, 0.0);
      return WF_OK;
    }
    return g((const double*)src, 4, 0, 3);
  }
  return wf_fail(d, WF_ERR_ARG, "unknown field: " + s);
}

int wf_get_field_i32(wf_domain* d, const char* name, int32_t* out) {
  if (!d || !name || !out) return WF_ERR_ARG;
  std::string s(name);
  const Fields& F = CF(d);
  const int32_t* src = nullptr;
  if (s == "ID") src = F.id;
  else if (s == "nb_count") src = d->nbc;
  else if (s == "BC_T") src = F.bct;
  else if (s == "cont_count") {          // zero until a rigid mesh is added
    if (!d->ccnt) {
      std::fill(out, out + d->n, 0);
      return WF_OK;
    }
    src = d->ccnt;
  }
  else return wf_fail(d, WF_ERR_ARG, "unknown field: " + s);
  k_gather_t<int32_t><<<nblk(d->n), 256, 0, d->stream>>>(d->n, d->inv, src, (int32_t*)d->d_stage);
  WF_CUDA_OK(cudaMemcpyAsync(out, d->d_stage, sizeof(int32_t) * d->n, cudaMemcpyDeviceToHost, d->stream));
  WF_CUDA_OK(cudaStreamSynchronize(d->stream));
  return WF_OK;
}

int wf_get_neighbors(wf_domain* d, int32_t* counts, int32_t* lists) {
  if (!d || !counts || !lists) return WF_ERR_ARG;
  if (!d->nb_built) return wf_fail(d, WF_ERR_STATE, "no neighbour list yet");
  int32_t *dc = nullptr, *dl = nullptr;
  WF_CUDA_OK(cudaMalloc((void**)&dc, sizeof(int32_t) * d->n));
  cudaError_t e = cudaMalloc((void**)&dl, sizeof(int32_t) * d->n * WF_NB);
  if (e != cudaSuccess) { cudaFree(dc); return wf_cuda_fail(d, e, "cudaMalloc"); }
  k_gather_nb<<<nblk(d->n), 256, 0, d->stream>>>(d->n, d->npad, d->inv, CF(d).perm, d->nb, d->nbc, dc, dl);
  cudaMemcpyAsync(counts, dc, sizeof(int32_t) * d->n, cudaMemcpyDeviceToHost, d->stream);
  cudaMemcpyAsync(lists, dl, sizeof(int32_t) * d->n * WF_NB, cudaMemcpyDeviceToHost, d->stream);
  e = cudaStreamSynchronize(d->stream);
  cudaFree(dc);
  cudaFree(dl);
  if (e != cudaSuccess) return wf_cuda_fail(d, e, "get_neighbors");
  return WF_OK;
}

int wf_get_scalar(wf_domain* d, const char* name, double* out) {
  if (!d || !name || !out) return WF_ERR_ARG;
  std::string s(name);
  if (s == "time") { *out = d->time; return WF_OK; }
  if (s == "step") { *out = (double)d->step; return WF_OK; }
  if (s == "is_yielding") { *out = d->is_yielding; return WF_OK; }
  if (s == "isfirst") { *out = d->isfirst; return WF_OK; }
  if (s == "launches") { *out = (double)d->launches; return WF_OK; }
  if (s == "rebuilds") { *out = (double)d->rebuilds; return WF_OK; }
  if (s == "graph_launches") { *out = (double)d->graph_launches; return WF_OK; }
  if (s == "graph_instantiations") { *out = (double)d->graph_instantiations; return WF_OK; }
  if (s == "contact_tests32" || s == "contact_tests64") {   // law 1, since creation
    unsigned long long c[2];
    WF_CUDA_OK(cudaMemcpyAsync(c, d->d_cstat, sizeof c, cudaMemcpyDeviceToHost, d->stream));
    WF_CUDA_OK(cudaStreamSynchronize(d->stream));
    *out = (double)c[s == "contact_tests32" ? 0 : 1];
    return WF_OK;
  }
  if (s == "newton_iters" || s == "newton_calls" || s == "mlp_used" || s == "status" ||
      s == "newton_capped") {
    int rc = read_status(d);
    if (rc) return rc;
    unsigned long long v;
    if (s == "status") { *out = d->h_status[0]; return WF_OK; }
    const int w = s == "newton_iters" ? 2 : (s == "newton_calls" ? 4 : (s == "mlp_used" ? 6 : 8));
    memcpy(&v, d->h_status + w, sizeof v);
    *out = (double)v;
    return WF_OK;
  }
  {  // values of the last output row
    static const char* names[] = {"max_disp_x", "max_disp_y", "max_disp_z", "max_pl_strain",
                                  "cont_force_sum", "cont_force_x", "cont_force_y",
                                  "cont_force_z", "int_energy_total", "reaction_x",
                                  "reaction_y", "reaction_z"};
    for (int k = 0; k < 12; k++) {
      if (s != names[k]) continue;
      if (k >= 9 && d->bc_zone.empty()) return wf_fail(d, WF_ERR_STATE, "no velocity BC");
      double r[3];
      const int rc = wf_get_output_row(d, r, 0, nullptr);   // WF_ERR_STATE before any row
      if (rc) return rc;
      const int col = k < 9 ? 2 + k : WF_ROW_FIXED + (k - 9);
      WF_CUDA_OK(cudaMemcpyAsync(out, d->out_last + col, sizeof(double), cudaMemcpyDeviceToHost,
                                 d->stream));
      WF_CUDA_OK(cudaStreamSynchronize(d->stream));
      return WF_OK;
    }
  }
  if (s == "tiles_staged" || s == "tile_halo_max" || s == "tile_cap") {
    // the tiles of the last neighbour rebuild: how many were staged, the largest halo
    if (s == "tile_cap") { *out = d->tile_cap; return WF_OK; }
    if (d->tile_cap == 0) { *out = 0.0; return WF_OK; }
    int rc = segment_end(d);
    if (rc) return rc;
    const int64_t tiles = d->npad / WF_TILE;
    std::vector<int32_t> hc(tiles);
    int mx = 0;
    WF_CUDA_OK(cudaMemcpyAsync(hc.data(), d->t_hcnt, sizeof(int32_t) * tiles,
                               cudaMemcpyDeviceToHost, d->stream));
    WF_CUDA_OK(cudaMemcpyAsync(&mx, d->d_mm + 6, sizeof(int), cudaMemcpyDeviceToHost, d->stream));
    WF_CUDA_OK(cudaStreamSynchronize(d->stream));
    if (s == "tile_halo_max") { *out = mx; return WF_OK; }
    int64_t staged = 0;
    for (int32_t h : hc) staged += h > 0;
    *out = (double)staged;
    return WF_OK;
  }
  if (s == "int_energy_sum") {
    std::vector<double> e(d->n);
    int rc = wf_get_field(d, "int_energy", e.data());
    if (rc) return rc;
    double sum = 0.0;
    for (double v : e) sum += v;
    *out = sum;
    return WF_OK;
  }
  return wf_fail(d, WF_ERR_ARG, "unknown scalar: " + s);
}

int wf_get_output_row(wf_domain* d, double* row, int64_t cap, int64_t* width) {
  if (!d || (cap > 0 && !row)) return WF_ERR_ARG;
  const int64_t w = WF_ROW_FIXED + 3 * (int64_t)d->bc_zone.size();
  if (width) *width = w;
  if (!d->row_recorded)
    return wf_fail(d, WF_ERR_STATE,
                   "no output row yet: rows are recorded at output times, or every step with "
                   "option output_every_step");
  {
    const int rc = segment_end(d);
    if (rc) return rc;
  }
  if (cap > 0) {
    WF_CUDA_OK(cudaMemcpyAsync(row, d->out_last, sizeof(double) * std::min(cap, w),
                               cudaMemcpyDeviceToHost, d->stream));
    WF_CUDA_OK(cudaStreamSynchronize(d->stream));
  }
  return WF_OK;
}

int wf_get_output_series(wf_domain* d, double* rows, int64_t cap_rows, int64_t* n_rows,
                         int64_t* width) {
  if (!d || !n_rows || (cap_rows > 0 && !rows)) return WF_ERR_ARG;
  const int64_t w = WF_ROW_FIXED + 3 * (int64_t)d->bc_zone.size();
  if (width) *width = w;
  *n_rows = 0;
  if (!d->series || d->series_width != w) return WF_OK;
  {
    const int rc = segment_end(d);
    if (rc) return rc;
  }
  unsigned long long c = 0;
  WF_CUDA_OK(cudaMemcpyAsync(&c, d->series_count, sizeof c, cudaMemcpyDeviceToHost, d->stream));
  WF_CUDA_OK(cudaStreamSynchronize(d->stream));
  const int64_t m = std::min<int64_t>((int64_t)c, cap_rows);
  if (m > 0) {
    WF_CUDA_OK(cudaMemcpyAsync(rows, d->series, sizeof(double) * m * w, cudaMemcpyDeviceToHost,
                               d->stream));
    WF_CUDA_OK(cudaStreamSynchronize(d->stream));
  }
  *n_rows = cap_rows > 0 ? m : (int64_t)c;
  return WF_OK;
}

int wf_get_reaction(wf_domain* d, int32_t bc_index, double* force) {
  if (!d || !force) return WF_ERR_ARG;
  if (bc_index < 0 || bc_index >= (int32_t)d->bc_zone.size())
    return wf_fail(d, WF_ERR_ARG, "no velocity BC with index " + std::to_string(bc_index));
  int rc = wf_get_output_row(d, nullptr, 0, nullptr);
  if (rc) return rc;
  WF_CUDA_OK(cudaMemcpyAsync(force, d->out_last + WF_ROW_FIXED + 3 * bc_index, 3 * sizeof(double),
                             cudaMemcpyDeviceToHost, d->stream));
  WF_CUDA_OK(cudaStreamSynchronize(d->stream));
  return WF_OK;
}

}  // extern "C"

// the output series as CSV, one row per recorded output
static int write_series_csv(wf_domain* d, const char* path) {
  int64_t n = 0, w = 0;
  int rc = wf_get_output_series(d, nullptr, 0, &n, &w);
  if (rc) return rc;
  std::vector<double> rows((size_t)std::max<int64_t>(n, 1) * w);
  rc = wf_get_output_series(d, rows.data(), n, &n, &w);
  if (rc) return rc;
  FILE* f = fopen(path, "w");
  if (!f) return wf_fail(d, WF_ERR_IO, std::string("cannot open ") + path);
  fprintf(f, "time, step, max_ux, max_uy, max_uz, max_pl_strain, cont_force_sum, CFx, CFy, CFz, "
             "int_energy");
  for (size_t b = 0; b < d->bc_zone.size(); b++)
    fprintf(f, ", BC%zu_Fx, BC%zu_Fy, BC%zu_Fz", b, b, b);
  fprintf(f, "\n");
  for (int64_t r = 0; r < n; r++) {
    for (int64_t k = 0; k < w; k++)
      fprintf(f, k == 1 ? "%.0f" : "%.9e", rows[(size_t)(r * w + k)]), fputs(k + 1 < w ? ", " : "\n", f);
  }
  fclose(f);
  return WF_OK;
}

extern "C" {

// Domain_d::WriteCSV (src/cuda/Domain_d.cu:556-587): same header and format.
int wf_write_csv(wf_domain* d, const char* path) {
  if (!d || !path) return WF_ERR_ARG;
  const int64_t n = d->n;
  std::vector<double> x(3 * n), u(3 * n), v(3 * n), a(3 * n), rho(n), p(n), seq(n), ps(n),
      cf(3 * n), nr(3 * n);
  std::vector<int32_t> id(n), nbc(n), cnc(n);
  int rc = 0;
  if ((rc = wf_get_field(d, "x", x.data())) || (rc = wf_get_field(d, "u", u.data())) ||
      (rc = wf_get_field(d, "v", v.data())) || (rc = wf_get_field(d, "a", a.data())) ||
      (rc = wf_get_field(d, "rho", rho.data())) || (rc = wf_get_field(d, "p", p.data())) ||
      (rc = wf_get_field(d, "sigma_eq", seq.data())) || (rc = wf_get_field(d, "pl_strain", ps.data())) ||
      (rc = wf_get_field(d, "contforce", cf.data())) || (rc = wf_get_field(d, "normal", nr.data())) ||
      (rc = wf_get_field_i32(d, "ID", id.data())) || (rc = wf_get_field_i32(d, "nb_count", nbc.data())) ||
      (rc = wf_get_field_i32(d, "cont_count", cnc.data())))
    return rc;
  FILE* f = fopen(path, "w");
  if (!f) return wf_fail(d, WF_ERR_IO, std::string("cannot open ") + path);
  fprintf(f, "ID, X, Y, Z, posX,posY,posZ,Ux, Uy, Uz, Vx, Vy, Vz, Ax, Ay, Az, rho, p, SigmaEq, "
             "Pl_Strain, Nb, ContNb, CFx, CFy, CFz, Nx, Ny, Nz, h\n");
  for (int64_t i = 0; i < n; i++) {
    fprintf(f,
            "%d, %.6e, %.6e, %.6e, %.6e, %.6e, %.6e, %.6e, %.6e, %.6e, %.6e, %.6e, %.6e, %.6e, "
            "%.6e, %.6e, %.6e, %.6e, %.6e, %.6e, %d, %d, %.6e, %.6e, %.6e, %.6e, %.6e, %.6e, %6e\n",
            id[i], x[3 * i], x[3 * i + 1], x[3 * i + 2], x[3 * i], x[3 * i + 1], x[3 * i + 2],
            u[3 * i], u[3 * i + 1], u[3 * i + 2], v[3 * i], v[3 * i + 1], v[3 * i + 2], a[3 * i],
            a[3 * i + 1], a[3 * i + 2], rho[i], p[i], seq[i], ps[i], nbc[i], cnc[i], cf[3 * i],
            cf[3 * i + 1], cf[3 * i + 2], nr[3 * i], nr[3 * i + 1], nr[3 * i + 2], d->h);
  }
  fclose(f);
  return WF_OK;
}

int wf_time_steps(wf_domain* d, int64_t nsteps, double* elapsed_ms, double* kernel_ms,
                  int64_t* kernel_launches, int64_t* total_launches) {
  if (!d || nsteps < 0) return WF_ERR_ARG;
  if (d->in_callback) return wf_fail(d, WF_ERR_STATE, "solvers cannot be called from the step callback");
  if (!d->started) {
    int rc = solve_begin(d, d->output_interval);
    if (rc) return rc;
  }
  cudaEvent_t e0, e1;
  WF_CUDA_OK(cudaEventCreate(&e0));
  WF_CUDA_OK(cudaEventCreate(&e1));
  d->ev_used = 0;
  const int64_t l0 = d->launches;
  WF_CUDA_OK(cudaStreamSynchronize(d->stream));
  cudaEventRecord(e0, d->stream);
  int rc = WF_OK;
  d->timing = true;
  for (int64_t k = 0; k < nsteps && rc == WF_OK; k++) rc = solve_step(d);
  flush_heat(d);   // the timed steps include their whole heat work
  if (rc == WF_OK) rc = segment_end(d);
  d->timing = false;
  cudaEventRecord(e1, d->stream);
  WF_CUDA_OK(cudaEventSynchronize(e1));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return rc;
  if (elapsed_ms) *elapsed_ms = ms;
  double kms = 0.0;
  for (size_t k = 0; k + 1 < d->ev_used; k += 2) {
    float t = 0.f;
    cudaEventElapsedTime(&t, d->ev_pool[k], d->ev_pool[k + 1]);
    kms += t;
  }
  if (kernel_ms) *kernel_ms = kms;
  if (kernel_launches) *kernel_launches = (int64_t)(d->ev_used / 2);
  if (total_launches) *total_launches = d->launches - l0;
  d->ev_used = 0;
  return finish(d);
}

}  // extern "C"
