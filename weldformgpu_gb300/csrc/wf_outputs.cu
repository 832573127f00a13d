// wf_outputs.cu — the FP64 output reductions of the Fraser loop.
//
// At every output time MechFraserSolve reads the whole state back and reduces
// it on the host (src/cuda/SolverFraser.cu:323-388): the component-wise
// maximum displacement (from 0), the maximum plastic strain and the contact
// force sum over free-surface particles (sum of |contforce| where ID ==
// id_free_surf).  Here the same quantities, plus the contact-force vector sum,
// the internal-energy sum and, per velocity BC, the force its zone carries
// (sum of m a over the zone before the BC zeroes a: the platen load of a
// compression test), are reduced on the device in FP64 into one output row.
//
// The reduction order is fixed and independent of the slot order: particles
// are visited by original id, kOutBlocks blocks of kOutThreads threads stride
// over the ids, each block reduces its threads' partials by a shuffle tree and
// a fixed pass over its warps, and one thread per value sums the blocks'
// partials in block order.  Two runs with the same values give the same bits.
// Compiled with -fmad=false (|contforce| = sqrt of the dot product, rounded
// like the reference's length()).
#include "wf_common.cuh"

namespace {

constexpr int kOutBlocks = 256;
constexpr int kOutThreads = 256;
constexpr int kOutWarps = kOutThreads / 32;
// values per row besides time and step: max u (3), max pl_strain, contact
// force sum, contact force vector (3), internal energy, then 3 per BC
constexpr int kOutFixed = WF_ROW_FIXED - 2;

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_max(double v) {
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
  return v;
}

// block-wide reduction (fixed order); thread 0 holds the result
template <bool kMax>
__device__ __forceinline__ double block_reduce(double v, double* sh) {
  v = kMax ? warp_max(v) : warp_sum(v);
  const int w = threadIdx.x >> 5;
  __syncthreads();                       // sh is reused by successive reductions
  if ((threadIdx.x & 31) == 0) sh[w] = v;
  __syncthreads();
  double r = sh[0];
  if (threadIdx.x == 0)
    for (int k = 1; k < kOutWarps; k++) r = kMax ? fmax(r, sh[k]) : r + sh[k];
  return r;
}

struct OutArgs {
  int64_t n;
  const int32_t* inv;     // inv[original id] = slot
  const int32_t* id;
  const double4* u;
  const double* eps_p;
  const double4* cf;      // null without contact
  const double* eint;
  const double4* fr;      // m a before the BCs (BC-zone slots), null: no BC rows
  int nbc;
  int32_t bc_zone[WF_MAX_BC];
  int32_t id_free_surf;
};

__global__ void __launch_bounds__(kOutThreads) k_out_partial(OutArgs A, double* __restrict__ part) {
  __shared__ double sh[kOutWarps];
  const int K = kOutFixed + 3 * A.nbc;
  double mux = 0.0, muy = 0.0, muz = 0.0, mps = 0.0;     // maxima start at 0 (SolverFraser.cu:375)
  double cs = 0.0, cx = 0.0, cy = 0.0, cz = 0.0, es = 0.0;
  const int64_t stride = (int64_t)kOutBlocks * kOutThreads;
  for (int64_t o = blockIdx.x * (int64_t)kOutThreads + threadIdx.x; o < A.n; o += stride) {
    const int64_t s = A.inv[o];
    const double4 u = A.u[s];
    mux = fmax(mux, u.x);
    muy = fmax(muy, u.y);
    muz = fmax(muz, u.z);
    mps = fmax(mps, A.eps_p[s]);
    es += A.eint[s];
    if (A.cf) {
      const double4 f = A.cf[s];
      if (A.id[s] == A.id_free_surf) cs += sqrt(f.x * f.x + f.y * f.y + f.z * f.z);
      cx += f.x;
      cy += f.y;
      cz += f.z;
    }
  }
  double* out = part + (int64_t)blockIdx.x * K;
  double r;
  r = block_reduce<true>(mux, sh); if (threadIdx.x == 0) out[0] = r;
  r = block_reduce<true>(muy, sh); if (threadIdx.x == 0) out[1] = r;
  r = block_reduce<true>(muz, sh); if (threadIdx.x == 0) out[2] = r;
  r = block_reduce<true>(mps, sh); if (threadIdx.x == 0) out[3] = r;
  r = block_reduce<false>(cs, sh); if (threadIdx.x == 0) out[4] = r;
  r = block_reduce<false>(cx, sh); if (threadIdx.x == 0) out[5] = r;
  r = block_reduce<false>(cy, sh); if (threadIdx.x == 0) out[6] = r;
  r = block_reduce<false>(cz, sh); if (threadIdx.x == 0) out[7] = r;
  r = block_reduce<false>(es, sh); if (threadIdx.x == 0) out[8] = r;
  // per BC zone: the recorded forces of its particles (a particle counts
  // once for every BC naming its zone, as every such BC acts on it)
  for (int b = 0; b < A.nbc; b++) {
    double fx = 0.0, fy = 0.0, fz = 0.0;
    if (A.fr)
      for (int64_t o = blockIdx.x * (int64_t)kOutThreads + threadIdx.x; o < A.n; o += stride) {
        const int64_t s = A.inv[o];
        if (A.id[s] == A.bc_zone[b]) {
          const double4 f = A.fr[s];
          fx += f.x;
          fy += f.y;
          fz += f.z;
        }
      }
    r = block_reduce<false>(fx, sh); if (threadIdx.x == 0) out[kOutFixed + 3 * b + 0] = r;
    r = block_reduce<false>(fy, sh); if (threadIdx.x == 0) out[kOutFixed + 3 * b + 1] = r;
    r = block_reduce<false>(fz, sh); if (threadIdx.x == 0) out[kOutFixed + 3 * b + 2] = r;
  }
}

// one thread per value: the blocks' partials in block order; thread 0 writes
// time and step.  The row goes to `last` and, when `append`, to the next row
// of the series (a device counter; rows beyond `cap` are dropped and flagged).
__global__ void k_out_final(int nbc, const double* __restrict__ part, double time, double step,
                            double* __restrict__ last, double* __restrict__ series, int64_t cap,
                            unsigned long long* __restrict__ count, int append,
                            int* __restrict__ status) {
  const int K = kOutFixed + 3 * nbc;
  const int W = K + 2;
  __shared__ unsigned long long row;
  if (threadIdx.x == 0) {
    row = append ? *count : 0ull;
    last[0] = time;
    last[1] = step;
  }
  __syncthreads();
  const bool keep = append && row < (unsigned long long)cap;
  if (threadIdx.x == 0 && keep) {
    series[row * W + 0] = time;
    series[row * W + 1] = step;
  }
  for (int k = threadIdx.x; k < K; k += blockDim.x) {
    const bool mx = k < 4;
    double r = part[k];
    for (int b = 1; b < kOutBlocks; b++) {
      const double v = part[(int64_t)b * K + k];
      r = mx ? fmax(r, v) : r + v;
    }
    last[2 + k] = r;
    if (keep) series[row * W + 2 + k] = r;
  }
  __syncthreads();
  if (threadIdx.x == 0 && append) {
    if (keep) *count = row + 1;
    else atomicOr(status, WF_STATUS_SERIES);
  }
}

}  // namespace

int wf_out_partial_words(int nbc) { return kOutBlocks * (kOutFixed + 3 * nbc); }

void launch_output_row(const StepParams& P, const Fields& F, double* part, double time,
                       double step, double* last, double* series, int64_t cap,
                       unsigned long long* count, int append, int* status, cudaStream_t s) {
  OutArgs A;
  A.n = P.n;
  A.inv = P.inv;
  A.id = F.id;
  A.u = F.u;
  A.eps_p = F.eps_p;
  A.cf = F.cf;
  A.eint = F.eint;
  A.fr = P.fr;
  A.nbc = P.nbc;
  for (int b = 0; b < WF_MAX_BC; b++) A.bc_zone[b] = b < P.nbc ? P.bc_zone[b] : 0;
  A.id_free_surf = P.id_free_surf;
  k_out_partial<<<kOutBlocks, kOutThreads, 0, s>>>(A, part);
  k_out_final<<<1, 64, 0, s>>>(P.nbc, part, time, step, last, series, cap, count, append, status);
}
