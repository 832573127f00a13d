// wf_nsearch.cu — neighbour search with cuNSearch's float32 rule, cell sort
// and physical reorder of every per-particle array.
//
// Rule (src/cuNSearch/src/cuNSearchKernels.cu:41-234, cuNSearchDeviceData.cu:
// 27-174): search radius r = float(2 h); cell = floor((p - GridMin) *
// GridDelta) in float; candidates from the 27 cells in z, y, x order;
// accept j when the float squared distance is < r*r and > 0; at most 70.
// The distance is computed with round-to-nearest intrinsics, so no fused
// multiply-add can change which pairs pass.
//
// Layout: particles are counting-sorted by linear cell index (z-major), ties
// by original id, and all state is gathered into the new order.  The three
// x-adjacent cells of a row are then one contiguous slot range, so a
// particle's candidates are 9 ranges, visited in the reference's order.
// Lists are stored in blocks of 8 entries (nb_at in wf_common.cuh): a thread
// reads 8 entries with two 16-byte loads and a warp reads contiguous memory.
#include <algorithm>

#include "wf_common.cuh"
#include "wf_nsearch.cuh"

namespace {

__device__ __forceinline__ int cell_coord(float p, float gmin, float gdelta) {
  return (int)floorf(__fmul_rn(__fsub_rn(p, gmin), gdelta));
}

// float positions the search reads: x_h snapshot or the current positions
__global__ void k_prep_positions(int64_t n, const Fields F, int use_current, float4* pf) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (use_current) {
    double4 x = F.xm[i];
    pf[i] = make_float4(__double2float_rn(x.x), __double2float_rn(x.y), __double2float_rn(x.z), 0.f);
  } else {
    pf[i] = F.xh[i];
  }
}

// kComputeMinMax: integer cell bounds of floor(p / r), block-reduced first
__global__ void k_minmax(int64_t n, const float4* __restrict__ pf, float r, int* mm) {
  __shared__ int smn[3][32], smx[3][32];
  int mn[3] = {INT_MAX, INT_MAX, INT_MAX}, mx[3] = {INT_MIN, INT_MIN, INT_MIN};
  // grid-stride over the particles: one block-reduced atomic per block
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float4 p = pf[i];
    const int c0 = (int)floorf(__fdiv_rn(p.x, r)), c1 = (int)floorf(__fdiv_rn(p.y, r)),
              c2 = (int)floorf(__fdiv_rn(p.z, r));
    mn[0] = min(mn[0], c0); mx[0] = max(mx[0], c0);
    mn[1] = min(mn[1], c1); mx[1] = max(mx[1], c1);
    mn[2] = min(mn[2], c2); mx[2] = max(mx[2], c2);
  }
  for (int a = 0; a < 3; a++) {
    for (int o = 16; o > 0; o >>= 1) {
      mn[a] = min(mn[a], __shfl_xor_sync(0xffffffffu, mn[a], o));
      mx[a] = max(mx[a], __shfl_xor_sync(0xffffffffu, mx[a], o));
    }
  }
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0)
    for (int a = 0; a < 3; a++) { smn[a][w] = mn[a]; smx[a][w] = mx[a]; }
  __syncthreads();
  if (w == 0) {
    int nw = blockDim.x >> 5;
    for (int a = 0; a < 3; a++) {
      int v = l < nw ? smn[a][l] : INT_MAX, u = l < nw ? smx[a][l] : INT_MIN;
      for (int o = 16; o > 0; o >>= 1) {
        v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
        u = max(u, __shfl_xor_sync(0xffffffffu, u, o));
      }
      if (l == 0) { atomicMin(mm + a, v); atomicMax(mm + 3 + a, u); }
    }
  }
}

__global__ void k_cell_count(int64_t n, const float4* __restrict__ pf, GridDev g,
                             uint32_t* __restrict__ cellid, uint32_t* __restrict__ count,
                             int* status) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  float4 p = pf[i];
  int cx = cell_coord(p.x, g.gmin[0], g.gdelta[0]);
  int cy = cell_coord(p.y, g.gmin[1], g.gdelta[1]);
  int cz = cell_coord(p.z, g.gmin[2], g.gdelta[2]);
  if (cx < 0 || cy < 0 || cz < 0 || cx >= g.dim[0] || cy >= g.dim[1] || cz >= g.dim[2]) {
    atomicOr(status, WF_STATUS_GRID);
    cx = min(max(cx, 0), g.dim[0] - 1);
    cy = min(max(cy, 0), g.dim[1] - 1);
    cz = min(max(cz, 0), g.dim[2] - 1);
  }
  uint32_t c = ((uint32_t)cz * g.dim[1] + cy) * g.dim[0] + cx;
  cellid[i] = c;
  atomicAdd(count + c, 1u);
}

// exclusive scan, 1024 elements per block (256 threads x 4)
__global__ void k_scan_block(uint32_t* data, int64_t n, uint32_t* block_sums) {
  __shared__ uint32_t warp_tot[8];
  int64_t base = (int64_t)blockIdx.x * 1024 + threadIdx.x * 4;
  uint32_t v[4];
  for (int k = 0; k < 4; k++) v[k] = (base + k < n) ? data[base + k] : 0u;
  uint32_t t = v[0] + v[1] + v[2] + v[3];
  uint32_t incl = t;
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) warp_tot[w] = incl;
  __syncthreads();
  if (w == 0) {
    uint32_t x = lane < 8 ? warp_tot[lane] : 0u;
    uint32_t xi = x;
    for (int o = 1; o < 8; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, xi, o);
      if (lane >= o) xi += y;
    }
    if (lane < 8) warp_tot[lane] = xi - x;
    if (lane == 7 && block_sums) block_sums[blockIdx.x] = xi;
  }
  __syncthreads();
  uint32_t run = warp_tot[w] + incl - t;
  for (int k = 0; k < 4; k++) {
    if (base + k < n) data[base + k] = run;
    run += v[k];
  }
}

__global__ void k_scan_add(uint32_t* data, int64_t n, const uint32_t* block_sums) {
  int64_t base = (int64_t)blockIdx.x * 1024 + threadIdx.x * 4;
  uint32_t add = block_sums[blockIdx.x];
  for (int k = 0; k < 4; k++)
    if (base + k < n) data[base + k] += add;
}

__global__ void k_cell_scatter(int64_t n, const uint32_t* __restrict__ cellid,
                               const uint32_t* __restrict__ start, uint32_t* __restrict__ cursor,
                               const int32_t* __restrict__ perm, int32_t* __restrict__ s_src,
                               int32_t* __restrict__ s_orig) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t c = cellid[i];
  uint32_t pos = start[c] + atomicAdd(cursor + c, 1u);
  s_src[pos] = (int32_t)i;
  s_orig[pos] = perm[i];
}

// Orders each cell's slots by original id, one warp per cell: original ids
// are distinct, so an element's place is the number of smaller ids in its
// cell (32 broadcast compares for a cell of at most 32; the cells hold ~14).
// Every lane reads before any writes.  A larger cell is insertion-sorted by
// one lane.
__global__ void k_cell_sort(int64_t ncell, const uint32_t* __restrict__ start,
                            int32_t* __restrict__ s_src, int32_t* __restrict__ s_orig) {
  const int64_t c = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (c >= ncell) return;                      // whole warps leave together
  const uint32_t b = start[c], e = start[c + 1];
  const uint32_t m = e - b;
  if (m <= 1u) return;
  if (m <= 32u) {
    const bool v = (uint32_t)lane < m;
    const int32_t o = v ? s_orig[b + lane] : 0;
    const int32_t sv = v ? s_src[b + lane] : 0;
    uint32_t rank = 0;
    for (uint32_t t = 0; t < m; t++) rank += __shfl_sync(0xffffffffu, o, (int)t) < o;
    __syncwarp();
    if (v) {
      s_orig[b + rank] = o;
      s_src[b + rank] = sv;
    }
    return;
  }
  if (lane != 0) return;
  for (uint32_t k = b + 1; k < e; k++) {
    const int32_t ko = s_orig[k], ks = s_src[k];
    uint32_t q = k;
    while (q > b && s_orig[q - 1] > ko) {
      s_orig[q] = s_orig[q - 1];
      s_src[q] = s_src[q - 1];
      q--;
    }
    s_orig[q] = ko;
    s_src[q] = ks;
  }
}

template <class T>
__device__ __forceinline__ void g1(T* dst, const T* src, int64_t k, int64_t s) {
  if (dst) dst[k] = src[s];
}
__device__ __forceinline__ void g6(double* dst, const double* src, int64_t k, int64_t s) {
  if (!dst) return;
  const double2* a = reinterpret_cast<const double2*>(src + 6 * s);
  double2* b = reinterpret_cast<double2*>(dst + 6 * k);
  b[0] = a[0]; b[1] = a[1]; b[2] = a[2];
}
__device__ __forceinline__ void g6f(float* dst, const float* src, int64_t k, int64_t s) {
  if (!dst) return;
  const float2* a = reinterpret_cast<const float2*>(src + 6 * s);
  float2* b = reinterpret_cast<float2*>(dst + 6 * k);
  b[0] = a[0]; b[1] = a[1]; b[2] = a[2];
}

// gather every per-slot array into the new order; inv[orig] = new slot
__global__ void k_reorder(int64_t n, const int32_t* __restrict__ s_src, const Fields A, Fields B,
                          const float4* __restrict__ pf, float4* __restrict__ pf2,
                          int32_t* __restrict__ inv) {
  int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= n) return;
  int64_t s = s_src[k];
  g1(B.xm, A.xm, k, s); g1(B.vd, A.vd, k, s); g1(B.u, A.u, k, s); g1(B.a, A.a, k, s);
  g6(B.sig6, A.sig6, k, s); g6(B.ss6, A.ss6, k, s); g6(B.eps6, A.eps6, k, s);
  g6(B.sr6, A.sr6, k, s); g6(B.rr6, A.rr6, k, s);
  g1(B.p, A.p, k, s); g1(B.seq, A.seq, k, s); g1(B.eps_p, A.eps_p, k, s); g1(B.sy, A.sy, k, s);
  g1(B.eff, A.eff, k, s); g1(B.dep, A.dep, k, s); g1(B.drho, A.drho, k, s);
  g1(B.eint, A.eint, k, s);
  g1(B.T, A.T, k, s); g1(B.Ta, A.Ta, k, s); g1(B.Tb, A.Tb, k, s); g1(B.dTdt, A.dTdt, k, s);
  g1(B.kT, A.kT, k, s); g1(B.cpT, A.cpT, k, s);
  g1(B.id, A.id, k, s); g1(B.bct, A.bct, k, s); g1(B.nw, A.nw, k, s); g1(B.xh, A.xh, k, s);
  g1(B.p32, A.p32, k, s); g1(B.v32, A.v32, k, s); g6f(B.ss32, A.ss32, k, s);
  g1(B.th32, A.th32, k, s); g1(B.pwn, A.pwn, k, s);
  g1(B.nrm, A.nrm, k, s); g1(B.cf, A.cf, k, s); g1(B.qf, A.qf, k, s);
  g1(B.eps_rb, A.eps_rb, k, s);
  int32_t o = A.perm[s];
  B.perm[k] = o;
  inv[o] = (int32_t)k;
  pf2[k] = pf[s];
}

// Neighbour lists, one warp per cell.  The particles of a cell share its
// candidate set: the nine rows of three x-adjacent cells around it, each one
// contiguous range of sorted slots, visited z outer, y, x inner
// (cuNSearchKernels.cu:170-234).  The warp stages in shared memory, in that
// order, the candidates that lie within r of the box around its particles
// (any other one fails the distance test for all of them: the box distance
// is at most the distance to each particle, and a 1e-4 relative margin
// covers the FP32 rounding of both).  Then, for each chunk of 32 staged
// candidates and each particle, the lanes test their candidate against that
// particle with the float rule and the accepted ones are appended in
// candidate order (ballot, prefix popcount).  Lists, counts and the 70-entry
// cap are those of a per-particle scan, entry for entry; the staging halves
// the distance tests (a CPU model of the jittered lattice keeps 161 of 332
// candidates per cell) and the warp shares one candidate range, where
// particles scanned by separate lanes diverge at cell boundaries.  786k
// particles: 0.295 ms per rebuild against 0.385 for the per-particle scan
// (0.348 with 64-bit entry indices in the append loop).
// slot_of == nullptr: the state is in sorted order (sorted index = slot);
// else slot_of[k] is the storage slot of the k-th sorted particle.
constexpr int kNbWarps = 4;      // warps (cells in flight) per block
// List entry index (nb_at) in the index type I: 32-bit when the lists hold
// fewer than 2^31 entries (fewer than ~29M particles), else 64-bit.
template <class I>
__device__ __forceinline__ I nb_at_i(I npad, I i, int k) {
  return ((I)(k >> 3) * npad + i) * (I)WF_NB_BLK + (I)(k & 7);
}
constexpr int kNbStage = 192;    // staged candidates per warp and round

// Tests the staged candidates against the group's particles (part[j]: position
// and, in w, the storage slot of particle j, whose count lane j holds) and appends the accepted ones to their lists.  Per chunk of 32
// candidates and per particle j, one ballot gives the accepting lanes; each
// writes its candidate at j's count before the chunk plus the accepting lanes
// below it, so the entries keep candidate order.  The counts advance once per
// chunk (lane j keeps particle j's mask of the chunk), which leaves no chain
// between the particles' iterations.
template <class I>
__device__ __forceinline__ void nb_append_round(int nstaged, const float4* __restrict__ sp,
                                                const int32_t* __restrict__ sid, int gn,
                                                const float4* __restrict__ part, float r2,
                                                int64_t npad, int32_t* __restrict__ nb,
                                                int& count) {
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  for (int ch = 0; ch < nstaged; ch += 32) {
    const int t = ch + lane;
    const bool v = t < nstaged;
    const float4 q = v ? sp[t] : make_float4(0.f, 0.f, 0.f, 0.f);
    const int32_t qid = v ? sid[t] : 0;
    unsigned mine = 0u;
#pragma unroll 4
    for (int j = 0; j < gn; j++) {
      const float4 pj = part[j];   // same address on every lane: one broadcast read
      const int32_t ij = __float_as_int(pj.w);
      const int base = __shfl_sync(0xffffffffu, count, j);
      const float dx = __fsub_rn(q.x, pj.x), dy = __fsub_rn(q.y, pj.y), dz = __fsub_rn(q.z, pj.z);
      const float sq =
          __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
      const bool acc = v && sq < r2 && sq > 0.0f;
      const unsigned m = __ballot_sync(0xffffffffu, acc);
      const int k = base + __popc(m & lt);
      if (acc && k < WF_NB) nb[nb_at_i<I>((I)npad, (I)ij, k)] = qid;
      mine = lane == j ? m : mine;
    }
    count += __popc(mine);
  }
}

template <class I>
__global__ void __launch_bounds__(32 * kNbWarps) k_nblist(int64_t ncell, int64_t npad,
                                                          const float4* __restrict__ pf, GridDev g,
                                                          const uint32_t* __restrict__ start,
                                                          const int32_t* __restrict__ slot_of,
                                                          int32_t* __restrict__ nb,
                                                          int32_t* __restrict__ cnt, int* status) {
  __shared__ float4 s_pos[kNbWarps][kNbStage];
  __shared__ int32_t s_id[kNbWarps][kNbStage];
  __shared__ float4 s_part[kNbWarps][32];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t c = blockIdx.x * (int64_t)kNbWarps + w;
  if (c >= ncell) return;                      // whole warps leave together
  const uint32_t ps = start[c], pe = start[c + 1];
  if (ps >= pe) return;
  // cell coordinates in 32-bit arithmetic (the grid holds at most 2e9 cells;
  // a 64-bit division is a long software sequence in this issue-bound kernel)
  const uint32_t cu = (uint32_t)c, dx = (uint32_t)g.dim[0], dy = (uint32_t)g.dim[1];
  const uint32_t cyz = cu / dx;
  const int cx = (int)(cu - cyz * dx);
  const int cy = (int)(cyz % dy);
  const int cz = (int)(cyz / dy);
  // row r = 3 (dz + 1) + (dy + 1): slot range [rb, rb + rn) on lane r
  uint32_t rb = 0, rn = 0;
  if (lane < 9) {
    const int fz = cz + lane / 3 - 1, fy = cy + lane % 3 - 1;
    if (fz >= 0 && fz < g.dim[2] && fy >= 0 && fy < g.dim[1]) {
      const int x0 = max(cx - 1, 0), x1 = min(cx + 1, g.dim[0] - 1);
      const uint32_t rowc = ((uint32_t)fz * g.dim[1] + fy) * g.dim[0];
      rb = start[rowc + x0];
      rn = start[rowc + x1 + 1] - rb;
    }
  }
  const float r2 = g.r2, thr = r2 * 1.0001f;
  float4* sp = s_pos[w];
  int32_t* sid = s_id[w];
  for (uint32_t g0 = ps; g0 < pe; g0 += 32) {
    const int gn = (int)min(32u, pe - g0);
    // this group's particles (lane j < gn holds particle g0 + j) and their box
    float px = 0.f, py = 0.f, pz = 0.f;
    int32_t myslot = 0;
    float lo[3], hi[3];
    if (lane < gn) {
      const float4 p = pf[g0 + lane];
      px = p.x; py = p.y; pz = p.z;
      myslot = slot_of ? slot_of[g0 + lane] : (int32_t)(g0 + lane);
      s_part[w][lane] = make_float4(px, py, pz, __int_as_float(myslot));
    }
    {
      const float4 p0 = pf[g0];
      lo[0] = hi[0] = lane < gn ? px : p0.x;
      lo[1] = hi[1] = lane < gn ? py : p0.y;
      lo[2] = hi[2] = lane < gn ? pz : p0.z;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
      for (int a = 0; a < 3; a++) {
        lo[a] = fminf(lo[a], __shfl_xor_sync(0xffffffffu, lo[a], o));
        hi[a] = fmaxf(hi[a], __shfl_xor_sync(0xffffffffu, hi[a], o));
      }
    int count = 0;
    int nstaged = 0;
    for (int r = 0; r < 9; r++) {
      const uint32_t b = __shfl_sync(0xffffffffu, rb, r);
      const uint32_t nr = __shfl_sync(0xffffffffu, rn, r);
      for (uint32_t t0 = 0; t0 < nr; t0 += 32) {
        if (nstaged > kNbStage - 32) {          // staging full: test what is staged
          __syncwarp();
          nb_append_round<I>(nstaged, sp, sid, gn, s_part[w], r2, npad, nb, count);
          __syncwarp();
          nstaged = 0;
        }
        const bool v = t0 + lane < nr;
        const uint32_t s = b + t0 + lane;
        float4 q = make_float4(0.f, 0.f, 0.f, 0.f);
        int32_t id = (int32_t)s;
        bool keep = false;
        if (v) {
          q = pf[s];
          if (slot_of) id = slot_of[s];
          const float ex = fmaxf(0.f, fmaxf(lo[0] - q.x, q.x - hi[0]));
          const float ey = fmaxf(0.f, fmaxf(lo[1] - q.y, q.y - hi[1]));
          const float ez = fmaxf(0.f, fmaxf(lo[2] - q.z, q.z - hi[2]));
          keep = ex * ex + ey * ey + ez * ez < thr;
        }
        const unsigned m = __ballot_sync(0xffffffffu, keep);
        if (keep) {
          const int at = nstaged + __popc(m & ((1u << lane) - 1u));
          sp[at] = q;
          sid[at] = id;
        }
        nstaged += __popc(m);
      }
    }
    __syncwarp();
    nb_append_round<I>(nstaged, sp, sid, gn, s_part[w], r2, npad, nb, count);
    __syncwarp();
    if (lane < gn) {
      if (count >= WF_NB) atomicOr(status, WF_STATUS_NB_CAP);
      const int cn = min(count, WF_NB);
      cnt[myslot] = cn;
      // pad the last block with the particle's own slot (see nb_at)
      for (int k = cn; k < ((cn + WF_NB_BLK - 1) & ~(WF_NB_BLK - 1)); k++)
        nb[nb_at(npad, myslot, k)] = myslot;
    }
  }
}

// the search positions in sorted order, for a rebuild that keeps the state in place
__global__ void k_gather_pf(int64_t n, const int32_t* __restrict__ s_src,
                            const float4* __restrict__ pf, float4* __restrict__ pf2) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k < n) pf2[k] = pf[s_src[k]];
}

__global__ void k_snapshot(int64_t n, Fields F) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  double4 x = F.xm[i];
  F.xh[i] = make_float4(__double2float_rn(x.x), __double2float_rn(x.y), __double2float_rn(x.z), 0.f);
}

inline int nblocks(int64_t n, int t) { return (int)((n + t - 1) / t); }

}  // namespace

// host-side grid set-up, computeCellInformation (cuNSearchDeviceData.cu:80-123)
void grid_from_minmax(const int mm[6], float r, GridDev* g) {
  for (int a = 0; a < 3; a++) {
    float Min = (float)mm[a] * r, Max = (float)mm[3 + a] * r;
    float gridSize = Max - Min;
    g->dim[a] = (int)((unsigned)ceilf(gridSize / r) + 4u);
    g->gmin[a] = Min - r * 2.0f;
    float gs2 = (float)(unsigned)g->dim[a] * r;
    g->gdelta[a] = (float)(unsigned)g->dim[a] / gs2;
  }
  g->r2 = r * r;
}

void device_exclusive_scan(uint32_t* data, int64_t n, uint32_t* tmp, cudaStream_t s) {
  int64_t nb = (n + 1023) / 1024;
  if (nb <= 1) {
    k_scan_block<<<1, 256, 0, s>>>(data, n, nullptr);
    return;
  }
  k_scan_block<<<(int)nb, 256, 0, s>>>(data, n, tmp);
  device_exclusive_scan(tmp, nb, tmp + nb, s);
  k_scan_add<<<(int)nb, 256, 0, s>>>(data, n, tmp);
}

int64_t scan_tmp_words(int64_t n) {
  int64_t w = 0;
  while (n > 1024) {
    n = (n + 1023) / 1024;
    w += n;
  }
  return w + 1;
}

void launch_prep_positions(int64_t n, const Fields& F, int use_current, float4* pf,
                           cudaStream_t s) {
  k_prep_positions<<<nblocks(n, 256), 256, 0, s>>>(n, F, use_current, pf);
}
void launch_minmax(int64_t n, const float4* pf, float r, int* mm, cudaStream_t s) {
  k_minmax<<<std::min(nblocks(n, 256), 1024), 256, 0, s>>>(n, pf, r, mm);
}
void launch_cell_count(int64_t n, const float4* pf, const GridDev& g, uint32_t* cellid,
                       uint32_t* count, int* status, cudaStream_t s) {
  k_cell_count<<<nblocks(n, 256), 256, 0, s>>>(n, pf, g, cellid, count, status);
}
void launch_cell_scatter(int64_t n, const uint32_t* cellid, const uint32_t* start,
                         uint32_t* cursor, const int32_t* perm, int32_t* s_src, int32_t* s_orig,
                         cudaStream_t s) {
  k_cell_scatter<<<nblocks(n, 256), 256, 0, s>>>(n, cellid, start, cursor, perm, s_src, s_orig);
}
void launch_cell_sort(int64_t ncell, const uint32_t* start, int32_t* s_src, int32_t* s_orig,
                      cudaStream_t s) {
  k_cell_sort<<<nblocks(ncell * 32, 256), 256, 0, s>>>(ncell, start, s_src, s_orig);
}
void launch_reorder(int64_t n, const int32_t* s_src, const Fields& A, const Fields& B,
                    const float4* pf, float4* pf2, int32_t* inv, cudaStream_t s) {
  k_reorder<<<nblocks(n, 256), 256, 0, s>>>(n, s_src, A, B, pf, pf2, inv);
}
void launch_nblist(int64_t n, int64_t npad, const float4* pf, const GridDev& g,
                   const uint32_t* start, const int32_t* slot_of, int32_t* nb, int32_t* cnt,
                   int* status, cudaStream_t s) {
  (void)n;
  const int64_t ncell = (int64_t)g.dim[0] * g.dim[1] * g.dim[2];
  if ((int64_t)WF_NB_ALLOC * npad < ((int64_t)1 << 31))
    k_nblist<uint32_t><<<nblocks(ncell, kNbWarps), 32 * kNbWarps, 0, s>>>(
        ncell, npad, pf, g, start, slot_of, nb, cnt, status);
  else
    k_nblist<int64_t><<<nblocks(ncell, kNbWarps), 32 * kNbWarps, 0, s>>>(
        ncell, npad, pf, g, start, slot_of, nb, cnt, status);
}
void launch_gather_pf(int64_t n, const int32_t* s_src, const float4* pf, float4* pf2,
                      cudaStream_t s) {
  k_gather_pf<<<nblocks(n, 256), 256, 0, s>>>(n, s_src, pf, pf2);
}
void launch_snapshot(int64_t n, const Fields& F, cudaStream_t s) {
  k_snapshot<<<nblocks(n, 256), 256, 0, s>>>(n, F);
}
