// wf_step_fp32.cu — mixed-precision form of the Fraser step.
//
// Pair loops, the Jaumann/J2 stress update and the heat flux run in FP32 with
// FP32 accumulation in the fixed neighbour order.  Kept in FP64 (they sum
// ~1e-7 s increments over long runs): positions, displacements, velocities
// and their update, density accumulation, equivalent plastic strain, yield
// stress and the Newton residual, and every reduction.  The gathered
// neighbour data are FP32 mirrors written by the integration kernel:
// p32 = (x, m), v32 = (v, rho), and (after the density pass) v32b = (v, rho_new).
// All FP32 constants arrive precomputed in StepParams: on GB300 a per-thread
// FP64 division or conversion costs as much as the whole FP32 pair loop.
#include "wf_common.cuh"
#include "wf_heat.cuh"
#include "wf_integrate.cuh"
#include "wf_mlp.cuh"
#include "wf_tensor.cuh"
#include "wf_tiles.cuh"

namespace {

struct T3f {
  float xx, xy, xz, yx, yy, yz, zx, zy, zz;
};

// operator*(tensor3, tensor3) of src/cuda/tensor3.cu:241-256 in FP32
__device__ __forceinline__ T3f mul_ref_f(const T3f& a, const T3f& b) {
  T3f r;
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

// ---- A32: density rate + update (InteractionAlt.cu:166-246, Mechanical.cu:198) --
// Lane groups of the pair passes: kLanes consecutive lanes share one particle;
// lane g of the group takes entries [8b + g W, 8b + (g + 1) W) of every list
// block b (W = 8 / kLanes, the list readers' sub<W>), and the lanes' partial
// sums are combined by an xor-shuffle tree, which gives every lane of the
// group the same value.  A warp then covers fewer particles and its gathers
// touch fewer L1 lines (the neighbours of consecutive sorted particles
// overlap), and each lane's chain of dependent gathers is shorter.

// lane group of G lanes (a power of two) that share one particle
template <int G>
__device__ __forceinline__ unsigned group_mask() {
  if constexpr (G == 32) return 0xffffffffu;
  return ((1u << G) - 1u) << ((threadIdx.x & 31u) & ~(unsigned)(G - 1));
}

// Density + heat pass: one lane per particle (786k particles: 0.199 ms with
// one lane and 6 blocks per SM, 0.202-0.213 ms with 2 or 4 lanes).
constexpr int kDensLanes = 1;
constexpr int kDensMinBlocks = 6;
constexpr int kDensBatch = 4;

// ---- A32 + heat: the previous step's heat pass fused into this density pass.
// Heat at the end of step n (ThermalSolveKernel + plastic heat + convection +
// leapfrog, src/cuda/Thermal.cu:16-142) and the density pass of step n+1 read
// the same positions x^{n+1}, velocities and densities, so one walk over the
// neighbour list serves both.  Neighbour temperatures come from the th32
// mirror (T^n, written by the integration kernel), so each thread may update
// its own FP64 temperature in place.  After a rebuild at the start of step
// n+1 the heat flux of step n uses the new list (built for these positions).
// The pair loop of the density + heat pass over the neighbour list L: its
// entries are slots (NbList32 / NbList16: records gathered from the global
// arrays gp, gv, gt) or ranks in the tile's halo (NbListS: the arrays are its
// shared-memory copies).
template <class L, bool kHeat = true>
__device__ __forceinline__ void density_heat_pairs(const StepParams& P, const Fields& F,
                                                   const float4* __restrict__ gp,
                                                   const float4* __restrict__ gv,
                                                   const float2* __restrict__ gt, const L& list,
                                                   int g, int c, float4 pi, float4 vi, float2 ti,
                                                   bool solid, int32_t idi, float& drho_out,
                                                   float& sf_out) {
  constexpr int W = WF_NB_BLK / kDensLanes;
  constexpr int NB = W < kDensBatch ? W : kDensBatch;   // neighbours gathered per batch
  const float invh = P.invhf, C = P.Cf, Ch = P.Chf;
  float drho = 0.0f, sf = 0.0f;
  int nx[W];
  if (c > 0) list.template sub<W>(0, g, nx);
  for (int b = 0; WF_NB_BLK * b < c; b++) {
    int js[W];
#pragma unroll
    for (int q = 0; q < W; q++) js[q] = nx[q];
    const int m = c - WF_NB_BLK * b - g * W;   // entries of this lane's sub-block in the list
    if (P.nb_pf && c > WF_NB_BLK * (b + P.nb_pf)) list.prefetch(b + P.nb_pf, kDensLanes);
    if (c > WF_NB_BLK * (b + 1)) list.template sub<W>(b + 1, g, nx);
#pragma unroll
    for (int h = 0; h < W; h += NB) {
      float4 pj[NB], vj[NB];
      float2 tj[NB];
#pragma unroll
      for (int q = 0; q < NB; q++) {
        pj[q] = gp[js[h + q]];
        vj[q] = gv[js[h + q]];
        if constexpr (kHeat) tj[q] = gt[js[h + q]];
      }
#pragma unroll
      for (int q = 0; q < NB; q++) {
        // Entries past the count are the particle's own slot (list padding):
        // r^2 = 0 gives GK = 0 exactly (gk32_r2), so they add exact zeros and
        // need no test, except under the contact filter.
        if (P.contact && h + q >= m) continue;
        const float xx = pi.x - pj[q].x, xy = pi.y - pj[q].y, xz = pi.z - pj[q].z;
        const float GK = gk32_r2(xx * xx + xy * xy + xz * xz, invh, Ch, C);
        // m_j / rho_j GK, shared by both sums
        const float mg = __fdividef(pj[q].w, vj[q].w) * GK;
        // heat flux (every particle, no contact filter); the pair
        // conductivity 4 k_i k_j / (k_i + k_j) = 2k multiplies the sum
        if constexpr (kHeat) {
          const float dT = (ti.x - tj[q].x) + (ti.y - tj[q].y);
          sf += mg * dT;
        }
        // density rate (solid particles, contact filter); rho_i multiplies the sum
        bool pass = solid;
        if constexpr (L::kSlots) pass = pass && !(P.contact && !pass_ij(P, idi, F.id[js[h + q]]));
        if (pass) {
          const float vx = vi.x - vj[q].x, vy = vi.y - vj[q].y, vz = vi.z - vj[q].z;
          drho += mg * (vx * xx + vy * xy + vz * xz);
        }
      }
    }
  }
  drho_out = drho * vi.w;
  sf_out = sf;
}

// ---- A32: the density pass without a heat pass to fuse (a call's first
// step; every step when heat is off): the density sum of density_heat_pairs.
__global__ void __launch_bounds__(128, kDensMinBlocks) k_density32(StepParams P, Fields F,
                                                                  double4* __restrict__ vd2,
                                                                  float4* __restrict__ v32b,
                                                                  const int32_t* __restrict__ nb,
                                                                  const int32_t* __restrict__ cnt,
                                                                  const List16 L16) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= P.n) return;
  const bool solid = F.perm[i] < P.n_solid;
  if (P.state_pf) prefetch_l2(F.vd + i);
  if (P.pf_ahead > 0) {
    const int64_t ia = i + P.pf_ahead;      // the slot this thread's successor will take
    if (ia < P.n) {
      prefetch_l2(F.p32 + ia); prefetch_l2(F.v32 + ia); prefetch_l2(cnt + ia);
      prefetch_l2(F.perm + ia);
      for (int b = 0; b < P.wave_pf && b < WF_NB_BLOCKS; b++) nb_prefetch(nb, P.npad, ia, b, 4);
    }
  }
  const float4 pi = F.p32[i];
  const float4 vi = F.v32[i];
  const int c = solid ? cnt[i] : 0;
  const int32_t idi = F.id[i];
  float drho = 0.0f, sf = 0.0f;
  const int b16 = L16.base ? L16.base[i / WF_TILE] : -1;     // uniform over the block
  const float2 t0 = make_float2(0.f, 0.f);
  if (b16 >= 0)
    density_heat_pairs<NbList16, false>(P, F, F.p32, F.v32, nullptr,
                                        NbList16{L16.off, P.npad, i, b16}, 0, c, pi, vi, t0, solid,
                                        idi, drho, sf);
  else
    density_heat_pairs<NbList32, false>(P, F, F.p32, F.v32, nullptr, NbList32{nb, P.npad, i}, 0,
                                        c, pi, vi, t0, solid, idi, drho, sf);
  const double4 vdi = F.vd[i];
  double rho_new = vdi.w;
  if (solid) {
    F.drho[i] = (double)drho;
    rho_new = vdi.w + P.dt * (double)drho;
  }
  vd2[i] = make_double4(vdi.x, vdi.y, vdi.z, rho_new);
  v32b[i] = make_float4(vi.x, vi.y, vi.z, (float)rho_new);
}

__global__ void __launch_bounds__(128, kDensMinBlocks) k_density_heat32(StepParams P, Fields F,
                                                        double4* __restrict__ vd2,
                                                        float4* __restrict__ v32b,
                                                        const int32_t* __restrict__ nb,
                                                        const int32_t* __restrict__ cnt,
                                                        int first, int plastic_heat,
                                                        const TileHalo T, const List16 L16) {
  // tile staging (one lane per particle: a block of 128 threads is one tile)
  extern __shared__ __align__(16) uint8_t sdh[];
  float4* sp = reinterpret_cast<float4*>(sdh);
  float4* sv = sp + T.cap;
  float2* st = reinterpret_cast<float2*>(sv + T.cap);
  uint16_t* sl = reinterpret_cast<uint16_t*>(st + T.cap);
  int staged = -1;
  if (kDensLanes == 1 && T.cap > 0) {
    float4* dst[2] = {sp, sv};
    const float4* src[2] = {F.p32, F.v32};
    const int H = T.hcnt[blockIdx.x];
    if (H >= 0 && H <= T.cap) {                 // uniform over the block
      const int32_t* hs = T.halo + T.hoff[blockIdx.x];
      for (int k = threadIdx.x; k < H; k += blockDim.x) {
        const int s = hs[k];
        cp_async16(dst[0] + k, src[0] + s);
        cp_async16(dst[1] + k, src[1] + s);
        cp_async8(st + k, F.th32 + s);
      }
      stage_lists(T.nbl, P.npad, blockIdx.x, sl);
      cp_async_wait_all();
      __syncthreads();
      staged = H;
    }
  }
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int g = (int)(t & (kDensLanes - 1));
  const int64_t i = t / kDensLanes;
  if (i >= P.n) return;
  const float4 pi = F.p32[i];
  const float4 vi = F.v32[i];
  const float2 ti = F.th32[i];
  const bool solid = F.perm[i] < P.n_solid;
  const int32_t idi = F.id[i];
  if (P.state_pf && g == 0) {
    prefetch_l2(F.vd + i); prefetch_l2(F.T + i); prefetch_l2(F.cpT + i);
    prefetch_l2(F.dep + i); prefetch_l2(F.sy + i); prefetch_l2(F.Ta + i);
  }
  if (P.pf_ahead > 0 && g == 0) {
    const int64_t ia = i + P.pf_ahead;      // the slot this thread's successor will take
    if (ia < P.n) {
      prefetch_l2(F.p32 + ia); prefetch_l2(F.v32 + ia); prefetch_l2(F.th32 + ia);
      prefetch_l2(cnt + ia); prefetch_l2(F.perm + ia);
      for (int b = 0; b < P.wave_pf && b < WF_NB_BLOCKS; b++) nb_prefetch(nb, P.npad, ia, b, 4);
    }
  }
  float drho, sf;
  const int c = cnt[i];
  const int b16 = L16.base ? L16.base[i / WF_TILE] : -1;     // uniform over the block
  if (staged >= 0)
    density_heat_pairs(P, F, sp, sv, st, NbListS{sl, (int)threadIdx.x}, g, c, pi, vi, ti, solid,
                       idi, drho, sf);
  else if (b16 >= 0)
    density_heat_pairs(P, F, F.p32, F.v32, F.th32, NbList16{L16.off, P.npad, i, b16}, g, c, pi, vi,
                       ti, solid, idi, drho, sf);
  else
    density_heat_pairs(P, F, F.p32, F.v32, F.th32, NbList32{nb, P.npad, i}, g, c, pi, vi, ti, solid,
                       idi, drho, sf);
  if constexpr (kDensLanes > 1) {
    const unsigned mask = group_mask<kDensLanes>();
#pragma unroll
    for (int o = 1; o < kDensLanes; o <<= 1) {
      sf += __shfl_xor_sync(mask, sf, o, kDensLanes);
      drho += __shfl_xor_sync(mask, drho, o, kDensLanes);
    }
  }
  if (g != 0) return;
  const double4 vdi = F.vd[i];
  // heat of the previous step: rate and leapfrog, own particle only
  const double dTdt = heat_rate_mixed(P, F, i, P.k2f * sf, vdi.w, (double)pi.w, F.T[i], plastic_heat);
  F.dTdt[i] = dTdt;
  heat_leapfrog_one(P, F, i, dTdt, first);
  // density of this step
  double rho_new = vdi.w;
  if (solid) {
    F.drho[i] = (double)drho;
    rho_new = vdi.w + P.dt * (double)drho;
  }
  vd2[i] = make_double4(vdi.x, vdi.y, vdi.z, rho_new);
  v32b[i] = make_float4(vi.x, vi.y, vi.z, (float)rho_new);
}

// ---- the heat pass alone (ThermalSolveKernel, src/cuda/Thermal.cu:101-142) --
// A call's last heat pass and every step of the mixed ThermalSolve: the heat
// sum of density_heat_pairs, the same operations in the same neighbour order
// (so a separate pass gives the fused pass's sum bit for bit), with the
// neighbour's density read as one float of its velocity record.
template <class L>
__device__ __forceinline__ float heat_pairs(const StepParams& P, const float4* __restrict__ gp,
                                            const float4* __restrict__ gv,
                                            const float2* __restrict__ gt, const L& list, int c,
                                            float4 pi, float2 ti) {
  constexpr int NB = kDensBatch;
  const float invh = P.invhf, C = P.Cf, Ch = P.Chf;
  float sf = 0.0f;
  int nx[WF_NB_BLK];
  if (c > 0) list.block(0, nx);
  for (int b = 0; WF_NB_BLK * b < c; b++) {
    int js[WF_NB_BLK];
#pragma unroll
    for (int q = 0; q < WF_NB_BLK; q++) js[q] = nx[q];
    if (P.nb_pf && c > WF_NB_BLK * (b + P.nb_pf)) list.prefetch(b + P.nb_pf, 1);
    if (c > WF_NB_BLK * (b + 1)) list.block(b + 1, nx);
#pragma unroll
    for (int h = 0; h < WF_NB_BLK; h += NB) {
      float4 pj[NB];
      float rj[NB];
      float2 tj[NB];
#pragma unroll
      for (int q = 0; q < NB; q++) {
        pj[q] = gp[js[h + q]];
        rj[q] = __ldg(&gv[js[h + q]].w);
        tj[q] = gt[js[h + q]];
      }
#pragma unroll
      for (int q = 0; q < NB; q++) {
        // padding entries (the particle's own slot) add exact zeros (gk32_r2)
        const float xx = pi.x - pj[q].x, xy = pi.y - pj[q].y, xz = pi.z - pj[q].z;
        const float GK = gk32_r2(xx * xx + xy * xy + xz * xz, invh, Ch, C);
        const float mg = __fdividef(pj[q].w, rj[q]) * GK;
        const float dT = (ti.x - tj[q].x) + (ti.y - tj[q].y);
        sf += mg * dT;
      }
    }
  }
  return sf;
}

__global__ void __launch_bounds__(128, kDensMinBlocks) k_heat32(StepParams P, Fields F,
                                                               const int32_t* __restrict__ nb,
                                                               const int32_t* __restrict__ cnt,
                                                               int plastic_heat) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= P.n) return;
  if (P.state_pf) {
    prefetch_l2(F.vd + i); prefetch_l2(F.xm + i); prefetch_l2(F.T + i); prefetch_l2(F.cpT + i);
    prefetch_l2(F.dep + i); prefetch_l2(F.sy + i);
  }
  if (P.pf_ahead > 0) {
    const int64_t ia = i + P.pf_ahead;      // the slot this thread's successor will take
    if (ia < P.n) {
      prefetch_l2(F.p32 + ia); prefetch_l2(F.th32 + ia); prefetch_l2(cnt + ia);
      for (int b = 0; b < P.wave_pf && b < WF_NB_BLOCKS; b++) nb_prefetch(nb, P.npad, ia, b, 4);
    }
  }
  const float4 pi = F.p32[i];
  const float2 ti = F.th32[i];
  const int c = cnt[i];
  const float sf = heat_pairs(P, F.p32, F.v32, F.th32, NbList32{nb, P.npad, i}, c, pi, ti);
  F.dTdt[i] = heat_rate_mixed(P, F, i, P.k2f * sf, F.vd[i].w, F.xm[i].w, F.T[i], plastic_heat);
}

// Johnson-Cook consistent return map of the mixed form, solved for the
// increment.  With the cached power pwn = ep^n and u = dl / ep,
//   f(dl) = d0 - 3G dl - B RT pwn ((1 + u)^n - 1),   d0 = st - (A + B pwn) RT,
// is the same residual as st - 3G dl - (A + B (ep + dl)^n) RT, but every term
// is of the size of the overshoot d0, so FP32 resolves the root to ~1e-7 of dl
// (st itself is an FP32 value).  The written form subtracts numbers ~1e3 times
// larger than d0 and needs FP64, which GB300 issues at 1/64 of the FP32 rate.
// Valid while the bracket [0, d0 / 3G] keeps u below 0.05: the 5-term binomial
// series of (1 + u)^n - 1 then has a relative truncation error of about
// |C(n,6)|/n u^5 (1.7e-8 for n = 0.42, below FP32 rounding; 0.05^5/6 = 5e-8 for
// any n <= 1).  Returns false otherwise (first yield, large increments, a power
// refresh step) and the caller takes the FP64 form.  On success pwn is advanced
// to (ep + dl)^n in FP64.
__device__ __forceinline__ bool jc_return_inc32(const StepParams& P, float st, float RT,
                                                double ep, double& pwn, float dl_ratio,
                                                float* dl_out, float* sy_out, int* iters) {
  if (!(pwn >= 0.0) || P.refresh_pow || !(ep > 0.0)) return false;
  const float pw = (float)pwn;
  const float BRp = P.jcBf * RT * pw;
  const float sy0 = P.jcAf * RT + BRp;
  const float d0 = st - sy0;
  *iters = 0;
  if (!(d0 > 0.0f)) {
    *dl_out = 0.0f;
    *sy_out = sy0;
    return true;
  }
  const float epf = (float)ep;
  float hi = d0 / P.G3f, lo = 0.0f;
  if (!(hi < 0.05f * epf)) return false;
  const float inv_ep = 1.0f / epf;
  const float b0 = P.binf[0], b1 = P.binf[1], b2 = P.binf[2], b3 = P.binf[3], b4 = P.binf[4];
  const float tol = fmaxf((float)P.newton_rtol * st, 16.0f * 1.1920929e-7f * d0);
  float dl = (dl_ratio > 0.0f && dl_ratio <= 1.0f) ? dl_ratio * hi : hi;
  int it = 0;
  for (; it < P.newton_max_iter; it++) {
    const float u = dl * inv_ep;
    const float ser = u * (b0 + u * (b1 + u * (b2 + u * (b3 + u * b4))));
    const float f = d0 - P.G3f * dl - BRp * ser;
    if (fabsf(f) <= tol) break;
    if (f > 0.0f) lo = dl; else hi = dl;
    // f'(dl) = -3G - B RT pwn n (1 + u)^(n - 1) / ep
    const float dser =
        inv_ep * (b0 + u * (2.0f * b1 + u * (3.0f * b2 + u * (4.0f * b3 + u * 5.0f * b4))));
    float dn = dl + f / (P.G3f + BRp * dser);
    if (!(dn > lo && dn < hi)) dn = 0.5f * (lo + hi);
    dl = dn;
  }
  const float u = dl * inv_ep;
  const float ser = u * (b0 + u * (b1 + u * (b2 + u * (b3 + u * b4))));
  *iters = it;
  *dl_out = dl;
  *sy_out = sy0 + BRp * ser;
  pwn += pwn * (double)ser;
  return true;
}

// ---- B32: rate tensors + EOS + stress (InteractionAlt.cu:262-383,
//      Mechanical.cu:289-298, :458-554), energy (Energy.cu:5-19, own tensors)
// The acceleration pass's per-particle stress / rho^2: the buffer of 8 floats
// per padded slot holds a float4 array (xx, yy, zz, xy) followed by a float2
// array (yz, xz).  Separate arrays, 16 and 8 bytes per particle, put more
// particles in each cache line than one 32-byte record: a warp's gather of
// its neighbours' stress touches about a quarter fewer L1 lines.
template <class F4, class F2, class T>
__device__ __forceinline__ void sigr32_split(T* base, int64_t npad, F4*& a, F2*& b) {
  a = reinterpret_cast<F4*>(base);
  b = reinterpret_cast<F2*>(base + 4 * npad);
}

// neighbours gathered per batch in the stress pass (position and velocity)
constexpr int kStressBatch = 4;
// hardening slope over 3G above which the warm-start network is asked: the
// radial start's relative overshoot must exceed the network's error (~1e-2)
constexpr float kMlpSteep = 0.02f;

// The rate-tensor pair loop of the stress pass (CalcRateTensors,
// InteractionAlt.cu:262-383, in FP32) over the neighbour list L (slots into
// the global arrays gp, gv, or ranks into the tile's halo in shared memory).
// acc = D xx yy zz xy yz xz, W xy yz xz, with the off-diagonal sums doubled
// (halved by the caller).  The off-diagonal terms of a pair are a + b (D) and
// a - b (W) of two products a = s_k x_l, b = s_l x_k: their two sums are
// accumulated (one FMA each) and combined once after the loop.
template <class L>
__device__ __forceinline__ void stress_pairs(const StepParams& P, const Fields& F,
                                             const float4* __restrict__ gp,
                                             const float4* __restrict__ gv, const L& list, int c,
                                             float4 pi, float4 vi, float* acc) {
  const float invh = P.invhf, C = P.Cf, Ch = P.Chf;
  float Dxx = 0.f, Dyy = 0.f, Dzz = 0.f;
  float Axy = 0.f, Bxy = 0.f, Axz = 0.f, Bxz = 0.f, Ayz = 0.f, Byz = 0.f;
  int nx[8];
  if (c > 0) list.block(0, nx);
  for (int b = 0; WF_NB_BLK * b < c; b++) {
    int js[8];
#pragma unroll
    for (int q = 0; q < 8; q++) js[q] = nx[q];
    const int m = c - WF_NB_BLK * b;
    if (P.nb_pf && m > P.nb_pf * WF_NB_BLK) list.prefetch(b + P.nb_pf, 1);
    if (m > WF_NB_BLK) list.block(b + 1, nx);
#pragma unroll
    for (int h = 0; h < WF_NB_BLK; h += kStressBatch) {
      float4 pj[kStressBatch], vj[kStressBatch];
#pragma unroll
      for (int q = 0; q < kStressBatch; q++) {
        pj[q] = gp[js[h + q]];
        vj[q] = gv[js[h + q]];
      }
#pragma unroll
      for (int q = 0; q < kStressBatch; q++) {
        // Entries past the count are the particle's own slot (list padding):
        // r^2 = 0 gives GK = 0 exactly (gk32_r2), so they add exact zeros and
        // need no test, except under the contact filter.
        if (P.contact && h + q >= m) continue;
        if constexpr (L::kSlots) {
          if (P.contact && !pass_j(P, F.id[js[h + q]])) continue;
        }
        const float xx = pi.x - pj[q].x, xy = pi.y - pj[q].y, xz = pi.z - pj[q].z;
        // w = 2 s of the reference's s = -GK m_j / (2 rho_j); the off-diagonal
        // sums carry the factor 2 and are halved after the loop
        const float w = -gk32_r2(xx * xx + xy * xy + xz * xz, invh, Ch, C) *
                        __fdividef(pj[q].w, vj[q].w);
        const float sa = (vi.x - vj[q].x) * w, sb = (vi.y - vj[q].y) * w,
                    sc = (vi.z - vj[q].z) * w;
        Dxx += sa * xx;
        Dyy += sb * xy;
        Dzz += sc * xz;
        Axy += sa * xy;
        Bxy += sb * xx;
        Axz += sa * xz;
        Bxz += sc * xx;
        Ayz += sb * xz;
        Byz += sc * xy;
      }
    }
  }
  acc[0] = Dxx; acc[1] = Dyy; acc[2] = Dzz;
  acc[3] = Axy + Bxy; acc[4] = Ayz + Byz; acc[5] = Axz + Bxz;
  acc[6] = Axy - Bxy; acc[7] = Ayz - Byz; acc[8] = Bxz - Axz;
}

// Copies the tile's halo records and local lists into shared memory (every
// thread of the block takes part; asynchronous 16-byte copies, then one
// barrier).  Returns the halo size, or -1 when the tile is not staged (the
// block then gathers from global memory).  n_arr arrays: dst[a][k] =
// src[a][halo[k]]; the lists go to sl.
__device__ __forceinline__ int stage_halo16(const TileHalo& T, int64_t npad, int tile, int n_arr,
                                            float4* const* dst, const float4* const* src,
                                            uint16_t* sl) {
  const int H = T.cap > 0 ? T.hcnt[tile] : -1;
  if (H < 0 || H > T.cap) return -1;        // uniform over the block
  const int32_t* hs = T.halo + T.hoff[tile];
  for (int k = threadIdx.x; k < H; k += blockDim.x) {
    const int s = hs[k];
    for (int a = 0; a < n_arr; a++) cp_async16(dst[a] + k, src[a] + s);
  }
  stage_lists(T.nbl, npad, tile, sl);
  cp_async_wait_all();
  __syncthreads();
  return H;
}

// The stress pass, with the warm-start network compiled in (kMlp: kernel
// k_stress32_mlp) or without it (k_stress32); both held to 80 registers for
// 6 blocks per SM (786k particles: 0.222 -> 0.213 ms without the network;
// with it, 6 blocks gained nothing while the network took 25 KB of shared
// memory per block, and 0.2335 -> 0.226 ms once it took 17 KB).
template <bool kMlp>
__device__ __forceinline__ void stress32_body(StepParams P, Fields F,
                                                  const float4* __restrict__ v32b,
                                                  float* __restrict__ sigr32,
                                                  const int32_t* __restrict__ nb,
                                                  const int32_t* __restrict__ cnt,
                                                  int* __restrict__ status,
                                                  const uint4* __restrict__ mlp,
                                                  const MlpL1 l1, const TileHalo T,
                                                  const List16 L16) {
  // The MLP runs on the tensor cores (tcgen05) for the block's 128 particles
  // at once: every thread of the block must reach it, so out-of-range and
  // non-solid threads are predicated rather than returned before that point.
  // Dynamic shared memory: the network's region (when it runs), then the
  // tile's halo records (positions, velocities) when the tile is staged.
  extern __shared__ __align__(1024) uint8_t smlp[];
  if constexpr (kMlp) mlp_umma_begin(smlp, mlp);
  float4* sp = reinterpret_cast<float4*>(smlp + (kMlp ? WF_UMMA_SMEM : 0));
  float4* sv = sp + T.cap;
  uint16_t* sl = reinterpret_cast<uint16_t*>(sv + T.cap);
  int staged;
  {
    float4* dst[2] = {sp, sv};
    const float4* src[2] = {F.p32, v32b};
    staged = stage_halo16(T, P.npad, blockIdx.x, 2, dst, src, sl);
  }
  const int64_t i0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const bool valid = i0 < P.n;
  const int64_t i = valid ? i0 : 0;
  const float4 pi = F.p32[i];
  const float4 vi = v32b[i];
  const double rho_new = F.vd[i].w + P.dt * F.drho[i];
  const double p = 0.0 + (P.Cs * P.Cs) * (rho_new - P.rho0);   // FP64: small density change
  if (valid) F.p[i] = p;
  const bool solid = valid && F.perm[i] < P.n_solid;
  if (!kMlp && !solid) return;
  if (P.state_pf && solid) {
    prefetch_l2(F.ss32 + 6 * i); prefetch_l2(F.eps_p + i); prefetch_l2(F.sy + i);
    prefetch_l2(F.pwn + i); prefetch_l2(F.T + i); prefetch_l2(F.eint + i);
  }
  if (P.pf_ahead > 0) {
    const int64_t ia = i0 + P.pf_ahead;     // the slot this thread's successor will take
    if (ia < P.n) {
      prefetch_l2(F.p32 + ia); prefetch_l2(v32b + ia); prefetch_l2(F.vd + ia);
      prefetch_l2(F.drho + ia); prefetch_l2(cnt + ia); prefetch_l2(F.perm + ia);
      for (int b = 0; b < P.wave_pf && b < WF_NB_BLOCKS; b++) nb_prefetch(nb, P.npad, ia, b, 4);
    }
  }
  const int c = solid ? cnt[i] : 0;
  float acc[9];
  const int b16 = L16.base ? L16.base[i0 / WF_TILE] : -1;    // uniform over the block
  if (staged >= 0)
    stress_pairs(P, F, sp, sv, NbListS{sl, (int)threadIdx.x}, c, pi, vi, acc);
  else if (b16 >= 0)
    stress_pairs(P, F, F.p32, v32b, NbList16{L16.off, P.npad, i, b16}, c, pi, vi, acc);
  else
    stress_pairs(P, F, F.p32, v32b, NbList32{nb, P.npad, i}, c, pi, vi, acc);
  float Dxx = acc[0], Dyy = acc[1], Dzz = acc[2], Dxy = acc[3], Dyz = acc[4], Dxz = acc[5];
  float Wxy = acc[6], Wyz = acc[7], Wxz = acc[8];
  Dxy *= 0.5f; Dxz *= 0.5f; Dyz *= 0.5f;
  Wxy *= 0.5f; Wxz *= 0.5f; Wyz *= 0.5f;
  // Jaumann update with the reference's product
  float2* ssp = reinterpret_cast<float2*>(F.ss32 + 6 * i);
  const float2 s01 = ssp[0], s23 = ssp[1], s45 = ssp[2];
  T3f S;
  S.xx = s01.x; S.yy = s01.y; S.zz = s23.x;
  S.xy = S.yx = s23.y; S.yz = S.zy = s45.x; S.xz = S.zx = s45.y;
  T3f W;
  W.xx = W.yy = W.zz = 0.f;
  W.xy = Wxy; W.yz = Wyz; W.xz = Wxz; W.yx = -Wxy; W.zy = -Wyz; W.zx = -Wxz;
  T3f WT;
  WT.xx = WT.yy = WT.zz = 0.f;
  WT.xy = W.yx; WT.xz = W.zx; WT.yx = W.xy; WT.yz = W.zy; WT.zx = W.xz; WT.zy = W.yz;
  const T3f SRT = mul_ref_f(S, WT);
  const T3f RS = mul_ref_f(W, S);
  const float G2 = P.G2f, dt = P.dtf;
  const float tr3 = (1.0f / 3.0f) * (Dxx + Dyy + Dzz);
  T3f Sn;
  Sn.xx = dt * (G2 * (Dxx - tr3) + SRT.xx + RS.xx) + S.xx;
  Sn.yy = dt * (G2 * (Dyy - tr3) + SRT.yy + RS.yy) + S.yy;
  Sn.zz = dt * (G2 * (Dzz - tr3) + SRT.zz + RS.zz) + S.zz;
  Sn.xy = dt * (G2 * Dxy + SRT.xy + RS.xy) + S.xy;
  Sn.yx = dt * (G2 * Dxy + SRT.yx + RS.yx) + S.yx;
  Sn.xz = dt * (G2 * Dxz + SRT.xz + RS.xz) + S.xz;
  Sn.zx = dt * (G2 * Dxz + SRT.zx + RS.zx) + S.zx;
  Sn.yz = dt * (G2 * Dyz + SRT.yz + RS.yz) + S.yz;
  Sn.zy = dt * (G2 * Dyz + SRT.zy + RS.zy) + S.zy;
  const float eff = sqrtf(0.5f * ((Dxx - Dyy) * (Dxx - Dyy) + (Dyy - Dzz) * (Dyy - Dzz) +
                                  (Dzz - Dxx) * (Dzz - Dxx)) +
                          3.0f * (Dxy * Dxy + Dyz * Dyz + Dxz * Dxz));
  const float J2 = 0.5f * (Sn.xx * Sn.xx + 2.0f * Sn.xy * Sn.yx + 2.0f * Sn.xz * Sn.zx +
                           Sn.yy * Sn.yy + 2.0f * Sn.yz * Sn.zy + Sn.zz * Sn.zz);
  const float st = sqrtf(3.0f * J2);
  double eps_p = F.eps_p[i], sy = F.sy[i];
  double dep = 0.0, seq = st;
  float scale = 1.0f;
  const MatParams& M = P.mat;
  // rate and thermal factors of the JC law in FP32 (mixed form)
  float Th = 0.0f, RTf = 1.0f;
  double pwn = F.pwn[i];
  const bool jc_newton = P.return_map == 1 && M.model == WF_JOHNSON_COOK;
  if (jc_newton) {
    Th = ((float)F.T[i] - P.jcTtf) * P.jcinvdTf;
    if (P.clamp_homologous) Th = fminf(fmaxf(Th, 0.0f), 0.999f);
    const float sr = eff == 0.0f ? 1.0e-5f : eff;
    RTf = (1.0f + P.jcCf * __logf(sr * P.jcinveps0f)) * (1.0f - __powf(Th, P.jcmf));
  }
  double ratio = -1.0;
  if constexpr (kMlp) {
    // warm start: sigma_y0 from the cached power (FP32 suffices for the features).
    // The network can only improve on the radial start where that start is
    // poor: it overshoots the increment by about H' / (3G + H'), with the
    // hardening slope H' = n B RT eps_p^(n - 1) = n B RT pwn / eps_p.  Where
    // that is below the network's own prediction error (~1e-2) the radial
    // start is the better one, and Newton needs one iteration from either.
    const float sy0f = ((float)M.A + (float)M.B * (float)fmax(pwn, 0.0)) * RTf;
    const bool steep = !(eps_p > 0.0) || !(pwn > 0.0) ||
                       P.jcnf * P.jcBf * RTf * __fdividef((float)pwn, (float)eps_p) >
                           kMlpSteep * P.G3f;
    const bool want = solid && jc_newton && st > sy0f && steep;
    float f[4] = {0.f, 0.f, 0.f, 0.f};
    if (want) mlp_features(st / sy0f, eps_p, eff, Th, f);
    const float y = mlp_umma_cta(smlp, mlp, f, want, status, l1);
    const float yc = mlp_accept(y);
    if (want && yc > 0.0f) ratio = (double)yc;
    if (!solid) return;
  }
  unsigned n_it = 0u, n_call = 0u, n_mlp = 0u;   // this particle's return-map counters
  bool capped = false;                            // Newton stopped at newton_max_iter
  if (P.return_map == 0) {
    // reference one-shot radial return (Mechanical.cu:503-536)
    if (sy < (double)st) scale = (float)(sy / (double)st);
    if (M.model == WF_HOLLOMON) sy = hollomon_yield(M, eps_p);
    else if (M.model == WF_JOHNSON_COOK) sy = jc_yield_ref(M, eps_p, (double)eff, F.T[i]);
    if ((double)st > sy) {
      dep = ((double)st - sy) / (3.0 * P.G);
      eps_p += dep;
      seq = sy;
      if (M.model == WF_BILINEAR) sy += dep * M.Ep;
    }
  } else if (jc_newton) {
    // consistent return map: FP32 Newton on the increment where the series
    // form holds, else the FP64 residual with the cached power
    int it = 0;
    double sy1;
    float dlf, sy1f;
    const bool inc32 = jc_return_inc32(P, st, RTf, eps_p, pwn, (float)ratio, &dlf, &sy1f, &it);
    if (inc32) {
      dep = (double)dlf;
      sy1 = (double)sy1f;
    } else {
      jc_return_cached(P, (double)st, 3.0 * P.G, eps_p, pwn, (double)RTf, ratio, &dep, &sy1,
                       &it);
    }
    F.pwn[i] = pwn;
    capped = it >= P.newton_max_iter;
    if (dep > 0.0) {
      scale = inc32 ? sy1f / st : (float)(sy1 / (double)st);
      eps_p += dep;
      seq = sy1;
      n_it = (unsigned)it;
      n_call = 1u;
      n_mlp = ratio > 0.0 ? 1u : 0u;
    }
    sy = sy1;
  } else {
    // bilinear / Hollomon consistent return map in FP64
    Hard H;
    H.model = M.model; H.R = 1.0; H.Th = 1.0; H.sy_cur = sy; H.Ep = M.Ep;
    double sy0, dsy0;
    hard_eval(M, H, eps_p, 0.0, &sy0, &dsy0);
    if ((double)st > sy0) {
      const double G3 = 3.0 * P.G;
      int it = 0;
      dep = newton_return(P, H, (double)st, G3, eps_p, sy0, ((double)st - sy0) / G3, &it);
      capped = it >= P.newton_max_iter;
      double sy1, dsy1;
      hard_eval(M, H, eps_p, dep, &sy1, &dsy1);
      scale = (float)(sy1 / (double)st);
      eps_p += dep;
      sy = sy1;
      seq = sy1;
      n_it = (unsigned)it;
      n_call = 1u;
    } else {
      sy = sy0;
    }
  }
  Sn.xx *= scale; Sn.yy *= scale; Sn.zz *= scale;
  Sn.xy *= scale; Sn.yz *= scale; Sn.xz *= scale;
  ssp[0] = make_float2(Sn.xx, Sn.yy);
  ssp[1] = make_float2(Sn.zz, Sn.xy);
  ssp[2] = make_float2(Sn.yz, Sn.xz);
  // stress / rho^2 for the acceleration pass: (xx, yy, zz, xy) in one float4
  // array and (yz, xz) in a float2 array behind it (sigr32_split)
  const float pf = (float)p;
  const float rf = vi.w;
  const float ir2 = 1.0f / (rf * rf);
  float4* sga;
  float2* sgb;
  sigr32_split(sigr32, P.npad, sga, sgb);
  sga[i] = make_float4((Sn.xx - pf) * ir2, (Sn.yy - pf) * ir2, (Sn.zz - pf) * ir2, Sn.xy * ir2);
  sgb[i] = make_float2(Sn.yz * ir2, Sn.xz * ir2);
  F.eps_p[i] = eps_p;
  F.sy[i] = sy;
  F.seq[i] = seq;
  F.dep[i] = dep;
  F.eff[i] = (double)eff;
  // CalcIntEnergy, accumulated in FP64: energy_mode 1 with the particle's own
  // tensors; energy_mode 0 (the reference's, Energy.cu:270-276) with particle
  // 0's for every particle: its S:D goes to *P.e0 and the integration adds
  // m/rho S0:D0 dt to each particle
  const float sd = Sn.xx * Dxx + Sn.yy * Dyy + Sn.zz * Dzz +
                   2.0f * (Sn.xy * Dxy + Sn.yz * Dyz + Sn.xz * Dxz);
  if (P.energy_mode != 0) {
    const float def = __fdividef(pi.w, rf) * sd;
    F.eint[i] += (double)def * P.dt;
  } else if (i == (int64_t)P.inv[0]) {
    *P.e0 = (double)sd;
  }
  warp_count(status, n_it, n_call, n_mlp, capped, eps_p > 1.e-6);
  if (!isfinite(st)) atomicOr(status, WF_STATUS_NAN);
}

__global__ void __launch_bounds__(128, 6) k_stress32_mlp(StepParams P, Fields F,
                                                      const float4* __restrict__ v32b,
                                                      float* __restrict__ sigr32,
                                                      const int32_t* __restrict__ nb,
                                                      const int32_t* __restrict__ cnt,
                                                      int* __restrict__ status,
                                                      const uint4* __restrict__ mlp,
                                                      const MlpL1 l1, const TileHalo T,
                                                      const List16 L16) {
  stress32_body<true>(P, F, v32b, sigr32, nb, cnt, status, mlp, l1, T, L16);
}
__global__ void __launch_bounds__(128, 6) k_stress32(StepParams P, Fields F,
                                                     const float4* __restrict__ v32b,
                                                     float* __restrict__ sigr32,
                                                     const int32_t* __restrict__ nb,
                                                     const int32_t* __restrict__ cnt,
                                                     int* __restrict__ status,
                                                     const TileHalo T, const List16 L16) {
  stress32_body<false>(P, F, v32b, sigr32, nb, cnt, status, nullptr, MlpL1{}, T, L16);
}

// ---- C32: acceleration + Monaghan viscosity (InteractionAlt.cu:18-150) ----
// Lane groups of kAccelLanes (see nb_sub).  Neighbours are gathered per batch
// of kAccelBatch: each carries 56 bytes (position, velocity, stress/rho^2).
// 786k particles: 0.278 ms with one lane per particle, 0.272 ms with two
// (71 registers, 7 blocks per SM), 0.31-0.39 ms with four.  With the L2
// prefetches the fused pass held to 64 registers (8 blocks per SM, no spill)
// runs 0.252 -> 0.245 ms; 6 blocks 0.270, 9 blocks spill.
constexpr int kAccelLanes = 2;
constexpr int kAccelBatch = 2;
static_assert(WF_NB_BLK / kAccelLanes >= kAccelBatch, "batch within the lane's sub-block");

// Neighbour records of the acceleration pass, from global memory (the slot
// arrays) or from the tile's halo in shared memory (indexed by local list).
struct AccelSrc {
  const float4* p;
  const float4* v;
  const float4* sa;
  const float2* sb;
};

template <class L>
__device__ __forceinline__ float4 accel_value(const StepParams& P, const Fields& F,
                                              const float4* __restrict__ v32b,
                                              const float* __restrict__ sigr32,
                                              const int32_t* __restrict__ cnt, int64_t i, int g,
                                              const AccelSrc& src, const L& list) {
  constexpr int W = WF_NB_BLK / kAccelLanes;
  const float4 pi = F.p32[i];
  const float4 vi = v32b[i];
  const int32_t idi = F.id[i];
  const float4* sga;
  const float2* sgb;
  sigr32_split(sigr32, P.npad, sga, sgb);
  const float4 s0 = sga[i];
  const float2 s1 = sgb[i];
  const float invh = P.invhf, C = P.Cf, Ch = P.Chf;
  const float h = P.hf, Cs = P.Csf, alpha = P.alphaf, beta = P.betaf, eps = P.epsf;
  const bool av = alpha != 0.0f || beta != 0.0f;
  float ax = 0.f, ay = 0.f, az = 0.f;
  const int c = cnt[i];
  int nx[W];
  if (c > 0) list.template sub<W>(0, g, nx);
  for (int b = 0; WF_NB_BLK * b < c; b++) {
    int js[W];
#pragma unroll
    for (int q = 0; q < W; q++) js[q] = nx[q];
    const int m = c - WF_NB_BLK * b - g * W;   // entries of this lane's sub-block in the list
    if (P.nb_pf && c > WF_NB_BLK * (b + P.nb_pf)) list.prefetch(b + P.nb_pf, kAccelLanes);
    if (c > WF_NB_BLK * (b + 1)) list.template sub<W>(b + 1, g, nx);
#pragma unroll
    for (int hh = 0; hh < W; hh += kAccelBatch) {
      float4 pj[kAccelBatch], vj[kAccelBatch], t0[kAccelBatch];
      float2 t1[kAccelBatch];
#pragma unroll
      for (int q = 0; q < kAccelBatch; q++) {
        const int j = js[hh + q];
        pj[q] = src.p[j];
        vj[q] = src.v[j];
        t0[q] = src.sa[j];
        t1[q] = src.sb[j];
      }
#pragma unroll
      for (int q = 0; q < kAccelBatch; q++) {
        // Entries past the count are the particle's own slot (list padding):
        // r^2 = 0 gives GK = 0 exactly (gk32_r2), so they add exact zeros and
        // need no test, except under the contact filter.
        if (P.contact && hh + q >= m) continue;
        if constexpr (L::kSlots) {
          if (P.contact && !pass_ij(P, idi, F.id[js[hh + q]])) continue;
        }
        const float xx = pi.x - pj[q].x, xy = pi.y - pj[q].y, xz = pi.z - pj[q].z;
        const float r2 = xx * xx + xy * xy + xz * xz;
        const float GK = gk32_r2(r2, invh, Ch, C) * pj[q].w;
        float PI = 0.f;
        if (av) {
          const float vdx =
              (vi.x - vj[q].x) * xx + (vi.y - vj[q].y) * xy + (vi.z - vj[q].z) * xz;
          if (vdx < 0.f) {
            const float MU = __fdividef(h * vdx, r2 + eps);
            PI = __fdividef(alpha * Cs * MU + beta * MU * MU, 0.5f * (vi.w + vj[q].w));
          }
        }
        const float Txx = s0.x + t0[q].x + PI, Tyy = s0.y + t0[q].y + PI,
                    Tzz = s0.z + t0[q].z + PI;
        const float Txy = s0.w + t0[q].w, Tyz = s1.x + t1[q].x, Txz = s1.y + t1[q].y;
        const float gx = xx * GK, gy = xy * GK, gz = xz * GK;
        ax += Txx * gx + Txy * gy + Txz * gz;
        ay += Txy * gx + Tyy * gy + Tyz * gz;
        az += Txz * gx + Tyz * gy + Tzz * gz;
      }
    }
  }
  if constexpr (kAccelLanes > 1) {
    const unsigned mask = group_mask<kAccelLanes>();
#pragma unroll
    for (int o = 1; o < kAccelLanes; o <<= 1) {
      ax += __shfl_xor_sync(mask, ax, o, kAccelLanes);
      ay += __shfl_xor_sync(mask, ay, o, kAccelLanes);
      az += __shfl_xor_sync(mask, az, o, kAccelLanes);
    }
  }
  return make_float4(ax, ay, az, 0.f);
}

// thread -> (slot, lane within the slot's group)
__device__ __forceinline__ int64_t accel_slot(int& g) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  g = (int)(t & (kAccelLanes - 1));
  return t / kAccelLanes;
}

__global__ void __launch_bounds__(128, 8) k_accel32(StepParams P, Fields F,
                                                 const float4* __restrict__ v32b,
                                                 const float* __restrict__ sigr32,
                                                 float4* __restrict__ a32,
                                                 const int32_t* __restrict__ nb,
                                                 const int32_t* __restrict__ cnt) {
  int g;
  const int64_t i = accel_slot(g);
  if (i >= P.n) return;
  const float4* sga;
  const float2* sgb;
  sigr32_split(sigr32, P.npad, sga, sgb);
  if (P.pf_ahead > 0 && g == 0) {
    const int64_t ia = i + P.pf_ahead;      // the slot this thread's successor will take
    if (ia < P.n) {
      prefetch_l2(F.p32 + ia); prefetch_l2(v32b + ia); prefetch_l2(sga + ia);
      prefetch_l2(sgb + ia); prefetch_l2(cnt + ia); prefetch_l2(F.perm + ia);
      prefetch_l2(F.id + ia);
      for (int b = 0; b < P.wave_pf && b < WF_NB_BLOCKS; b++)
        nb_prefetch(nb, P.npad, ia, b, 2 * kAccelLanes);
    }
  }
  if (F.perm[i] >= P.n_solid) return;
  const AccelSrc src{F.p32, v32b, sga, sgb};
  const float4 af = accel_value(P, F, v32b, sigr32, cnt, i, g, src, NbList32{nb, P.npad, i});
  if (g == 0) a32[i] = af;
}

// The acceleration pass with the integration of the same slot behind it
// (no contact stage in between): one pass instead of two, the integration's
// FP64 work and traffic overlapping the other warps' neighbour gathers.
// Neighbours' positions are read from F.p32 while the new positions go to
// p32n (the two are swapped by the host after the launch); the other mirrors
// written here (v32, th32) are not read by this pass.
__global__ void __launch_bounds__(128, 8) k_accel_int32(StepParams P, Fields F,
                                                     const float4* __restrict__ v32b,
                                                     const float* __restrict__ sigr32,
                                                     const double4* __restrict__ vd2,
                                                     const int32_t* __restrict__ nb,
                                                     const int32_t* __restrict__ cnt,
                                                     float4* __restrict__ p32n, const List16 L16) {
  int g;
  const int64_t i = accel_slot(g);
  if (i >= P.n) return;
  const float4* sga;
  const float2* sgb;
  sigr32_split(sigr32, P.npad, sga, sgb);
  const AccelSrc src{F.p32, v32b, sga, sgb};
  if (P.state_pf && g == 0) {
    prefetch_l2(F.xm + i); prefetch_l2(vd2 + i); prefetch_l2(F.u + i); prefetch_l2(F.T + i);
  }
  if (P.pf_ahead > 0 && g == 0) {
    const int64_t ia = i + P.pf_ahead;      // the slot this thread's successor will take
    if (ia < P.n) {
      prefetch_l2(F.p32 + ia); prefetch_l2(v32b + ia); prefetch_l2(sga + ia);
      prefetch_l2(sgb + ia); prefetch_l2(cnt + ia); prefetch_l2(F.perm + ia);
      prefetch_l2(F.id + ia);
      for (int b = 0; b < P.wave_pf && b < WF_NB_BLOCKS; b++) nb_prefetch(nb, P.npad, ia, b, 2 * kAccelLanes);
    }
  }
  // rigid (non-solid) slots: zero acceleration, moved by their BCs
  float4 af = make_float4(0.f, 0.f, 0.f, 0.f);
  if (F.perm[i] < P.n_solid) {
    const int b16 = L16.base ? L16.base[i / WF_TILE] : -1;   // uniform over the block
    if (b16 >= 0)
      af = accel_value(P, F, v32b, sigr32, cnt, i, g, src, NbList16{L16.off, P.npad, i, b16});
    else
      af = accel_value(P, F, v32b, sigr32, cnt, i, g, src, NbList32{nb, P.npad, i});
  }
  if (g == 0) integrate_mixed_one(P, F, vd2, i, af, p32n);
}

// The same pass for staged tiles: a block of 2 x 128 threads is one tile;
// it copies the halo's positions, velocities and stress / rho^2 records into
// shared memory, then reads the neighbours from there through the local
// lists.  Tiles that are not staged gather from global memory.
__global__ void __launch_bounds__(2 * WF_TILE, 3) k_accel_int32_tiles(
    StepParams P, Fields F, const float4* __restrict__ v32b, const float* __restrict__ sigr32,
    const double4* __restrict__ vd2, const int32_t* __restrict__ nb,
    const int32_t* __restrict__ cnt, float4* __restrict__ p32n, const TileHalo T) {
  static_assert(kAccelLanes == 2, "one tile per block of 2 lanes per slot");
  extern __shared__ __align__(16) uint8_t sac[];
  const float4* sga;
  const float2* sgb;
  sigr32_split(sigr32, P.npad, sga, sgb);
  float4* sp = reinterpret_cast<float4*>(sac);
  float4* sv = sp + T.cap;
  float4* ssa = sv + T.cap;
  float2* ssb = reinterpret_cast<float2*>(ssa + T.cap);
  uint16_t* sl = reinterpret_cast<uint16_t*>(ssb + T.cap);
  int staged = -1;
  {
    const int H = T.cap > 0 ? T.hcnt[blockIdx.x] : -1;
    if (H >= 0 && H <= T.cap) {                 // uniform over the block
      const int32_t* hs = T.halo + T.hoff[blockIdx.x];
      for (int k = threadIdx.x; k < H; k += blockDim.x) {
        const int s = hs[k];
        cp_async16(sp + k, F.p32 + s);
        cp_async16(sv + k, v32b + s);
        cp_async16(ssa + k, sga + s);
        cp_async8(ssb + k, sgb + s);
      }
      stage_lists(T.nbl, P.npad, blockIdx.x, sl);
      cp_async_wait_all();
      __syncthreads();
      staged = H;
    }
  }
  int g;
  const int64_t i = accel_slot(g);
  if (i >= P.n) return;
  float4 af = make_float4(0.f, 0.f, 0.f, 0.f);   // rigid (non-solid) slots: moved by their BCs
  if (F.perm[i] < P.n_solid) {
    if (staged >= 0) {
      const AccelSrc src{sp, sv, ssa, ssb};
      af = accel_value(P, F, v32b, sigr32, cnt, i, g, src, NbListS{sl, (int)(threadIdx.x >> 1)});
    } else {
      const AccelSrc src{F.p32, v32b, sga, sgb};
      af = accel_value(P, F, v32b, sigr32, cnt, i, g, src, NbList32{nb, P.npad, i});
    }
  }
  if (g == 0) integrate_mixed_one(P, F, vd2, i, af, p32n);
}

}  // namespace

static inline int blocks_for(int64_t n, int t) { return (int)((n + t - 1) / t); }

// Slots one resident wave ahead for `kernel` (SMs x resident blocks x threads
// per block / lanes per slot): block b + (resident blocks) starts about when
// block b ends, so the prologue a block prefetches for the slots that far on
// is in L2 when their block starts.  Cached per dynamic shared memory size.
template <class K>
static int64_t wave_slots(K kernel, int threads, size_t smem, int lanes, size_t* c_smem,
                          int64_t* c_val) {
  if (*c_val > 0 && *c_smem == smem) return *c_val;
  int dev = 0, sms = 0, per = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, threads, smem) != cudaSuccess)
    return 0;
  *c_smem = smem;
  *c_val = (int64_t)sms * per * threads / lanes;
  return *c_val;
}

void launch_fp32_density(const StepParams& P, const Fields& F, double4* vd2, float4* v32b,
                         const NbBuffers& N, const List16& L16, cudaStream_t s) {
  static size_t c_smem = 0;
  static int64_t c_val = 0;
  StepParams Q = P;
  Q.pf_ahead = !P.wave_pf ? 0 : (int64_t)(P.wave_dist * (double)wave_slots(
      k_density32, 128, 0, 1, &c_smem, &c_val));
  k_density32<<<blocks_for(P.n, 128), 128, 0, s>>>(Q, F, vd2, v32b, N.nb, N.cnt, L16);
}
void launch_fp32_density_heat(const StepParams& P, const Fields& F, double4* vd2, float4* v32b,
                              const NbBuffers& N, int first, int plastic_heat, const TileHalo& T,
                              const List16& L16, cudaStream_t s) {
  TileHalo Tl = T;
  if (kDensLanes != 1) Tl.cap = 0;
  const size_t smem =
      Tl.cap > 0 ? (2 * sizeof(float4) + sizeof(float2)) * (size_t)Tl.cap + WF_TILE_LIST_BYTES : 0;
  static size_t opted[64] = {};     // per device: dynamic shared memory opted in so far
  opt_in_smem(k_density_heat32, smem, opted);
  static size_t c_smem = 0;
  static int64_t c_val = 0;
  StepParams Q = P;
  Q.pf_ahead = !P.wave_pf ? 0 : (int64_t)(P.wave_dist * (double)wave_slots(
      k_density_heat32, 128, smem, kDensLanes, &c_smem, &c_val));
  k_density_heat32<<<blocks_for(P.n * kDensLanes, 128), 128, smem, s>>>(
      Q, F, vd2, v32b, N.nb, N.cnt, first, plastic_heat, Tl, L16);
}
void launch_fp32_heat(const StepParams& P, const Fields& F, const NbBuffers& N, int plastic_heat,
                      cudaStream_t s) {
  static size_t c_smem = 0;
  static int64_t c_val = 0;
  StepParams Q = P;
  Q.pf_ahead = !P.wave_pf ? 0 : (int64_t)(P.wave_dist * (double)wave_slots(
      k_heat32, 128, 0, 1, &c_smem, &c_val));
  k_heat32<<<blocks_for(P.n, 128), 128, 0, s>>>(Q, F, N.nb, N.cnt, plastic_heat);
}
void launch_fp32_stress(const StepParams& P, const Fields& F, const float4* v32b, float* sigr32,
                        const NbBuffers& N, int* status, const void* mlp_packed,
                        const MlpL1* mlp_l1, const TileHalo& T, const List16& L16,
                        cudaStream_t s) {
  const uint4* W = reinterpret_cast<const uint4*>(mlp_packed);
  const MlpL1 l1 = (W && mlp_l1) ? *mlp_l1 : MlpL1{};
  const size_t smem = (W ? WF_UMMA_SMEM : 0) +
                      (T.cap > 0 ? 2 * sizeof(float4) * (size_t)T.cap + WF_TILE_LIST_BYTES : 0);
  static size_t opted[2][64] = {};  // per variant and device: dynamic shared memory opted in
  static size_t c_smem[2] = {0, 0};
  static int64_t c_val[2] = {0, 0};
  StepParams Q = P;
  if (W) {
    opt_in_smem(k_stress32_mlp, smem, opted[1]);
    Q.pf_ahead = !P.wave_pf ? 0 : (int64_t)(P.wave_dist * (double)wave_slots(
        k_stress32_mlp, 128, smem, 1, &c_smem[1], &c_val[1]));
    k_stress32_mlp<<<blocks_for(P.n, 128), 128, smem, s>>>(Q, F, v32b, sigr32, N.nb, N.cnt,
                                                           status, W, l1, T, L16);
  } else {
    opt_in_smem(k_stress32, smem, opted[0]);
    Q.pf_ahead = !P.wave_pf ? 0 : (int64_t)(P.wave_dist * (double)wave_slots(
        k_stress32, 128, smem, 1, &c_smem[0], &c_val[0]));
    k_stress32<<<blocks_for(P.n, 128), 128, smem, s>>>(Q, F, v32b, sigr32, N.nb, N.cnt, status,
                                                       T, L16);
  }
}
void launch_fp32_accel(const StepParams& P, const Fields& F, const float4* v32b,
                       const float* sigr32, float4* a32, const NbBuffers& N, cudaStream_t s) {
  static size_t c_smem = 0;
  static int64_t c_val = 0;
  StepParams Q = P;
  Q.pf_ahead = !P.wave_pf ? 0 : (int64_t)(P.wave_dist * (double)wave_slots(
      k_accel32, 128, 0, kAccelLanes, &c_smem, &c_val));
  k_accel32<<<blocks_for(P.n * kAccelLanes, 128), 128, 0, s>>>(Q, F, v32b, sigr32, a32, N.nb, N.cnt);
}
void launch_fp32_accel_integrate(const StepParams& P, const Fields& F, const float4* v32b,
                                 const float* sigr32, const double4* vd2, const NbBuffers& N,
                                 const TileHalo& T, const List16& L16, cudaStream_t s) {
  if (T.cap > 0) {
    const size_t smem = (3 * sizeof(float4) + sizeof(float2)) * (size_t)T.cap + WF_TILE_LIST_BYTES;
    static size_t opted[64] = {};
    opt_in_smem(k_accel_int32_tiles, smem, opted);
    k_accel_int32_tiles<<<blocks_for(P.n * kAccelLanes, 2 * WF_TILE), 2 * WF_TILE, smem, s>>>(
        P, F, v32b, sigr32, vd2, N.nb, N.cnt, F.p32n, T);
    return;
  }
  static size_t c_smem = 0;
  static int64_t c_val = 0;
  StepParams Q = P;
  Q.pf_ahead = !P.wave_pf ? 0 : (int64_t)(P.wave_dist * (double)wave_slots(
      k_accel_int32, 128, 0, kAccelLanes, &c_smem, &c_val));
  k_accel_int32<<<blocks_for(P.n * kAccelLanes, 128), 128, 0, s>>>(Q, F, v32b, sigr32, vd2, N.nb,
                                                                   N.cnt, F.p32n, L16);
}
