// wf_mlp.cuh — the small MLP that proposes the starting plastic-multiplier
// increment of the Johnson-Cook return-mapping Newton solve.
//
// Layers 4 -> 64 -> 64 -> 1 with SiLU on the hidden layers.  Parameters are
// packed as W1[64*4], b1[64], W2[64*64], b2[64], W3[64], b3[1] (row-major,
// out x in).  Inputs (features) and the output are dimensionless:
//   f0 = sigma_trial / sigma_y0 - 1
//   f1 = (log10(eps_p + 1e-6) + 3) / 3
//   f2 = (log10(max(strain_rate, 1e-12)) - 1.5) / 3.5
//   f3 = homologous temperature
//   y  = dlambda / dlambda_radial, where dlambda_radial = (sigma_trial - sigma_y0) / 3G
// A prediction outside (0, 1] is ignored and Newton starts from the radial value.
// Inference runs on the 5th-generation tensor cores (tcgen05, mlp_umma_cta)
// for a block's 128 particles at once, inside the stress kernel.
#pragma once
#include <cuda_runtime.h>

#define WF_MLP_IN 4
#define WF_MLP_H 64
#define WF_MLP_NPARAM (WF_MLP_H * WF_MLP_IN + WF_MLP_H + WF_MLP_H * WF_MLP_H + WF_MLP_H + WF_MLP_H + 1)
#define WF_MLP_OFF_W1 0
#define WF_MLP_OFF_B1 (WF_MLP_H * WF_MLP_IN)
#define WF_MLP_OFF_W2 (WF_MLP_OFF_B1 + WF_MLP_H)
#define WF_MLP_OFF_B2 (WF_MLP_OFF_W2 + WF_MLP_H * WF_MLP_H)
#define WF_MLP_OFF_W3 (WF_MLP_OFF_B2 + WF_MLP_H)
#define WF_MLP_OFF_B3 (WF_MLP_OFF_W3 + WF_MLP_H)

#include <cuda_bf16.h>
#include <stdint.h>

// SiLU with the fast reciprocal: for z << 0, 1 + exp(-z) overflows to +inf
// and the quotient is 0 (the limit of z sigmoid(z)); z is finite here.
__device__ __forceinline__ float mlp_silu(float z) { return __fdividef(z, 1.0f + __expf(-z)); }

// The fallback rule: a prediction in (0, 1] is the start; one slightly above
// 1 (up to 1.1) means "at the radial value" and is clamped to 1; anything
// else is rejected (returns 0) and Newton starts from the radial value.
__device__ __forceinline__ float mlp_accept(float y) {
  if (y > 0.0f && y <= 1.0f) return y;
  if (y > 1.0f && y <= 1.1f) return 1.0f;
  return 0.0f;
}

__device__ __forceinline__ uint32_t bf16x2(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t*>(&v);
}

// SiLU(z) = z sigmoid(z) = h (1 + tanh(h)), h = z / 2, with the hardware tanh
// approximation: one MUFU operation per value instead of an exponential and a
// reciprocal (the tensor-core inference is MUFU-bound otherwise).
__device__ __forceinline__ float silu_tanh(float z) {
  const float h = 0.5f * z;
  float t;
  asm("tanh.approx.f32 %0, %1;" : "=f"(t) : "f"(h));
  return fmaf(h, t, h);
}

// Two SiLUs in BF16: tanh.approx.bf16x2 handles both values in one MUFU
// operation.
__device__ __forceinline__ uint32_t silu_bf16x2(float z0, float z1) {
  const uint32_t h = bf16x2(0.5f * z0, 0.5f * z1);
  uint32_t t, r;
  asm("tanh.approx.bf16x2 %0, %1;" : "=r"(t) : "r"(h));
  asm("fma.rn.bf16x2 %0, %1, %2, %3;" : "=r"(r) : "r"(h), "r"(t), "r"(h));
  return r;
}

// ---------------------------------------------------------------------------
// tcgen05 inference: one CTA of 128 threads evaluates the network for its 128
// particles, row m of every matrix being thread m's particle.
//   layer 1: each thread, FP32 on the CUDA cores: h = SiLU(W1 f + b1), written
//            in BF16 as its row of A2 (128 x 64), half a row at a time
//   layer 2: D2 (128 x 64, FP32 in tensor memory) = A2 x B2^T, B2 = W2; four
//            MMAs of K = 16 accumulate in the same 64 columns, two per half
//            of A2 (hidden units 0-31, then 32-63), the halves passing
//            through one 8 KB buffer: 8 KB less shared memory per block
//            (more L1 for the pass's gathers) for one more MMA round trip
//   layer 3: each thread reads its row of D2, adds b2, applies SiLU and
//            takes the dot product with W3 (FP32).
// One thread issues each half's two MMAs and commits them to an mbarrier
// (phase 0, then 1); every thread waits (bounded) before the second half
// overwrites the buffer and before reading its own row with tcgen05.ld.  The 64 tensor-
// memory columns are allocated at kernel entry and freed inside the call.
//
// Dynamic shared memory (bytes): the weight image (copied from the packed
// parameters, k_mlp_pack_umma), then A2, the mbarriers and the tensor-memory
// address.  K-major, no swizzle (wf_umma.cuh).
// ---------------------------------------------------------------------------
#include "wf_common.cuh"
#include "wf_umma.cuh"
#define WF_UMMA_B2 0          // 64 x 64 BF16 (SBO 1024)
#define WF_UMMA_BIAS2 8192    // 64 floats
#define WF_UMMA_W3 8448       // 64 floats
#define WF_UMMA_B3 8704       // 1 float
#define WF_UMMA_IMAGE 8832    // bytes of the packed weight image (a multiple of 128)
#define WF_UMMA_A2 8832       // 128 x 32 BF16, one half of A2 at a time (SBO 512)
#define WF_UMMA_MBAR 17024    // mbarrier of the MMAs, 8 bytes
#define WF_UMMA_TSLOT 17032   // tensor-memory base address, 4 bytes
#define WF_UMMA_MBAR_W 17040  // mbarrier of the weight-image copy, 8 bytes
#define WF_UMMA_SMEM 17152    // dynamic shared memory of a kernel that runs the MLP

// Layer 1 (4 -> 64) runs on the CUDA cores in FP32: its weights travel as a
// kernel parameter, so every multiply-add reads its weight from the constant
// bank.  On the tensor cores it took a K = 16 MMA of its own (4 features, the
// bias column, zeros), a block barrier and a completion round trip.
struct MlpL1 {
  float w[WF_MLP_H][WF_MLP_IN];
  float b[WF_MLP_H];
};

// layer 1 of the packed parameters (W1 row-major out x in, then b1)
inline MlpL1 mlp_l1_from(const float* P) {
  MlpL1 l;
  for (int n = 0; n < WF_MLP_H; n++) {
    for (int k = 0; k < WF_MLP_IN; k++) l.w[n][k] = P[WF_MLP_OFF_W1 + n * WF_MLP_IN + k];
    l.b[n] = P[WF_MLP_OFF_B1 + n];
  }
  return l;
}

// byte offset of BF16 element (r, k) of a K-major operand with K columns
__host__ __device__ __forceinline__ int umma_kmajor_off(int r, int k, int K) {
  return (r >> 3) * (K * 16) + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2;
}

// Kernel entry of every kernel that contains the MLP (all threads of the
// block, before anything else): with the network on (image != nullptr) one
// thread initialises the mbarriers and warp 0 allocates the 64 tensor-memory
// columns; in every case warp 0 gives up the allocation permit so further
// CTAs can start on the SM.  The weight image is copied later, by
// mlp_umma_cta, and only in blocks where some thread wants a prediction.
__device__ __forceinline__ void mlp_umma_begin(uint8_t* sm, const uint4* __restrict__ image) {
  const uint32_t s0 = umma::smem_addr(sm);
  if (image && threadIdx.x == 0) {
    umma::mbar_init(s0 + WF_UMMA_MBAR, 1);
    umma::mbar_init(s0 + WF_UMMA_MBAR_W, 1);
  }
  if (threadIdx.x < 32) {
    if (image) umma::tmem_alloc(s0 + WF_UMMA_TSLOT, 64);
    umma::relinquish_permit();
  }
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
}

// Block-collective, once per kernel after mlp_umma_begin(sm, image != nullptr):
// blockDim.x == 128 and every thread calls it at the same point.  Frees the
// tensor memory.  Returns the network output for the calling thread's row,
// or -1 when no thread of the block wants a prediction or a completion wait
// ran out (then WF_STATUS_MMA_WAIT is set in *status).
static __device__ __forceinline__ float mlp_umma_cta(uint8_t* sm, const uint4* __restrict__ image,
                                                     const float f[4], bool want, int* status,
                                                     const MlpL1& l1) {
  constexpr int kWaitLimit = 1 << 20;
  constexpr uint32_t kId = umma::idesc_bf16_f32(128, 64);
  const int tid = threadIdx.x, warp = tid >> 5;
  const uint32_t tmem = *reinterpret_cast<volatile uint32_t*>(sm + WF_UMMA_TSLOT);
  const uint32_t s0 = umma::smem_addr(sm);
  // No thread of the block wants a prediction: one barrier, and warp 0 frees
  // the tensor memory (no weight copy was started).
  if (!__syncthreads_or(want)) {
    if (warp == 0) umma::tmem_dealloc(tmem, 64);
    return -1.0f;
  }
  // the weight image: one bulk copy into the start of the dynamic shared
  // memory, completing on its mbarrier; every thread waits (bounded)
  if (tid == 0) umma::bulk_load(s0, image, WF_UMMA_IMAGE, s0 + WF_UMMA_MBAR_W);
  const bool image_ok = umma::mbar_wait(s0 + WF_UMMA_MBAR_W, 0, kWaitLimit);
  if (!__syncthreads_and(image_ok)) {
    if (warp == 0) umma::tmem_dealloc(tmem, 64);
    if (tid == 0) atomicOr(status, WF_STATUS_MMA_WAIT);
    return -1.0f;
  }
  const uint32_t mbar = s0 + WF_UMMA_MBAR;
  // layer 1 and its SiLU (BF16 pairs) into this thread's row of A2
  uint4* a2 = reinterpret_cast<uint4*>(sm + WF_UMMA_A2 + umma_kmajor_off(tid, 0, 32));
  bool ok = true;
#pragma unroll
  for (int half = 0; half < 2; half++) {
    if (half == 1) {
      // the first half's MMAs have read the buffer once their commit arrived
      ok = umma::mbar_wait(mbar, 0, kWaitLimit);
      if (!__syncthreads_and(ok)) break;
      umma::fence_after_sync();
    }
#pragma unroll
    for (int cc = 0; cc < 2; cc++) {
      const int c = 2 * half + cc;                      // hidden units 16c .. 16c+15
      uint32_t r[8];
#pragma unroll
      for (int j = 0; j < 8; j++) {
        const int n0 = 16 * c + 2 * j;
        float z0 = l1.b[n0], z1 = l1.b[n0 + 1];
#pragma unroll
        for (int k = 0; k < WF_MLP_IN; k++) {
          z0 = fmaf(l1.w[n0][k], f[k], z0);
          z1 = fmaf(l1.w[n0 + 1][k], f[k], z1);
        }
        r[j] = silu_bf16x2(z0, z1);
      }
      a2[16 * cc] = make_uint4(r[0], r[1], r[2], r[3]);       // columns 16cc .. 16cc+7
      a2[16 * cc + 8] = make_uint4(r[4], r[5], r[6], r[7]);   // columns 16cc+8 .. 16cc+15
    }
    umma::fence_async_smem();
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    if (tid == 0) {
#pragma unroll
      for (int kk = 0; kk < 2; kk++) {
        const int kg = 2 * half + kk;                   // K step of the whole product
        umma::mma_bf16(tmem, umma::smem_desc(s0 + WF_UMMA_A2 + 256 * kk, 128, 512),
                       umma::smem_desc(s0 + WF_UMMA_B2 + 256 * kg, 128, 1024), kId,
                       kg > 0 ? 1u : 0u);
      }
      umma::commit(mbar);
    }
  }
  if (ok) ok = umma::mbar_wait(mbar, 1, kWaitLimit);
  umma::fence_after_sync();
  const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);   // this warp's 32 lanes
  const float* bias2 = reinterpret_cast<const float*>(sm + WF_UMMA_BIAS2);
  const float* w3 = reinterpret_cast<const float*>(sm + WF_UMMA_W3);
  float y = 0.0f;
#pragma unroll
  for (int c = 0; c < 4; c++) {
    float v[16];
    umma::ld16(trow + 16 * c, v);
#pragma unroll
    for (int j = 0; j < 16; j++) y += w3[16 * c + j] * silu_tanh(v[j] + bias2[16 * c + j]);
  }
  umma::fence_before_sync();
  __syncthreads();
  if (warp == 0) umma::tmem_dealloc(tmem, 64);
  if (!ok) {
    if (tid == 0) atomicOr(status, WF_STATUS_MMA_WAIT);
    return -1.0f;
  }
  return y + *reinterpret_cast<const float*>(sm + WF_UMMA_B3);
}

__device__ __forceinline__ void mlp_features(float ratio, double eps_p, float eff, float Th,
                                             float f[4]) {
  f[0] = ratio - 1.0f;
  f[1] = (log10f((float)eps_p + 1.0e-6f) + 3.0f) / 3.0f;
  f[2] = (log10f(fmaxf(eff, 1.0e-12f)) - 1.5f) / 3.5f;
  f[3] = Th;
}
