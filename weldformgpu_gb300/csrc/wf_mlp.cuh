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

// ---------------------------------------------------------------------------
// BF16 tensor-core inference (mma.sync m16n8k16, FP32 accumulation).
//
// One warp evaluates the network for its 32 particles: rows of the A operand
// are particles (two m-tiles of 16), columns are input features.  Layer 1 has
// K = 16 (4 features, a constant 1 that carries the bias b1, zeros); layer 2
// has K = 64 in 4 k-steps; both have N = 64 in 8 n-tiles.  The FP32 layer-1
// accumulator fragments become the BF16 A fragments of layer 2 without data
// movement (for m16n8k16 the C layout of n-tiles 2k, 2k+1 is the A layout of
// k-step k).  Layer 3 (N = 1) is a dot product reduced across each quad.
//
// Fragment layouts (PTX ISA, mma.m16n8k16 with .bf16): lane = 4 g + t;
//   A regs: {A[g][2t..2t+1]}, {A[g+8][2t..]}, {A[g][2t+8..]}, {A[g+8][2t+8..]}
//   B regs: {B[2t..2t+1][g]}, {B[2t+8..2t+9][g]}
//   C/D:    C[g][2t], C[g][2t+1], C[g+8][2t], C[g+8][2t+1]
// ---------------------------------------------------------------------------
struct MlpPacked {
  uint2 b1[8][32];       // layer-1 B fragments per n-tile and lane (W1 | b1)
  uint2 b2[4][8][32];    // layer-2 B fragments per k-step, n-tile and lane
  float bias2[WF_MLP_H];
  float w3[WF_MLP_H];
  float b3;
  float pad[3];
};
#define WF_MLP_PACKED_WORDS ((int)(sizeof(MlpPacked) / 4))

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

// Two SiLUs in BF16 for a pair of layer-1 outputs that become one BF16x2 A
// operand of layer 2 anyway: tanh.approx.bf16x2 handles both values in one
// MUFU operation.
__device__ __forceinline__ uint32_t silu_bf16x2(float z0, float z1) {
  const uint32_t h = bf16x2(0.5f * z0, 0.5f * z1);
  uint32_t t, r;
  asm("tanh.approx.bf16x2 %0, %1;" : "=r"(t) : "r"(h));
  asm("fma.rn.bf16x2 %0, %1, %2, %3;" : "=r"(r) : "r"(h), "r"(t), "r"(h));
  return r;
}

__device__ __forceinline__ void mma_bf16_16816(float c[4], const uint32_t a[4], uint2 b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
      "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b.x), "r"(b.y));
}

// Warp-collective: every lane of the warp must call it, convergent.  Lanes
// with want == false pass dummy features; returns the network output for the
// calling lane's particle, or -1 when no lane of the warp wants a prediction.
__device__ __forceinline__ float mlp_tc_warp(const MlpPacked& W, const float f[4], bool want) {
  const unsigned full = 0xffffffffu;
  if (__ballot_sync(full, want) == 0u) return -1.0f;
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  float out = 0.0f;
#pragma unroll
  for (int mt = 0; mt < 2; mt++) {
    // layer-1 A fragment: feature columns 2t, 2t+1 of particles mt*16+g and mt*16+g+8
    uint32_t a1[4];
#pragma unroll
    for (int half = 0; half < 2; half++) {
      const int src = mt * 16 + g + half * 8;
      const float f0 = __shfl_sync(full, f[0], src), f1 = __shfl_sync(full, f[1], src);
      const float f2 = __shfl_sync(full, f[2], src), f3 = __shfl_sync(full, f[3], src);
      const float c0 = t == 0 ? f0 : (t == 1 ? f2 : (t == 2 ? 1.0f : 0.0f));
      const float c1 = t == 0 ? f1 : (t == 1 ? f3 : 0.0f);
      a1[half] = bf16x2(c0, c1);
    }
    a1[2] = 0u;
    a1[3] = 0u;
    float acc1[8][4];
#pragma unroll
    for (int j = 0; j < 8; j++) {
      acc1[j][0] = acc1[j][1] = acc1[j][2] = acc1[j][3] = 0.0f;
      mma_bf16_16816(acc1[j], a1, W.b1[j][lane]);
    }
    // SiLU, then the accumulators of n-tiles 2k, 2k+1 are the A fragment of k-step k
    uint32_t a2[4][4];
#pragma unroll
    for (int kk = 0; kk < 4; kk++) {
      a2[kk][0] = silu_bf16x2(acc1[2 * kk][0], acc1[2 * kk][1]);
      a2[kk][1] = silu_bf16x2(acc1[2 * kk][2], acc1[2 * kk][3]);
      a2[kk][2] = silu_bf16x2(acc1[2 * kk + 1][0], acc1[2 * kk + 1][1]);
      a2[kk][3] = silu_bf16x2(acc1[2 * kk + 1][2], acc1[2 * kk + 1][3]);
    }
    float y0 = 0.0f, y1 = 0.0f;   // rows g and g+8 of this m-tile
#pragma unroll
    for (int j = 0; j < 8; j++) {
      const int col = 8 * j + 2 * t;
      float acc2[4] = {W.bias2[col], W.bias2[col + 1], W.bias2[col], W.bias2[col + 1]};
#pragma unroll
      for (int kk = 0; kk < 4; kk++) mma_bf16_16816(acc2, a2[kk], W.b2[kk][j][lane]);
      y0 += W.w3[col] * silu_tanh(acc2[0]) + W.w3[col + 1] * silu_tanh(acc2[1]);
      y1 += W.w3[col] * silu_tanh(acc2[2]) + W.w3[col + 1] * silu_tanh(acc2[3]);
    }
    y0 += __shfl_xor_sync(full, y0, 1);
    y0 += __shfl_xor_sync(full, y0, 2);
    y1 += __shfl_xor_sync(full, y1, 1);
    y1 += __shfl_xor_sync(full, y1, 2);
    // particle p = mt*16 + half*8 + r sits in row r (+8 for half 1) of quad r
    const float v0 = __shfl_sync(full, y0, 4 * (lane & 7));
    const float v1 = __shfl_sync(full, y1, 4 * (lane & 7));
    if ((lane >> 4) == mt) out = ((lane >> 3) & 1) ? v1 : v0;
  }
  return out + W.b3;
}

__device__ __forceinline__ void mlp_features(float ratio, double eps_p, float eff, float Th,
                                             float f[4]) {
  f[0] = ratio - 1.0f;
  f[1] = (log10f((float)eps_p + 1.0e-6f) + 3.0f) / 3.0f;
  f[2] = (log10f(fmaxf(eff, 1.0e-12f)) - 1.5f) / 3.5f;
  f[3] = Th;
}
