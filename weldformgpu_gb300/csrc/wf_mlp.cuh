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

__device__ __forceinline__ float mlp_silu(float z) { return z / (1.0f + __expf(-z)); }

__device__ __forceinline__ void mlp_features(float ratio, double eps_p, float eff, float Th,
                                             float f[4]) {
  f[0] = ratio - 1.0f;
  f[1] = (log10f((float)eps_p + 1.0e-6f) + 3.0f) / 3.0f;
  f[2] = (log10f(fmaxf(eff, 1.0e-12f)) - 1.5f) / 3.5f;
  f[3] = Th;
}
