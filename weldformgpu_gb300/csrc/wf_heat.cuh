// wf_heat.cuh — per-particle parts of the heat step, shared by the standalone
// heat kernels (wf_integrate.cu) and the mixed form's fused density + heat
// pass (wf_step_fp32.cu).
#pragma once
#include "wf_common.cuh"

// dT/dt of the mixed form from the FP32 flux sum sf = sum_j m_j/rho_j
// 4 k_i k_j/(k_i + k_j) (T_i - T_j) GK_ij (ThermalSolveKernel,
// src/cuda/Thermal.cu:101-142), plus the Taylor-Quinney plastic heat and the
// convection of boundary particles (CalcConvHeatKernel, Thermal.cu:36-64).
// The rate needs FP32 accuracy only (T integrates in FP64): no FP64 division
// or pow per particle.
__device__ __forceinline__ double heat_rate_mixed(const StepParams& P, const Fields& F, int64_t i,
                                                  float sf, double rhoi, double mass, double Ti,
                                                  int plastic_heat) {
  const float rf = (float)rhoi, cpf = (float)F.cpT[i];
  float sm = sf / (rf * cpf);
  if (plastic_heat && F.perm[i] < P.n_solid) {
    const double dep = F.dep[i];
    if (dep > 0.0) sm += P.chif * (float)F.sy[i] * (float)dep / (rf * cpf * P.dtf);
  }
  if (F.qf && F.qf[i] > 0.0) sm += (float)F.qf[i] / ((float)mass * cpf);   // frictional heat
  if (F.bct[i] == 1) {
    const float mf = (float)mass;
    const float dS2 = powf(mf / rf, 0.666666666f);
    sm += P.h_convf * dS2 * (P.T_inff - (float)Ti) / (mf * cpf);
  }
  return (double)sm;
}

// TempCalcLeapfrogFirst / TempCalcLeapfrog (src/cuda/Thermal.cu:16-31) for
// one particle; returns the new temperature (unchanged on the first step).
__device__ __forceinline__ double heat_leapfrog_one(const StepParams& P, const Fields& F,
                                                    int64_t i, double dTdt, int first) {
  const double dt = P.dt;
  if (first) {
    F.Ta[i] = F.T[i] - dt / 2.0 * dTdt;
    return F.T[i];
  }
  const double ta = F.Ta[i];
  F.Tb[i] = ta;
  const double ta2 = ta + dTdt * dt;
  F.Ta[i] = ta2;
  const double T = (ta2 + ta) / 2.;
  F.T[i] = T;
  return T;
}
