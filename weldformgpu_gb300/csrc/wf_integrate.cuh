// wf_integrate.cuh — the integration of one slot, shared by the integration
// kernel and the mixed form's fused acceleration + integration pass.
//
// GeneralAfter/ApplyBCVel (src/WeldFormGPU.cu:103-106, src/cuda/Mechanical.cu:572-584),
// UpdatePosFraser (:179-187), UpdateVel (:142-148), in SolverFraser.cu:273-287 order.
// The FP32 operations are explicit round-to-nearest intrinsics, so every
// translation unit rounds them alike whatever its contraction flags.
#pragma once
#include "wf_common.cuh"

// The force m a on a BC-zone particle before its BC zeroes a: the load its
// boundary carries.  Written only when an output row is due this step.
__device__ __forceinline__ void record_bc_force(const StepParams& P, int64_t i, int32_t id,
                                                double m, double ax, double ay, double az) {
  if (!P.fr) return;
  bool in_bc = false;
  for (int b = 0; b < P.nbc; b++) in_bc |= id == P.bc_zone[b];
  if (in_bc) P.fr[i] = make_double4(m * ax, m * ay, m * az, 0.0);
}

__device__ __forceinline__ void apply_bc(const StepParams& P, int32_t id, double& vx, double& vy,
                                         double& vz, double& ax, double& ay, double& az) {
  for (int b = 0; b < P.nbc; b++)
    if (id == P.bc_zone[b]) {
      ax = 0.0; ay = 0.0; az = 0.0;
      vx = P.bc_v[b][0]; vy = P.bc_v[b][1]; vz = P.bc_v[b][2];
    }
}

// Mixed form: the increments in FP32 (relative error ~1e-7 of the increment),
// added to the FP64 positions, displacements and velocities; then the FP32
// mirrors (positions to p32_out, velocities, temperature pair).  af is the
// acceleration of the step (zero for rigid slots).
__device__ __forceinline__ void integrate_mixed_one(const StepParams& P, const Fields& F,
                                                    const double4* __restrict__ vd2, int64_t i,
                                                    float4 af, float4* __restrict__ p32_out) {
  double4 xm = F.xm[i];
  const double4 v4 = vd2[i];
  const int32_t id = F.id[i];
  double vx = v4.x, vy = v4.y, vz = v4.z, ax = af.x, ay = af.y, az = af.z;
  record_bc_force(P, i, id, xm.w, ax, ay, az);
  apply_bc(P, id, vx, vy, vz, ax, ay, az);
  const float dtf = P.dtf, hdt2 = __fmul_rn(__fmul_rn(0.5f, P.dtf), P.dtf);
  const float fax = (float)ax, fay = (float)ay, faz = (float)az;
  const double ux = (double)__fadd_rn(__fmul_rn((float)vx, dtf), __fmul_rn(fax, hdt2));
  const double uy = (double)__fadd_rn(__fmul_rn((float)vy, dtf), __fmul_rn(fay, hdt2));
  const double uz = (double)__fadd_rn(__fmul_rn((float)vz, dtf), __fmul_rn(faz, hdt2));
  xm.x += ux; xm.y += uy; xm.z += uz;
  double4 u = F.u[i];
  u.x += ux; u.y += uy; u.z += uz;
  vx += (double)__fmul_rn(fax, dtf);
  vy += (double)__fmul_rn(fay, dtf);
  vz += (double)__fmul_rn(faz, dtf);
  apply_bc(P, id, vx, vy, vz, ax, ay, az);
  F.xm[i] = xm;
  F.vd[i] = make_double4(vx, vy, vz, v4.w);
  F.u[i] = u;
  F.a[i] = make_double4(ax, ay, az, 0.0);
  // energy_mode 0: particle 0's S:D of this step (written by the stress pass)
  // for every particle, as k_integrate's FP64 form
  if (P.energy_mode == 0) F.eint[i] += xm.w / v4.w * *P.e0 * P.dt;
  p32_out[i] = make_float4((float)xm.x, (float)xm.y, (float)xm.z, (float)xm.w);
  F.v32[i] = make_float4((float)vx, (float)vy, (float)vz, (float)v4.w);
  const double T = F.T[i];
  const float thi = (float)T;
  F.th32[i] = make_float2(thi, (float)(T - (double)thi));
}
