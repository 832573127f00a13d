// wf_integrate.cu — per-particle integration and heat conduction kernels.
//
// Compiled with -fmad=false: the FP64 leapfrog, position and temperature
// updates round exactly like the reference (--fmad=false).
#include "wf_common.cuh"
#include "wf_heat.cuh"
#include "wf_integrate.cuh"

namespace {

// ---- D: BC, UpdatePosFraser, UpdateVel, BC, CalcIntEnergy ---------------
// GeneralAfter/ApplyBCVel (src/WeldFormGPU.cu:103-106, src/cuda/Mechanical.cu:572-584),
// UpdatePosFraser (:179-187), UpdateVel (:142-148), CalcIntEnergy
// (src/cuda/Energy.cu:5-19), in SolverFraser.cu:273-287 order.
__global__ void __launch_bounds__(256) k_integrate(StepParams P, Fields F,
                                                   const double4* __restrict__ vd2,
                                                   const float4* __restrict__ a32) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= P.n) return;
  if (a32) {
    // rigid (non-solid) slots keep the acceleration the BCs left (zero)
    const float4 af = F.perm[i] < P.n_solid ? a32[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    integrate_mixed_one(P, F, vd2, i, af, F.p32);
    return;
  }
  double4 xm = F.xm[i];
  const double4 v4 = vd2[i];
  const double4 a4 = F.a[i];
  const int32_t id = F.id[i];
  double vx = v4.x, vy = v4.y, vz = v4.z, ax = a4.x, ay = a4.y, az = a4.z;
  record_bc_force(P, i, id, xm.w, ax, ay, az);
  apply_bc(P, id, vx, vy, vz, ax, ay, az);
  const double dt = P.dt;
  const double ux = vx * dt + ((ax * 0.5) * dt) * dt;
  const double uy = vy * dt + ((ay * 0.5) * dt) * dt;
  const double uz = vz * dt + ((az * 0.5) * dt) * dt;
  xm.x = xm.x + ux; xm.y = xm.y + uy; xm.z = xm.z + uz;
  double4 u = F.u[i];
  u.x = u.x + ux; u.y = u.y + uy; u.z = u.z + uz;
  vx = vx + ax * dt; vy = vy + ay * dt; vz = vz + az * dt;
  apply_bc(P, id, vx, vy, vz, ax, ay, az);
  // energy_mode 0 reads particle 0's tensors for every particle, like the
  // reference; mode 1 uses each particle's own.
  const bool own = P.energy_mode != 0;
  if (!own || F.perm[i] < P.n_solid) {
    const double* ss = F.ss6 + 6 * (own ? i : (int64_t)P.inv[0]);
    const double* sr = F.sr6 + 6 * (own ? i : (int64_t)P.inv[0]);
    const double de = xm.w / v4.w *
                      (ss[0] * sr[0] + ss[1] * sr[1] + ss[2] * sr[2] +
                       2.0 * (ss[3] * sr[3] + ss[4] * sr[4] + ss[5] * sr[5]));
    F.eint[i] += de * dt;
  }
  F.xm[i] = xm;
  F.vd[i] = make_double4(vx, vy, vz, v4.w);
  F.u[i] = u;
  F.a[i] = make_double4(ax, ay, az, 0.0);
}

// ---- heat: ThermalSolveKernel + plastic heat + CalcConvHeatKernel -------
// src/cuda/Thermal.cu:101-142 and :36-64, FP64 form: the reference's
// arithmetic in its order.  The mixed form's heat pass is k_heat32
// (wf_step_fp32.cu): pair flux in FP32 with the temperature difference taken
// from the (hi, lo) float pair; dT/dt and T stay FP64.
__global__ void __launch_bounds__(128) k_heat_rate(StepParams P, Fields F,
                                                   const int32_t* __restrict__ nb,
                                                   const int32_t* __restrict__ cnt,
                                                   int plastic_heat) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= P.n) return;
  const double4 xi = F.xm[i];
  const double rhoi = F.vd[i].w;
  const double Ti = F.T[i], ki = F.kT[i];
  const int c = cnt[i];
  double s = 0.0;
  for (int k = 0; k < c; k++) {
    const int j = __ldg(nb + nb_at(P.npad, i, k));
    const double4 xj = F.xm[j];
    const double rhoj = F.vd[j].w;
    const double kj = F.kT[j];
    const double xx = xi.x - xj.x, xy = xi.y - xj.y, xz = xi.z - xj.z;
    const double nxij = sqrt(xx * xx + xy * xy + xz * xz);
    const double GK = gradK64(nxij / P.h, P.h, P.gkC);
    s += xj.w / rhoj * (4.0 * ki * kj / (ki + kj) * (Ti - F.T[j])) *
         (xx * (xx * GK) + xy * (xy * GK) + xz * (xz * GK)) / (nxij * nxij);
  }
  s *= 1. / (rhoi * F.cpT[i]);
  if (plastic_heat && F.perm[i] < P.n_solid) {
    const double dep = F.dep[i];
    if (dep > 0.0) s += P.chi * F.sy[i] * dep / (rhoi * F.cpT[i] * P.dt);
  }
  if (F.qf && F.qf[i] > 0.0) s += F.qf[i] / (xi.w * F.cpT[i]);   // frictional heat, law 1
  if (F.bct[i] == 1) {
    const double dS2 = pow(xi.w / rhoi, 0.666666666);
    const double q_conv = P.h_conv * dS2 * (P.T_inf - Ti) / xi.w;
    s += 1. / F.cpT[i] * q_conv;
  }
  F.dTdt[i] = s;
}

// TempCalcLeapfrogFirst / TempCalcLeapfrog (src/cuda/Thermal.cu:16-31)
__global__ void __launch_bounds__(256) k_heat_leapfrog(StepParams P, Fields F, int first,
                                                       int mixed) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= P.n) return;
  const double T = heat_leapfrog_one(P, F, i, F.dTdt[i], first);
  if (mixed && !first) {
    const float thi = (float)T;
    F.th32[i] = make_float2(thi, (float)(T - (double)thi));
  }
}

}  // namespace

static inline int blocks_for(int64_t n, int t) { return (int)((n + t - 1) / t); }

void launch_integrate(const StepParams& P, const Fields& F, const double4* vd2,
                      const float4* a32, cudaStream_t s) {
  k_integrate<<<blocks_for(P.n, 256), 256, 0, s>>>(P, F, vd2, a32);
}

void launch_thermal(const StepParams& P, const Fields& F, const NbBuffers& N, int first,
                    int plastic_heat, int mixed, cudaStream_t s) {
  if (mixed) launch_fp32_heat(P, F, N, plastic_heat, s);
  else k_heat_rate<<<blocks_for(P.n, 128), 128, 0, s>>>(P, F, N.nb, N.cnt, plastic_heat);
  k_heat_leapfrog<<<blocks_for(P.n, 256), 256, 0, s>>>(P, F, first, mixed);
}
