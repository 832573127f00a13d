// wf_step_fp64.cu — plain-FP64 form of the Fraser step (one thread per
// particle, neighbours in search order).
//
// Compiled with -fmad=false, like the reference (--fmad=false,
// src/CMakeLists.txt:29): every multiply and add rounds separately, so with
// the same neighbour order the sums are bit-identical to the CPU oracle.
// Each kernel states the reference kernel(s) it replaces.
#include "wf_common.cuh"
#include "wf_mlp.cuh"
#include "wf_tensor.cuh"

namespace {

// ---- A: Domain_d::CalcDensInc + UpdateDensity ---------------------------
// src/cuda/InteractionAlt.cu:166-246, src/cuda/Mechanical.cu:198-203.
// Writes vd2 = (v, rho + dt*drho): the density the later passes of the step
// read, next to the velocity so one 32-byte load serves both.
__global__ void __launch_bounds__(128) k_density64(StepParams P, Fields F,
                                                   double4* __restrict__ vd2,
                                                   const int32_t* __restrict__ nb,
                                                   const int32_t* __restrict__ cnt) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= P.n) return;
  const double4 xi = F.xm[i];
  const double4 vi = F.vd[i];
  double rho_new = vi.w;
  if (F.perm[i] < P.n_solid) {
    const int32_t idi = F.id[i];
    double drho = 0.0;
    const int c = cnt[i];
    for (int k = 0; k < c; k++) {
      const int j = __ldg(nb + nb_at(P.npad, i, k));
      if (P.contact && !pass_ij(P, idi, F.id[j])) continue;
      const double4 xj = F.xm[j];
      const double4 vj = F.vd[j];
      const double xx = xi.x - xj.x, xy = xi.y - xj.y, xz = xi.z - xj.z;
      const double rij = sqrt(xx * xx + xy * xy + xz * xz);
      const double di = vi.w, dj = vj.w, mj = xj.w;
      const double vx = vi.x - vj.x, vy = vi.y - vj.y, vz = vi.z - vj.z;
      const double GK = gradK64(rij / P.h, P.h, P.gkC);
      const double temp1 = vx * (xx * GK) + vy * (xy * GK) + vz * (xz * GK);
      drho += mj * (di / dj) * temp1;
    }
    F.drho[i] = drho;
    rho_new = vi.w + P.dt * drho;
  }
  vd2[i] = make_double4(vi.x, vi.y, vi.z, rho_new);
}

// ---- B: CalcRateTensors + PressureKernelExt + StressStrainOne -----------
// src/cuda/InteractionAlt.cu:262-383, src/cuda/Mechanical.cu:289-298 and
// :458-554.  The per-particle EOS and stress update need only the particle's
// own rates, so they run in the epilogue of the rate-tensor pair loop.
__global__ void __launch_bounds__(128) k_stress64(StepParams P, Fields F,
                                                  const double4* __restrict__ vd2,
                                                  const int32_t* __restrict__ nb,
                                                  const int32_t* __restrict__ cnt,
                                                  int* __restrict__ status) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= P.n) return;
  const double4 xi = F.xm[i];
  const double4 vi = vd2[i];
  // PressureKernelExt runs over every particle (EOS case 0, P0 = 0)
  const double p = 0.0 + (P.Cs * P.Cs) * (vi.w - P.rho0);
  F.p[i] = p;
  if (F.perm[i] >= P.n_solid) return;

  T3 SRS = t3_zero(), RRS = t3_zero();
  const int c = cnt[i];
  for (int k = 0; k < c; k++) {
    const int j = __ldg(nb + nb_at(P.npad, i, k));
    if (P.contact && !pass_j(P, F.id[j])) continue;
    const double4 xj = F.xm[j];
    const double4 vj = vd2[j];
    const double xx = xi.x - xj.x, xy = xi.y - xj.y, xz = xi.z - xj.z;
    const double rij = sqrt(xx * xx + xy * xy + xz * xz);
    const double dj = vj.w, mj = xj.w;
    const double ax = vi.x - vj.x, ay = vi.y - vj.y, az = vi.z - vj.z;
    const double GK = gradK64(rij / P.h, P.h, P.gkC);
    const double s = (-0.5) * GK;
    const double mj_dj = mj / dj;
    // StrainRate (symmetric) scaled by -GK/2, then by mj/dj
    const double Sxx = (2.0 * ax * xx) * s, Syy = (2.0 * ay * xy) * s, Szz = (2.0 * az * xz) * s;
    const double Sxy = (ax * xy + ay * xx) * s;
    const double Sxz = (ax * xz + az * xx) * s;
    const double Syz = (ay * xz + az * xy) * s;
    SRS.xx += Sxx * mj_dj; SRS.yy += Syy * mj_dj; SRS.zz += Szz * mj_dj;
    SRS.xy += Sxy * mj_dj; SRS.yx += Sxy * mj_dj;
    SRS.xz += Sxz * mj_dj; SRS.zx += Sxz * mj_dj;
    SRS.yz += Syz * mj_dj; SRS.zy += Syz * mj_dj;
    // RotationRate with the reference's xz sign flip (zx left 0), :358-365
    const double Rxy = (ax * xy - ay * xx) * s;
    const double Rxz = (-(ax * xz - az * xx)) * s;
    const double Ryz = (ay * xz - az * xy) * s;
    RRS.xy += Rxy * mj_dj;
    RRS.xz += Rxz * mj_dj;
    RRS.yz += Ryz * mj_dj;
  }
  double* sr = F.sr6 + 6 * i;
  double* rr = F.rr6 + 6 * i;
  sr[0] = SRS.xx; sr[1] = SRS.yy; sr[2] = SRS.zz; sr[3] = SRS.xy; sr[4] = SRS.yz; sr[5] = SRS.xz;
  rr[0] = 0.0; rr[1] = 0.0; rr[2] = 0.0; rr[3] = RRS.xy; rr[4] = RRS.yz; rr[5] = RRS.xz;

  StressIn in;
  in.S = t3_from_sym(F.ss6 + 6 * i);
  in.D = SRS;
  in.Wflat[0] = 0.0; in.Wflat[1] = 0.0; in.Wflat[2] = 0.0;
  in.Wflat[3] = RRS.xy; in.Wflat[4] = RRS.yz; in.Wflat[5] = RRS.xz;
  in.p = p;
  in.G = P.G;
  in.T = F.T[i];
  StressState st;
  st.eps_p = F.eps_p[i];
  st.sy = F.sy[i];
  st.pwn = F.pwn[i];
  StressOut out;
  stress_update_fp64(P, in, st, out);
  F.pwn[i] = st.pwn;
  F.eff[i] = out.eff;
  F.seq[i] = out.seq;
  F.eps_p[i] = st.eps_p;
  F.sy[i] = st.sy;
  F.dep[i] = out.dep;
  double* sg = F.sig6 + 6 * i;
  double* ss = F.ss6 + 6 * i;
  double* ep = F.eps6 + 6 * i;
  t3_store_flat(out.Sig, sg);
  t3_store_flat(out.S, ss);
  // strain += dt * D (the reference accumulates into an uninitialised local)
  ep[0] += SRS.xx * P.dt; ep[1] += SRS.yy * P.dt; ep[2] += SRS.zz * P.dt;
  ep[3] += SRS.xy * P.dt; ep[4] += SRS.yz * P.dt; ep[5] += SRS.xz * P.dt;
  if (P.log_cap > 0 && out.dep > 0.0 && P.mat.model == WF_JOHNSON_COOK && P.return_map == 1) {
    // (state, converged increment) pairs for training the warm-start MLP
    const unsigned long long slot = atomicAdd((unsigned long long*)P.log_count, 1ull);
    if (slot < (unsigned long long)P.log_cap) {
      float f[4];
      mlp_features((float)(out.st / out.sy0), st.eps_p - out.dep, (float)out.eff, (float)out.Th, f);
      P.log_x[slot] = make_float4(f[0], f[1], f[2], f[3]);
      P.log_y[slot] = (float)(out.dep / ((out.st - out.sy0) / (3.0 * P.G)));
    }
  }
  if (!isfinite(out.seq)) atomicOr(status, WF_STATUS_NAN);
  // Newton counters and the is_yielding flag (eps_p > 1e-6), one atomic per warp
  warp_count(status, (unsigned)out.newton_iters, out.newton_iters > 0 ? 1u : 0u, 0u,
             P.return_map == 1 && out.newton_iters >= P.newton_max_iter, st.eps_p > 1.e-6);
}

// ---- C: Domain_d::CalcAccel (src/cuda/InteractionAlt.cu:18-150) ---------
__global__ void __launch_bounds__(128) k_accel64(StepParams P, Fields F,
                                                 const double4* __restrict__ vd2,
                                                 const int32_t* __restrict__ nb,
                                                 const int32_t* __restrict__ cnt) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= P.n) return;
  if (F.perm[i] >= P.n_solid) return;
  const double4 xi = F.xm[i];
  const double4 vi = vd2[i];
  const int32_t idi = F.id[i];
  const double* si = F.sig6 + 6 * i;
  const double Sixx = si[0], Siyy = si[1], Sizz = si[2], Sixy = si[3], Siyz = si[4], Sixz = si[5];
  const double di = vi.w;
  const double ai = 1.0 / (di * di);
  double ax = 0.0, ay = 0.0, az = 0.0;
  const int c = cnt[i];
  for (int k = 0; k < c; k++) {
    const int j = __ldg(nb + nb_at(P.npad, i, k));
    if (P.contact && !pass_ij(P, idi, F.id[j])) continue;
    const double4 xj = F.xm[j];
    const double4 vj = vd2[j];
    const double2* sj2 = reinterpret_cast<const double2*>(F.sig6 + 6 * (int64_t)j);
    const double2 s01 = sj2[0], s23 = sj2[1], s45 = sj2[2];
    const double xx = xi.x - xj.x, xy = xi.y - xj.y, xz = xi.z - xj.z;
    const double rij = sqrt(xx * xx + xy * xy + xz * xz);
    const double dj = vj.w, mj = xj.w;
    const double vx = vi.x - vj.x, vy = vi.y - vj.y, vz = vi.z - vj.z;
    const double GK = gradK64(rij / P.h, P.h, P.gkC);
    double PI = 0.0;
    if (P.alpha != 0.0 || P.beta != 0.0) {
      const double vdx = vx * xx + vy * xy + vz * xz;
      const double MU = P.h * vdx / (rij * rij + 0.01 * P.h * P.h);
      const double Cij = 0.5 * (P.Cs + P.Cs);
      if (vdx < 0) PI = (P.alpha * Cij * MU + P.beta * MU * MU) / (0.5 * (di + dj));
    }
    const double aj = 1.0 / (dj * dj);
    // (Si/di^2 + Sj/dj^2 + PI*I) * mj, then times GK*xij (tensor3.cu:225)
    const double Txx = (Sixx * ai + s01.x * aj) + PI, Tyy = (Siyy * ai + s01.y * aj) + PI;
    const double Tzz = (Sizz * ai + s23.x * aj) + PI;
    const double Txy = Sixy * ai + s23.y * aj;
    const double Tyz = Siyz * ai + s45.x * aj;
    const double Txz = Sixz * ai + s45.y * aj;
    const double gx = xx * GK, gy = xy * GK, gz = xz * GK;
    const double Mxx = Txx * mj, Myy = Tyy * mj, Mzz = Tzz * mj;
    const double Mxy = Txy * mj, Myz = Tyz * mj, Mxz = Txz * mj;
    ax += Mxx * gx + Mxy * gy + Mxz * gz;
    ay += Mxy * gx + Myy * gy + Myz * gz;
    az += Mxz * gx + Myz * gy + Mzz * gz;
  }
  F.a[i] = make_double4(ax, ay, az, 0.0);
}

}  // namespace

static inline int blocks_for(int64_t n, int t) { return (int)((n + t - 1) / t); }

void launch_fp64_density(const StepParams& P, const Fields& F, double4* vd2, const NbBuffers& N,
                         cudaStream_t s) {
  k_density64<<<blocks_for(P.n, 128), 128, 0, s>>>(P, F, vd2, N.nb, N.cnt);
}
void launch_fp64_stress(const StepParams& P, const Fields& F, const double4* vd2,
                        const NbBuffers& N, int* status, cudaStream_t s) {
  k_stress64<<<blocks_for(P.n, 128), 128, 0, s>>>(P, F, vd2, N.nb, N.cnt, status);
}
void launch_fp64_accel(const StepParams& P, const Fields& F, const double4* vd2,
                       const NbBuffers& N, cudaStream_t s) {
  k_accel64<<<blocks_for(P.n, 128), 128, 0, s>>>(P, F, vd2, N.nb, N.cnt);
}
