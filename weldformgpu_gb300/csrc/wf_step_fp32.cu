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
#include "wf_mlp.cuh"
#include "wf_tensor.cuh"

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

// cubic-spline gradient factor GK (Functions.cu:82-88) with invh = 1/h,
// Ch = C/h; the q < 1 branch is C/(q h) * q (-3 + 9/4 q) without the division.
__device__ __forceinline__ float gk32(float r, float invh, float Ch, float C) {
  const float q = r * invh;
  if (q < 1.0f) return Ch * (-3.0f + 2.25f * q);
  if (q < 2.0f) return __fdividef(C, r) * (-0.75f * (2.0f - q) * (2.0f - q));
  return 0.0f;
}

// ---- A32: density rate + update (InteractionAlt.cu:166-246, Mechanical.cu:198) --
__global__ void __launch_bounds__(128) k_density32(StepParams P, Fields F,
                                                   double4* __restrict__ vd2,
                                                   float4* __restrict__ v32b,
                                                   const int32_t* __restrict__ nb,
                                                   const int32_t* __restrict__ cnt) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= P.n) return;
  const float4 pi = F.p32[i];
  const float4 vi = F.v32[i];
  const double4 vdi = F.vd[i];
  double rho_new = vdi.w;
  if (F.perm[i] < P.n_solid) {
    const float invh = P.invhf, C = P.Cf, Ch = P.Chf;
    const int32_t idi = F.id[i];
    float drho = 0.0f;
    const int c = cnt[i];
    for (int k = 0; k < c; k++) {
      const int j = __ldg(nb + (int64_t)k * P.npad + i);
      if (P.contact && !pass_ij(P, idi, F.id[j])) continue;
      const float4 pj = F.p32[j];
      const float4 vj = F.v32[j];
      const float xx = pi.x - pj.x, xy = pi.y - pj.y, xz = pi.z - pj.z;
      const float r = sqrtf(xx * xx + xy * xy + xz * xz);
      const float GK = gk32(r, invh, Ch, C);
      const float vx = vi.x - vj.x, vy = vi.y - vj.y, vz = vi.z - vj.z;
      drho += pj.w * __fdividef(vi.w, vj.w) * ((vx * xx + vy * xy + vz * xz) * GK);
    }
    F.drho[i] = (double)drho;
    rho_new = vdi.w + P.dt * (double)drho;
  }
  vd2[i] = make_double4(vdi.x, vdi.y, vdi.z, rho_new);
  v32b[i] = make_float4(vi.x, vi.y, vi.z, (float)rho_new);
}

// ---- B32: rate tensors + EOS + stress (InteractionAlt.cu:262-383,
//      Mechanical.cu:289-298, :458-554), energy (Energy.cu:5-19, own tensors)
__global__ void __launch_bounds__(128) k_stress32(StepParams P, Fields F,
                                                  const float4* __restrict__ v32b,
                                                  float* __restrict__ sigr32,
                                                  const int32_t* __restrict__ nb,
                                                  const int32_t* __restrict__ cnt,
                                                  int* __restrict__ status,
                                                  const MlpPacked* __restrict__ mlp) {
  // The MLP runs on tensor cores with warp-collective mma.sync: every lane of
  // a warp must reach it, so out-of-range and non-solid lanes are predicated
  // rather than returned before that point.
  extern __shared__ uint32_t smlp[];
  const MlpPacked& Wm = *reinterpret_cast<const MlpPacked*>(smlp);
  if (mlp) {
    for (int k = threadIdx.x; k < WF_MLP_PACKED_WORDS; k += blockDim.x)
      smlp[k] = reinterpret_cast<const uint32_t*>(mlp)[k];
    __syncthreads();
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
  if (!mlp && !solid) return;
  const float invh = P.invhf, C = P.Cf, Ch = P.Chf;
  float Dxx = 0.f, Dyy = 0.f, Dzz = 0.f, Dxy = 0.f, Dyz = 0.f, Dxz = 0.f;
  float Wxy = 0.f, Wyz = 0.f, Wxz = 0.f;
  const int c = solid ? cnt[i] : 0;
  for (int k = 0; k < c; k++) {
    const int j = __ldg(nb + (int64_t)k * P.npad + i);
    if (P.contact && !pass_j(P, F.id[j])) continue;
    const float4 pj = F.p32[j];
    const float4 vj = v32b[j];
    const float xx = pi.x - pj.x, xy = pi.y - pj.y, xz = pi.z - pj.z;
    const float r = sqrtf(xx * xx + xy * xy + xz * xz);
    const float s = -0.5f * gk32(r, invh, Ch, C) * __fdividef(pj.w, vj.w);
    const float ax = vi.x - vj.x, ay = vi.y - vj.y, az = vi.z - vj.z;
    Dxx += 2.0f * ax * xx * s;
    Dyy += 2.0f * ay * xy * s;
    Dzz += 2.0f * az * xz * s;
    Dxy += (ax * xy + ay * xx) * s;
    Dxz += (ax * xz + az * xx) * s;
    Dyz += (ay * xz + az * xy) * s;
    Wxy += (ax * xy - ay * xx) * s;
    Wxz -= (ax * xz - az * xx) * s;
    Wyz += (ay * xz - az * xy) * s;
  }
  // Jaumann update with the reference's product
  float* ssp = F.ss32 + 6 * i;
  T3f S;
  S.xx = ssp[0]; S.yy = ssp[1]; S.zz = ssp[2];
  S.xy = S.yx = ssp[3]; S.yz = S.zy = ssp[4]; S.xz = S.zx = ssp[5];
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
    Th = (float)(F.T[i] - M.Tt) * (float)(1.0 / (M.Tm - M.Tt));
    if (P.clamp_homologous) Th = fminf(fmaxf(Th, 0.0f), 0.999f);
    const float sr = eff == 0.0f ? 1.0e-5f : eff;
    RTf = (1.0f + (float)M.C * __logf(sr * (float)(1.0 / M.eps0))) *
          (1.0f - __powf(Th, (float)M.m));
  }
  double ratio = -1.0;
  if (mlp) {
    // warm start: sigma_y0 from the cached power (FP32 suffices for the features)
    const float sy0f = ((float)M.A + (float)M.B * (float)fmax(pwn, 0.0)) * RTf;
    const bool want = solid && jc_newton && st > sy0f;
    float f[4] = {0.f, 0.f, 0.f, 0.f};
    if (want) mlp_features(st / sy0f, eps_p, eff, Th, f);
    __syncwarp();
    const float y = mlp_tc_warp(Wm, f, want);
    const float yc = mlp_accept(y);
    if (want && yc > 0.0f) ratio = (double)yc;
    if (!solid) return;
  }
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
    // consistent return map: the yield function and its Newton residual in
    // FP64 with the cached power
    int it = 0;
    double sy1;
    jc_return_cached(P, (double)st, 3.0 * P.G, eps_p, pwn, (double)RTf, ratio, &dep, &sy1, &it);
    F.pwn[i] = pwn;
    if (dep > 0.0) {
      scale = (float)(sy1 / (double)st);
      eps_p += dep;
      seq = sy1;
      atomicAdd((unsigned long long*)(status + 2), (unsigned long long)it);
      atomicAdd((unsigned long long*)(status + 4), 1ull);
      if (ratio > 0.0) atomicAdd((unsigned long long*)(status + 6), 1ull);
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
      double sy1, dsy1;
      hard_eval(M, H, eps_p, dep, &sy1, &dsy1);
      scale = (float)(sy1 / (double)st);
      eps_p += dep;
      sy = sy1;
      seq = sy1;
      atomicAdd((unsigned long long*)(status + 2), (unsigned long long)it);
      atomicAdd((unsigned long long*)(status + 4), 1ull);
    } else {
      sy = sy0;
    }
  }
  Sn.xx *= scale; Sn.yy *= scale; Sn.zz *= scale;
  Sn.xy *= scale; Sn.yz *= scale; Sn.xz *= scale;
  ssp[0] = Sn.xx; ssp[1] = Sn.yy; ssp[2] = Sn.zz; ssp[3] = Sn.xy; ssp[4] = Sn.yz; ssp[5] = Sn.xz;
  // stress / rho^2 for the acceleration pass: two float4 per particle
  const float pf = (float)p;
  const float rf = vi.w;
  const float ir2 = 1.0f / (rf * rf);
  float4* sg = reinterpret_cast<float4*>(sigr32 + 8 * i);
  sg[0] = make_float4((Sn.xx - pf) * ir2, (Sn.yy - pf) * ir2, (Sn.zz - pf) * ir2, Sn.xy * ir2);
  sg[1] = make_float4(Sn.yz * ir2, Sn.xz * ir2, 0.f, 0.f);
  F.eps_p[i] = eps_p;
  F.sy[i] = sy;
  F.seq[i] = seq;
  F.dep[i] = dep;
  F.eff[i] = (double)eff;
  // CalcIntEnergy with the particle's own tensors, accumulated in FP64
  const float def = __fdividef(pi.w, rf) *
                    (Sn.xx * Dxx + Sn.yy * Dyy + Sn.zz * Dzz +
                     2.0f * (Sn.xy * Dxy + Sn.yz * Dyz + Sn.xz * Dxz));
  F.eint[i] += (double)def * P.dt;
  if (eps_p > 1.e-6) status[1] = 1;
  if (!isfinite(st)) atomicOr(status, WF_STATUS_NAN);
}

// ---- C32: acceleration + Monaghan viscosity (InteractionAlt.cu:18-150) ----
__global__ void __launch_bounds__(128) k_accel32(StepParams P, Fields F,
                                                 const float4* __restrict__ v32b,
                                                 const float* __restrict__ sigr32,
                                                 float4* __restrict__ a32,
                                                 const int32_t* __restrict__ nb,
                                                 const int32_t* __restrict__ cnt) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= P.n) return;
  if (F.perm[i] >= P.n_solid) return;
  const float4 pi = F.p32[i];
  const float4 vi = v32b[i];
  const int32_t idi = F.id[i];
  const float4* si = reinterpret_cast<const float4*>(sigr32 + 8 * i);
  const float4 s0 = si[0], s1 = si[1];
  const float invh = P.invhf, C = P.Cf, Ch = P.Chf;
  const float h = P.hf, Cs = P.Csf, alpha = P.alphaf, beta = P.betaf, eps = P.epsf;
  const bool av = alpha != 0.0f || beta != 0.0f;
  float ax = 0.f, ay = 0.f, az = 0.f;
  const int c = cnt[i];
  for (int k = 0; k < c; k++) {
    const int j = __ldg(nb + (int64_t)k * P.npad + i);
    if (P.contact && !pass_ij(P, idi, F.id[j])) continue;
    const float4 pj = F.p32[j];
    const float4 vj = v32b[j];
    const float4* sjp = reinterpret_cast<const float4*>(sigr32 + 8 * (int64_t)j);
    const float4 t0 = sjp[0], t1 = sjp[1];
    const float xx = pi.x - pj.x, xy = pi.y - pj.y, xz = pi.z - pj.z;
    const float r2 = xx * xx + xy * xy + xz * xz;
    const float r = sqrtf(r2);
    const float GK = gk32(r, invh, Ch, C) * pj.w;
    float PI = 0.f;
    if (av) {
      const float vdx = (vi.x - vj.x) * xx + (vi.y - vj.y) * xy + (vi.z - vj.z) * xz;
      if (vdx < 0.f) {
        const float MU = h * vdx / (r2 + eps);
        PI = (alpha * Cs * MU + beta * MU * MU) / (0.5f * (vi.w + vj.w));
      }
    }
    const float Txx = s0.x + t0.x + PI, Tyy = s0.y + t0.y + PI, Tzz = s0.z + t0.z + PI;
    const float Txy = s0.w + t0.w, Tyz = s1.x + t1.x, Txz = s1.y + t1.y;
    const float gx = xx * GK, gy = xy * GK, gz = xz * GK;
    ax += Txx * gx + Txy * gy + Txz * gz;
    ay += Txy * gx + Tyy * gy + Tyz * gz;
    az += Txz * gx + Tyz * gy + Tzz * gz;
  }
  a32[i] = make_float4(ax, ay, az, 0.f);
}

}  // namespace

static inline int blocks_for(int64_t n, int t) { return (int)((n + t - 1) / t); }

void launch_fp32_density(const StepParams& P, const Fields& F, double4* vd2, float4* v32b,
                         const NbBuffers& N, cudaStream_t s) {
  k_density32<<<blocks_for(P.n, 128), 128, 0, s>>>(P, F, vd2, v32b, N.nb, N.cnt);
}
void launch_fp32_stress(const StepParams& P, const Fields& F, const float4* v32b, float* sigr32,
                        const NbBuffers& N, int* status, const void* mlp_packed, cudaStream_t s) {
  const MlpPacked* W = reinterpret_cast<const MlpPacked*>(mlp_packed);
  size_t smem = W ? sizeof(MlpPacked) : 0;
  k_stress32<<<blocks_for(P.n, 128), 128, smem, s>>>(P, F, v32b, sigr32, N.nb, N.cnt, status, W);
}
void launch_fp32_accel(const StepParams& P, const Fields& F, const float4* v32b,
                       const float* sigr32, float4* a32, const NbBuffers& N, cudaStream_t s) {
  k_accel32<<<blocks_for(P.n, 128), 128, 0, s>>>(P, F, v32b, sigr32, a32, N.nb, N.cnt);
}
