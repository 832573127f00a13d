// wf_tensor.cuh — 3x3 tensor algebra with the reference's semantics and the
// per-particle stress update (Jaumann rate, J2 return map, hardening).
#pragma once
#include "wf_common.cuh"

struct T3 {
  double xx, xy, xz, yx, yy, yz, zx, zy, zz;
};

__device__ __forceinline__ T3 t3_zero() {
  T3 r;
  r.xx = r.xy = r.xz = r.yx = r.yy = r.yz = r.zx = r.zy = r.zz = 0.0;
  return r;
}
// FromFlatSym (src/cuda/tensor3.cu:62)
__device__ __forceinline__ T3 t3_from_sym(const double* f) {
  T3 r;
  r.xx = f[0]; r.yy = f[1]; r.zz = f[2];
  r.xy = r.yx = f[3];
  r.yz = r.zy = f[4];
  r.xz = r.zx = f[5];
  return r;
}
// FromFlatAntiSym (tensor3.cu:72)
__device__ __forceinline__ T3 t3_from_antisym(const double* f) {
  T3 r;
  r.xx = f[0]; r.yy = f[1]; r.zz = f[2];
  r.xy = f[3]; r.yz = f[4]; r.xz = f[5];
  r.yx = -f[3]; r.zy = -f[4]; r.zx = -f[5];
  return r;
}
// ToFlatSymPtr (tensor3.cu:95): upper triangle only
__device__ __forceinline__ void t3_store_flat(const T3& t, double* f) {
  f[0] = t.xx; f[1] = t.yy; f[2] = t.zz; f[3] = t.xy; f[4] = t.yz; f[5] = t.xz;
}
__device__ __forceinline__ T3 t3_scale(const T3& m, double f) {
  T3 r;
  r.xx = m.xx * f; r.xy = m.xy * f; r.xz = m.xz * f;
  r.yx = m.yx * f; r.yy = m.yy * f; r.yz = m.yz * f;
  r.zx = m.zx * f; r.zy = m.zy * f; r.zz = m.zz * f;
  return r;
}
__device__ __forceinline__ T3 t3_add(const T3& a, const T3& b) {
  T3 r;
  r.xx = a.xx + b.xx; r.xy = a.xy + b.xy; r.xz = a.xz + b.xz;
  r.yx = a.yx + b.yx; r.yy = a.yy + b.yy; r.yz = a.yz + b.yz;
  r.zx = a.zx + b.zx; r.zy = a.zy + b.zy; r.zz = a.zz + b.zz;
  return r;
}
// f * Identity() (tensor3.cu:102,294)
__device__ __forceinline__ T3 t3_ident(double f) {
  T3 r;
  r.xx = r.yy = r.zz = 1.0 * f;
  r.xy = r.xz = r.yx = r.yz = r.zx = r.zy = 0.0 * f;
  return r;
}
__device__ __forceinline__ T3 t3_sub(const T3& a, const T3& b) {
  T3 r;
  r.xx = a.xx - b.xx; r.xy = a.xy - b.xy; r.xz = a.xz - b.xz;
  r.yx = a.yx - b.yx; r.yy = a.yy - b.yy; r.yz = a.yz - b.yz;
  r.zx = a.zx - b.zx; r.zy = a.zy - b.zy; r.zz = a.zz - b.zz;
  return r;
}
__device__ __forceinline__ T3 t3_trans(const T3& m) {
  T3 r;
  r.xx = m.xx; r.yy = m.yy; r.zz = m.zz;
  r.xy = m.yx; r.xz = m.zx; r.yx = m.xy; r.yz = m.zy; r.zx = m.xz; r.zy = m.yz;
  return r;
}
// operator*(tensor3, tensor3) as written in tensor3.cu:241-256: column x of
// the result is (A.B), columns y and z are (A.B^T).  Kept for parity.
__device__ __forceinline__ T3 t3_mul_ref(const T3& a, const T3& b) {
  T3 r;
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

struct StressIn {
  T3 S;            // shear stress at the start of the step
  T3 D;            // strain rate
  double Wflat[6]; // rotation rate, flat
  double p, G, T;
};
struct StressState {
  double eps_p, sy;
  double pwn;   // cached eps_p^n (Johnson-Cook), < 0 when not cached
};
struct StressOut {
  T3 S, Sig;
  double seq, eff, dep;
  int newton_iters;
  double sy0, Th, st;   // JC return map: yield stress at the start, homologous T, trial stress
};

// ---- hardening laws (src/cuda/Material.cuh:257-307) ----------------------
__device__ __forceinline__ double jc_yield_ref(const MatParams& M, double strain, double sr_in,
                                               double temp) {
  double T_h = (temp - M.Tt) / (M.Tm - M.Tt);
  double sr = sr_in;
  if (sr_in == 0.0) sr = 1.e-5;
  return (M.A + M.B * pow(strain, M.n)) * (1.0 + M.C * log(sr / M.eps0)) * (1.0 - pow(T_h, M.m));
}
__device__ __forceinline__ double hollomon_yield(const MatParams& M, double strain) {
  if (strain + M.eps0_hol > M.eps1_hol) return M.K_hol * pow(strain + M.eps0_hol, M.m_hol);
  return M.sy0;
}

// sigma_y(eps_p0 + dl) and its slope for the consistent return map
struct Hard {
  int model;
  double R, Th, sy_cur, Ep;
};
__device__ __forceinline__ void hard_eval(const MatParams& M, const Hard& H, double ep0, double dl,
                                          double* sy, double* dsy) {
  if (H.model == WF_JOHNSON_COOK) {
    double e = ep0 + dl;
    if (e > 0.0) {
      double pw = pow(e, M.n);
      *sy = (M.A + M.B * pw) * H.R * H.Th;
      *dsy = M.n * M.B * pw / e * H.R * H.Th;
    } else {
      *sy = M.A * H.R * H.Th;
      *dsy = 1.0e300;
    }
  } else if (H.model == WF_HOLLOMON) {
    double e = ep0 + dl + M.eps0_hol;
    if (e > M.eps1_hol) {
      double pw = pow(e, M.m_hol);
      *sy = M.K_hol * pw;
      *dsy = M.m_hol * M.K_hol * pw / e;
    } else {
      *sy = M.sy0;
      *dsy = 0.0;
    }
  } else {
    *sy = H.sy_cur + H.Ep * dl;
    *dsy = H.Ep;
  }
}

// Newton on f(dl) = st - 3G dl - sy(ep0 + dl) over [0, (st - sy0)/3G], with a
// bisection safeguard; stops at |f| <= rtol * st.  Iterations are capped.
__device__ __forceinline__ double newton_return(const StepParams& P, const Hard& H, double st,
                                                double G3, double ep0, double sy0, double dl0,
                                                int* iters) {
  double hi = (st - sy0) / G3, lo = 0.0;
  double dl = dl0;
  if (!(dl > lo && dl <= hi)) dl = hi;
  int it = 0;
  for (; it < P.newton_max_iter; it++) {
    double sy, dsy;
    hard_eval(P.mat, H, ep0, dl, &sy, &dsy);
    double f = st - G3 * dl - sy;
    if (fabs(f) <= P.newton_rtol * st) break;
    if (f > 0.0) lo = dl; else hi = dl;
    double dn = dl + f / (G3 + dsy);
    if (!(dn > lo && dn < hi)) dn = 0.5 * (lo + hi);
    dl = dn;
  }
  *iters = it;
  return dl;
}

// (ep + dl)^n from the cached ep^n.  Plastic increments per step are ~1e-4 of
// the accumulated strain, so (1 + u)^n with u = dl / ep is summed as a
// binomial series to u^5 (truncation below 1e-18 relative for |u| < 1e-3);
// larger steps, and ep = 0, fall back to pow().  This keeps the yield
// function FP64-exact without an FP64 transcendental per Newton iterate.
__device__ __forceinline__ double pow_inc(const MatParams& M, double ep, double inv_ep, double pwn,
                                          double dl) {
  if (ep > 0.0 && fabs(dl) < 1.0e-3 * ep) {
    const double u = dl * inv_ep;
    const double s =
        1.0 + u * (M.bin[0] + u * (M.bin[1] + u * (M.bin[2] + u * (M.bin[3] + u * M.bin[4]))));
    return pwn * s;
  }
  const double e = ep + dl;
  return e > 0.0 ? pow(e, M.n) : 0.0;
}

// Johnson-Cook consistent return map: Newton on
//   f(dl) = st - 3G dl - (A + B (ep + dl)^n) * RT = 0,  RT = rate * thermal factor,
// bracketed on [0, (st - sy0)/3G], stopping at |f| <= rtol * st.  `pwn` is the
// cached ep^n (refreshed with pow() when < 0); on return it is (ep + dl)^n.
// dl_ratio in (0, 1] scales the radial start (the MLP warm start).
__device__ __forceinline__ void jc_return_cached(const StepParams& P, double st, double G3,
                                                 double ep, double& pwn, double RT,
                                                 double dl_ratio, double* dl_out, double* sy_out,
                                                 int* iters) {
  const MatParams& M = P.mat;
  if (!(pwn >= 0.0) || P.refresh_pow) pwn = ep > 0.0 ? pow(ep, M.n) : 0.0;
  const double inv_ep = ep > 0.0 ? 1.0 / ep : 0.0;
  const double sy0 = (M.A + M.B * pwn) * RT;
  *iters = 0;
  if (!(st > sy0)) {
    *dl_out = 0.0;
    *sy_out = sy0;
    return;
  }
  double hi = (st - sy0) / G3, lo = 0.0;
  double dl = (dl_ratio > 0.0 && dl_ratio <= 1.0) ? dl_ratio * hi : hi;
  double pw = pwn, sy = sy0;
  int it = 0;
  for (; it < P.newton_max_iter; it++) {
    pw = pow_inc(M, ep, inv_ep, pwn, dl);
    sy = (M.A + M.B * pw) * RT;
    const double f = st - G3 * dl - sy;
    if (fabs(f) <= P.newton_rtol * st) break;
    if (f > 0.0) lo = dl; else hi = dl;
    // the step needs the slope only to FP32 accuracy
    const float e = (float)(ep + dl);
    const float dsy = e > 0.0f ? (float)M.n * (float)M.B * (float)pw / e * (float)RT : 1.0e30f;
    double dn = dl + (double)((float)f / ((float)G3 + dsy));
    if (!(dn > lo && dn < hi)) dn = 0.5 * (lo + hi);
    dl = dn;
  }
  *iters = it;
  *dl_out = dl;
  *sy_out = sy;
  pwn = pw;
}

// Domain_d::StressStrainOne (src/cuda/Mechanical.cu:458-554): Jaumann update
// of the shear stress, J2 trial, then the reference radial return
// (return_map 0) or the consistent Newton return map (return_map 1).
// `dl_start` < 0 means "plain start" for the Newton map.
__device__ __forceinline__ void stress_update_fp64(const StepParams& P, const StressIn& in,
                                                   StressState& st, StressOut& out,
                                                   double dl_start_ratio = -1.0) {
  const MatParams& M = P.mat;
  T3 S = in.S;
  const T3& D = in.D;
  T3 W = t3_from_antisym(in.Wflat);
  T3 WT = t3_trans(W);
  T3 SRT = t3_mul_ref(S, WT);
  T3 RS = t3_mul_ref(W, S);
  T3 Dd = t3_sub(D, t3_ident(1.0 / 3.0 * (D.xx + D.yy + D.zz)));
  T3 T1 = t3_add(t3_add(t3_scale(Dd, 2.0 * in.G), SRT), RS);
  S = t3_add(t3_scale(T1, P.dt), S);
  double eff = sqrt(0.5 * ((D.xx - D.yy) * (D.xx - D.yy) + (D.yy - D.zz) * (D.yy - D.zz) +
                           (D.zz - D.xx) * (D.zz - D.xx)) +
                    3.0 * (D.xy * D.xy + D.yz * D.yz + D.zx * D.zx));
  double J2 = 0.5 * (S.xx * S.xx + 2.0 * S.xy * S.yx + 2.0 * S.xz * S.zx + S.yy * S.yy +
                     2.0 * S.yz * S.zy + S.zz * S.zz);
  double sig_trial = sqrt(3.0 * J2);
  double dep = 0.0;
  out.newton_iters = 0;
  if (P.return_map == 0) {
    if (st.sy < sig_trial) S = t3_scale(S, st.sy / sig_trial);
    if (M.model == WF_HOLLOMON) st.sy = hollomon_yield(M, st.eps_p);
    else if (M.model == WF_JOHNSON_COOK) st.sy = jc_yield_ref(M, st.eps_p, eff, in.T);
    out.seq = sig_trial;
    if (sig_trial > st.sy) {
      double Ep = 0.0;
      if (M.model == WF_BILINEAR) Ep = M.Ep;
      if (Ep < 0) Ep = 1.0 * M.E;
      dep = (sig_trial - st.sy) / (3. * in.G);
      st.eps_p += dep;
      out.seq = st.sy;
      if (M.model == WF_BILINEAR) st.sy += dep * Ep;
    }
  } else {
    Hard H;
    H.model = M.model;
    H.R = 1.0; H.Th = 1.0; H.sy_cur = st.sy; H.Ep = M.Ep;
    if (M.model == WF_JOHNSON_COOK) {
      double Th = (in.T - M.Tt) / (M.Tm - M.Tt);
      if (P.clamp_homologous) Th = Th < 0.0 ? 0.0 : (Th > 0.999 ? 0.999 : Th);
      double sr = eff == 0.0 ? 1.e-5 : eff;
      const double RT = (1.0 + M.C * log(sr / M.eps0)) * (1.0 - pow(Th, M.m));
      out.seq = sig_trial;
      if (!(st.pwn >= 0.0) || P.refresh_pow) st.pwn = st.eps_p > 0.0 ? pow(st.eps_p, M.n) : 0.0;
      out.sy0 = (M.A + M.B * st.pwn) * RT;
      out.Th = Th;
      out.st = sig_trial;
      double sy1;
      int it = 0;
      jc_return_cached(P, sig_trial, 3.0 * in.G, st.eps_p, st.pwn, RT, dl_start_ratio, &dep,
                       &sy1, &it);
      out.newton_iters = it;
      if (dep > 0.0) {
        S = t3_scale(S, sy1 / sig_trial);
        st.eps_p += dep;
        out.seq = sy1;
      }
      st.sy = sy1;
      out.dep = dep;
      out.eff = eff;
      out.S = S;
      out.Sig = t3_add(t3_ident(-in.p), S);
      return;
    }
    double sy0, dsy0;
    hard_eval(M, H, st.eps_p, 0.0, &sy0, &dsy0);
    out.seq = sig_trial;
    if (sig_trial > sy0) {
      double G3 = 3.0 * in.G;
      double dl0 = (sig_trial - sy0) / G3;
      if (dl_start_ratio > 0.0 && dl_start_ratio <= 1.0) dl0 = dl_start_ratio * dl0;
      int it = 0;
      dep = newton_return(P, H, sig_trial, G3, st.eps_p, sy0, dl0, &it);
      out.newton_iters = it;
      double sy1, dsy1;
      hard_eval(M, H, st.eps_p, dep, &sy1, &dsy1);
      S = t3_scale(S, sy1 / sig_trial);
      st.eps_p += dep;
      st.sy = sy1;
      out.seq = sy1;
    } else {
      st.sy = sy0;
    }
  }
  out.dep = dep;
  out.eff = eff;
  out.S = S;
  out.Sig = t3_add(t3_ident(-in.p), S);
}
