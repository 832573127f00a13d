// wf_contact.cu — contact of the SPH solid with rigid triangle meshes.
//
// Free-surface tagging (Domain_d::CalculateSurface, src/cuda/Geometry.cu:26-88),
// the contact neighbour list (CalcContactNb, src/cuda/Contact.cu:29-62), the
// penalty force with friction (CalcContactForcesWang, Contact.cu:134-321), the
// rigid mesh motion (MeshUpdateKernel, src/cuda/Mesh.cu:24-29, 222-276) and the
// rigid centroid particles (UpdateContactParticles, Contact.cu:85-112).
//
// Compiled with -fmad=false: the FP64 arithmetic follows the reference's
// operation order (vector_math.h: a / s is a * (1.0 / s), dot sums left to
// right, length = sqrt(dot)), so the plain form matches the oracle bit for bit.
// One thread per particle (surface, list, force), per node (mesh motion) or
// per element (element geometry, rigid particles).
#include "wf_common.cuh"
#include "wf_nsearch.cuh"

namespace {

struct V3 {
  double x, y, z;
};
__device__ __forceinline__ V3 mk(double x, double y, double z) { return V3{x, y, z}; }
__device__ __forceinline__ V3 mk(const double4& a) { return V3{a.x, a.y, a.z}; }
__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ V3 scale(V3 a, double s) { return mk(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ V3 divide(V3 a, double s) { return scale(a, 1.0 / s); }
__device__ __forceinline__ double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ double len(V3 a) { return sqrt(dot(a, a)); }
__device__ __forceinline__ V3 cross(V3 a, V3 b) {
  return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ double4 d4(V3 a, double w = 0.0) { return make_double4(a.x, a.y, a.z, w); }

// the mesh whose element centroids include the particle of original id `orig`
__device__ __forceinline__ int mesh_of(const StepParams& P, int32_t orig) {
  for (int m = 0; m < P.ncsid; m++)
    if (orig >= P.mesh[m].first && orig < P.mesh[m].first + P.mesh[m].ne) return m;
  return -1;
}

// CalculateSurface: normal = N / (M n') sum m_j (x_i - x_j) over the n'
// neighbours that are not rigid particles of the first mesh; |normal| >= 0.25 h
// with n' <= 46 tags the particle as free surface unless its zone is protected.
// Other threads may turn a neighbour's id into the free-surface id meanwhile;
// that id is never a mesh zone id, so the test on ID[j] does not change.
__global__ void __launch_bounds__(128) k_surface(StepParams P, Fields F,
                                                 const int32_t* __restrict__ nb,
                                                 const int32_t* __restrict__ cnt) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= P.n || F.perm[i] >= P.n_solid) return;
  const V3 xi = mk(F.xm[i]);
  V3 nrm = mk(0.0, 0.0, 0.0);
  int corr = 0;
  const int c = cnt[i];
  for (int k = 0; k < c; k++) {
    const int j = __ldg(nb + nb_at(P.npad, i, k));
    const double4 xj = F.xm[j];
    const V3 xij = xi - mk(xj);
    if (F.id[j] != P.csid[0]) {
      nrm = nrm + scale(xij, xj.w);
      corr++;
    }
  }
  nrm = scale(nrm, (double)P.n / (P.totmass * (double)corr));
  F.nrm[i] = d4(nrm);
  if (len(nrm) >= 0.25 * P.h && corr <= 46 && !F.nw[i]) F.id[i] = P.id_free_surf;
}

// CalcContactNb: rigid neighbours within 2h of a free-surface particle, in
// neighbour order, once per mesh whose zone id matches; at most WF_CONT_NB
// (the reference writes past its 20 slots).  Column-major: cnb[k * npad + i].
__global__ void __launch_bounds__(128) k_contact_nb(StepParams P, Fields F,
                                                    const int32_t* __restrict__ nb,
                                                    const int32_t* __restrict__ cnt) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= P.n || F.perm[i] >= P.n_solid) return;
  int cc = 0;
  if (F.id[i] == P.id_free_surf) {
    const V3 xi = mk(F.xm[i]);
    const int c = cnt[i];
    for (int k = 0; k < c; k++) {
      const int j = __ldg(nb + nb_at(P.npad, i, k));
      const int32_t idj = F.id[j];
      const double r = len(xi - mk(F.xm[j]));
      for (int mc = 0; mc < P.ncsid; mc++)
        if (idj == P.csid[mc] && r < 2. * P.h && cc < WF_CONT_NB)
          P.cnb[(int64_t)(cc++) * P.npad + i] = j;
    }
  }
  P.ccnt[i] = cc;
}

// CalcContactForcesWang: for each contact neighbour j (the centroid particle of
// element e), the predicted position x + v dt + a dt^2 / 2 is tested against
// the element's plane and, projected on it, against the triangle's edges; a
// hit adds the penalty force 0.4 kij (h - dist) n, kij = 2 m / dt^2, with
// static or dynamic friction.  contforce keeps the last contact's force; the
// acceleration accumulates all of them, and later contacts see the earlier
// ones through the predicted position.  Mixed form: the acceleration comes
// from and returns to the FP32 array.
__global__ void __launch_bounds__(128) k_contact_force(StepParams P, Fields F, float4* a32) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= P.n || F.perm[i] >= P.n_solid) return;
  const int cc = P.ccnt[i];
  V3 cf = mk(0.0, 0.0, 0.0);
  if (cc > 0) {
    const double4 x4 = F.xm[i];
    const V3 xi = mk(x4), vi = mk(F.vd[i]);
    const double mi = x4.w, dt = P.dt, h = P.h;
    V3 a;
    if (a32) {
      const float4 af = a32[i];
      a = mk(af.x, af.y, af.z);
    } else {
      a = mk(F.a[i]);
    }
    for (int k = 0; k < cc; k++) {
      const int j = P.cnb[(int64_t)k * P.npad + i];
      const int32_t oj = F.perm[j];
      const int mid = mesh_of(P, oj);
      const MeshDev& M = P.mesh[mid];
      const int e = oj - M.first;
      const V3 x_pred = (xi + scale(vi, dt)) + divide(scale(scale(a, dt), dt), 2.);
      const V3 n = mk(M.normal[e]);
      const double dist = dot(n, x_pred) - M.pplane[e];
      if (!(dist < h)) continue;
      const V3 Qj = xi - scale(n, dist);
      bool inside = true;
      for (int l = 0; l < 3 && inside; l++) {
        const int nx = l + 1 > 2 ? 0 : l + 1;
        const V3 pl = mk(M.node[M.elnode[3 * e + l]]);
        const V3 pn = mk(M.node[M.elnode[3 * e + nx]]);
        if (dot(cross(pn - pl, Qj - pl), n) < 0.0) inside = false;
      }
      if (!inside) continue;
      const double delta = h - dist;
      const double kij = 2.0 * mi / (dt * dt);
      cf = scale(n, 0.4 * kij * delta);
      a = a + divide(cf, mi);
      if (P.mu_s > 0.) {
        const V3 du = (x_pred - xi) - scale(mk(F.vd[j]), dt);
        const V3 dtg = du - scale(n, dot(du, n));
        const V3 ft = scale(dtg, kij);
        if (len(ft) < P.mu_s * len(cf)) {
          a = a - divide(ft, mi);
        } else {
          const V3 fd = divide(scale(ft, P.mu_d * len(cf)), len(ft));
          cf = cf - fd;
          a = a - divide(fd, mi);
        }
      }
    }
    if (a32) a32[i] = make_float4((float)a.x, (float)a.y, (float)a.z, 0.f);
    else F.a[i] = d4(a);
  }
  F.cf[i] = d4(cf);
}

// Closest point of triangle abc to p (Ericson, Real-Time Collision Detection,
// 5.1.5: Voronoi regions of the vertices, edges and face).
__device__ V3 closest_on_tri(V3 p, V3 a, V3 b, V3 c) {
  const V3 ab = b - a, ac = c - a, ap = p - a;
  const double d1 = dot(ab, ap), d2 = dot(ac, ap);
  if (d1 <= 0.0 && d2 <= 0.0) return a;
  const V3 bp = p - b;
  const double d3 = dot(ab, bp), d4 = dot(ac, bp);
  if (d3 >= 0.0 && d4 <= d3) return b;
  const double vc = d1 * d4 - d3 * d2;
  if (vc <= 0.0 && d1 >= 0.0 && d3 <= 0.0) return a + scale(ab, d1 / (d1 - d3));
  const V3 cp = p - c;
  const double d5 = dot(ab, cp), d6 = dot(ac, cp);
  if (d6 >= 0.0 && d5 <= d6) return c;
  const double vb = d5 * d2 - d1 * d6;
  if (vb <= 0.0 && d2 >= 0.0 && d6 <= 0.0) return a + scale(ac, d2 / (d2 - d6));
  const double va = d3 * d6 - d5 * d4;
  if (va <= 0.0 && (d4 - d3) >= 0.0 && (d5 - d6) >= 0.0)
    return b + scale(c - b, (d4 - d3) / ((d4 - d3) + (d5 - d6)));
  const double denom = 1.0 / (va + vb + vc);
  return (a + scale(ab, vb * denom)) + scale(ac, vc * denom);
}

// The same closest-point rule in FP32 on tool-relative coordinates; returns
// the squared distance.  Used only to choose which triangles the FP64 rule
// evaluates (the FP64 pipe runs at 1/64 of the FP32 rate on this GPU).
__device__ __forceinline__ float3 f3sub(float3 a, float3 b) {
  return make_float3(a.x - b.x, a.y - b.y, a.z - b.z);
}
__device__ __forceinline__ float f3dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float3 f3axpy(float3 a, float3 d, float t) {
  return make_float3(a.x + d.x * t, a.y + d.y * t, a.z + d.z * t);
}
__device__ float closest_sq32(float3 p, float3 a, float3 b, float3 c) {
  const float3 ab = f3sub(b, a), ac = f3sub(c, a), ap = f3sub(p, a);
  const float d1 = f3dot(ab, ap), d2 = f3dot(ac, ap);
  float3 q;
  const float3 bp = f3sub(p, b), cp = f3sub(p, c);
  const float d3 = f3dot(ab, bp), d4 = f3dot(ac, bp);
  const float d5 = f3dot(ab, cp), d6 = f3dot(ac, cp);
  const float vc = d1 * d4 - d3 * d2, vb = d5 * d2 - d1 * d6, va = d3 * d6 - d5 * d4;
  if (d1 <= 0.f && d2 <= 0.f) q = a;
  else if (d3 >= 0.f && d4 <= d3) q = b;
  else if (vc <= 0.f && d1 >= 0.f && d3 <= 0.f) q = f3axpy(a, ab, d1 / (d1 - d3));
  else if (d6 >= 0.f && d5 <= d6) q = c;
  else if (vb <= 0.f && d2 >= 0.f && d6 <= 0.f) q = f3axpy(a, ac, d2 / (d2 - d6));
  else if (va <= 0.f && (d4 - d3) >= 0.f && (d5 - d6) >= 0.f)
    q = f3axpy(b, f3sub(c, b), (d4 - d3) / ((d4 - d3) + (d5 - d6)));
  else {
    const float den = 1.f / (va + vb + vc);
    q = f3axpy(f3axpy(a, ab, vb * den), ac, vc * den);
  }
  const float3 dq = f3sub(p, q);
  return f3dot(dq, dq);
}

__device__ __forceinline__ float3 rel32(const float4* r, int q) {
  const float4 v = r[q];
  return make_float3(v.x, v.y, v.z);
}

// The particle's cell in mesh M's bins, or -1 outside the grid (compared in
// double first: a particle far outside the grid, or a NaN position, is
// skipped before any integer conversion; the bins carry a margin of h, so the
// rounding of the product cannot lose a triangle within h).
__device__ __forceinline__ int tool_cell(const MeshDev& M, V3 xi) {
  const V3 r = xi - mk(M.node[0]);
  const double fx = floor((r.x - M.grel[0]) * M.inv_cs);
  const double fy = floor((r.y - M.grel[1]) * M.inv_cs);
  const double fz = floor((r.z - M.grel[2]) * M.inv_cs);
  if (!(fx >= 0.0 && fy >= 0.0 && fz >= 0.0 && fx < (double)M.dims[0] &&
        fy < (double)M.dims[1] && fz < (double)M.dims[2]))
    return -1;
  return ((int)fz * M.dims[1] + (int)fy) * M.dims[0] + (int)fx;
}

// Bins of a rotating tool, rebuilt every step from the current nodes: every
// triangle goes into each cell that its bounding box (relative to node 0)
// widened by the margin touches, with its vertices relative to node 0 in
// FP32.  Count, exclusive scan (cstart), fill; the order within a cell depends
// on the atomics, which the search's explicit tie rule makes irrelevant.
__device__ __forceinline__ void tri_cells(const MeshDev& M, int e, V3 rv[3], int r0[3], int r1[3]) {
  const int32_t* en = M.elnode + 3 * e;
  const V3 n0 = mk(M.node[0]);
  for (int k = 0; k < 3; k++) rv[k] = mk(M.node[en[k]]) - n0;
  const double lo[3] = {fmin(fmin(rv[0].x, rv[1].x), rv[2].x), fmin(fmin(rv[0].y, rv[1].y), rv[2].y),
                        fmin(fmin(rv[0].z, rv[1].z), rv[2].z)};
  const double hi[3] = {fmax(fmax(rv[0].x, rv[1].x), rv[2].x), fmax(fmax(rv[0].y, rv[1].y), rv[2].y),
                        fmax(fmax(rv[0].z, rv[1].z), rv[2].z)};
  for (int k = 0; k < 3; k++) {
    const double a = floor((lo[k] - M.margin - M.grel[k]) * M.inv_cs);
    const double b = floor((hi[k] + M.margin - M.grel[k]) * M.inv_cs);
    // clamped in double before the conversion (NaN gives an empty range)
    r0[k] = (int)fmin(fmax(a, 0.0), (double)M.dims[k]);
    r1[k] = (int)fmax(fmin(b, (double)(M.dims[k] - 1)), -1.0);
  }
}
__global__ void k_bins_count(MeshDev M) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= M.ne) return;
  V3 rv[3];
  int r0[3], r1[3];
  tri_cells(M, e, rv, r0, r1);
  uint32_t* cnt = reinterpret_cast<uint32_t*>(M.cstart);
  for (int z = r0[2]; z <= r1[2]; z++)
    for (int y = r0[1]; y <= r1[1]; y++)
      for (int x = r0[0]; x <= r1[0]; x++)
        atomicAdd(cnt + ((int64_t)z * M.dims[1] + y) * M.dims[0] + x, 1u);
}
__global__ void k_bins_fill(MeshDev M) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= M.ne) return;
  V3 rv[3];
  int r0[3], r1[3];
  tri_cells(M, e, rv, r0, r1);
  for (int z = r0[2]; z <= r1[2]; z++)
    for (int y = r0[1]; y <= r1[1]; y++)
      for (int x = r0[0]; x <= r1[0]; x++) {
        const uint32_t pos = atomicAdd(M.cursor + ((int64_t)z * M.dims[1] + y) * M.dims[0] + x, 1u);
        if ((int64_t)pos >= M.cap) continue;   // bounded by construction (cap)
        float4* v = M.cvert + 3 * (int64_t)pos;
        v[0] = make_float4((float)rv[0].x, (float)rv[0].y, (float)rv[0].z, __int_as_float(e));
        v[1] = make_float4((float)rv[1].x, (float)rv[1].y, (float)rv[1].z, 0.f);
        v[2] = make_float4((float)rv[2].x, (float)rv[2].y, (float)rv[2].z, 0.f);
      }
}

// Contact law 1 (the 2M-particle contact workload; no reference
// counterpart).  A solid particle looks up its cell in each tool's triangle
// bins (built once in the tool's frame; the frame moves with node 0) and takes
// the nearest triangle whose closest point q lies within h (ties: first mesh,
// lowest triangle index), searched in FP32 and decided in FP64.  With the gap
// g = |x - q| along n = (x - q)/g (the face normal and the signed gap for a
// centre behind the face) and the penetration delta = dx/2 - g > 0 the normal
// force is
// kappa K dx delta (pressure kappa K / dx on the face dx^2); friction is
// Coulomb, regularised below v_reg: F_t = -mu F_n v_t / max(|v_t|, v_reg);
// eta of the frictional power heats the particle.  Mixed form: the
// acceleration comes from and returns to the FP32 array.
__global__ void __launch_bounds__(128) k_contact_law1(StepParams P, Fields F, float4* a32) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= P.n || F.perm[i] >= P.n_solid) return;
  // FP32 early-out against each tool's bin grid widened by one cell (far
  // larger than FP32 rounding): most particles are nowhere near a tool and
  // skip all FP64 work.  The mixed form keeps an FP32 position mirror.
  float px, py, pz;
  if (a32) {
    const float4 p = F.p32[i];
    px = p.x; py = p.y; pz = p.z;
  } else {
    const double4 p = F.xm[i];
    px = (float)p.x; py = (float)p.y; pz = (float)p.z;
  }
  bool near = false;
  for (int m = 0; m < P.ncsid; m++) {
    const MeshDev& M = P.mesh[m];
    const float4 o = M.off32[0];
    const float tx = px - o.x, ty = py - o.y, tz = pz - o.z;
    near |= tx >= M.glo[0] && tx <= M.ghi[0] && ty >= M.glo[1] && ty <= M.ghi[1] &&
            tz >= M.glo[2] && tz <= M.ghi[2];
  }
  if (!near) {
    F.cf[i] = make_double4(0.0, 0.0, 0.0, 0.0);
    F.qf[i] = 0.0;
    P.ccnt[i] = 0;
    return;
  }
  const double4 x4 = F.xm[i];
  const V3 xi = mk(x4);
  // Pass 1, FP32: the smallest squared distance over the candidate triangles,
  // in coordinates relative to each tool's node 0 (each bin entry carries its
  // triangle's FP32 vertices, so the loads of successive entries overlap).
  float m32 = P.hf * P.hf, tol = 0.f;
  unsigned n32 = 0, n64 = 0;
  for (int m = 0; m < P.ncsid; m++) {
    const MeshDev& M = P.mesh[m];
    const int cell = tool_cell(M, xi);
    if (cell < 0) continue;
    tol = fmaxf(tol, M.tol32);
    const double4 n0 = M.node[0];
    const float3 pr = make_float3((float)(xi.x - n0.x), (float)(xi.y - n0.y), (float)(xi.z - n0.z));
    const int t0 = M.cstart[cell], t1 = M.cstart[cell + 1];
    n32 += (unsigned)(t1 - t0);
#pragma unroll 4
    for (int t = t0; t < t1; t++) {
      const float4* v = M.cvert + 3 * (int64_t)t;
      m32 = fminf(m32, closest_sq32(pr, rel32(v, 0), rel32(v, 1), rel32(v, 2)));
    }
  }
  // Pass 2, FP64: the triangles within tol (in distance) of that minimum, in
  // the order and with the tie rule of a scan of every triangle.  tol is far
  // above the FP32 distance error, so the FP64 minimum is always among them.
  // Candidates are collected first (FP32) and evaluated together: inside the
  // scan, lanes pass the filter at different entries and a warp would run the
  // FP64 test once per such entry.  A lane with more than kCand candidates
  // (never seen on tessellated tools) scans again in FP64.
  constexpr int kCand = 8;
  const float lim = sqrtf(m32) + tol;
  const float thr = lim * lim;
  int cand[kCand];
  int ncand = 0;
  for (int m = 0; m < P.ncsid; m++) {
    const MeshDev& M = P.mesh[m];
    const int cell = tool_cell(M, xi);
    if (cell < 0) continue;
    const double4 n0 = M.node[0];
    const float3 pr = make_float3((float)(xi.x - n0.x), (float)(xi.y - n0.y), (float)(xi.z - n0.z));
    const int t1 = M.cstart[cell + 1];
#pragma unroll 4
    for (int t = M.cstart[cell]; t < t1; t++) {
      const float4* v = M.cvert + 3 * (int64_t)t;
      const float4 v0 = v[0];
      if (closest_sq32(pr, make_float3(v0.x, v0.y, v0.z), rel32(v, 1), rel32(v, 2)) > thr)
        continue;
      if (ncand < kCand) cand[ncand] = (m << 24) | __float_as_int(v0.w);
      ncand++;
    }
  }
  double best = P.h * P.h;
  int bm = -1, be = -1;
  V3 bq = mk(0.0, 0.0, 0.0);
  auto consider = [&](int m, int e) {
    const MeshDev& M = P.mesh[m];
    const int32_t* en = M.elnode + 3 * e;
    const V3 q = closest_on_tri(xi, mk(M.node[en[0]]), mk(M.node[en[1]]), mk(M.node[en[2]]));
    const V3 dv = xi - q;
    const double d2 = dot(dv, dv);
    if (d2 < best || (d2 == best && bm == m && e < be)) {
      best = d2; bm = m; be = e; bq = q;
    }
  };
  if (ncand <= kCand) {
    for (int k = 0; k < ncand; k++) consider(cand[k] >> 24, cand[k] & 0xffffff);
    n64 += (unsigned)ncand;
  } else {
    for (int m = 0; m < P.ncsid; m++) {
      const MeshDev& M = P.mesh[m];
      const int cell = tool_cell(M, xi);
      if (cell < 0) continue;
      const double4 n0 = M.node[0];
      const float3 pr = make_float3((float)(xi.x - n0.x), (float)(xi.y - n0.y), (float)(xi.z - n0.z));
      for (int t = M.cstart[cell]; t < M.cstart[cell + 1]; t++) {
        const float4* v = M.cvert + 3 * (int64_t)t;
        const float4 v0 = v[0];
        if (closest_sq32(pr, make_float3(v0.x, v0.y, v0.z), rel32(v, 1), rel32(v, 2)) > thr)
          continue;
        consider(m, __float_as_int(v0.w));
        n64++;
      }
    }
  }
  {
    const unsigned mask = __activemask();
    const unsigned s32 = __reduce_add_sync(mask, n32), s64 = __reduce_add_sync(mask, n64);
    if ((int)(threadIdx.x & 31) == __ffs(mask) - 1 && s32) {
      atomicAdd(P.cstat, (unsigned long long)s32);
      atomicAdd(P.cstat + 1, (unsigned long long)s64);
    }
  }
  V3 f = mk(0.0, 0.0, 0.0);
  double qf = 0.0;
  int cnt = 0;
  if (bm >= 0) {
    const MeshDev& M = P.mesh[bm];
    // contact normal: from the nearest surface point to the particle (the
    // face normal inside a face, continuous across edges and vertices); the
    // face normal and its signed gap for a centre behind the face
    const V3 dv = xi - bq;
    const double dist = sqrt(best);
    const double gf = dot(dv, mk(M.normal[be]));
    V3 n;
    double g;
    if (gf >= 0.0 && dist > 0.0) {
      n = divide(dv, dist);
      g = dist;
    } else {
      n = mk(M.normal[be]);
      g = gf;
    }
    const double delta = 0.5 * P.c_dx - g;
    if (delta > 0.0) {
      const double fn = P.c_kappa * P.Kbulk * P.c_dx * delta;
      f = scale(n, fn);
      // relative to the tool surface at the nearest point: m_v + m_w x q
      const V3 vtool = mk(M.mv[0], M.mv[1], M.mv[2]) + cross(mk(M.mw[0], M.mw[1], M.mw[2]), bq);
      const V3 vrel = mk(F.vd[i]) - vtool;
      const V3 vt = vrel - scale(n, dot(vrel, n));
      const double vtl = len(vt);
      if (P.mu_s > 0.0) {
        const double s = P.mu_s * fn / (vtl > P.c_vreg ? vtl : P.c_vreg);
        f = f - scale(vt, s);
        qf = P.c_eta * s * vtl * vtl;
      }
      V3 a;
      if (a32) {
        const float4 af = a32[i];
        a = mk(af.x, af.y, af.z);
      } else {
        a = mk(F.a[i]);
      }
      a = a + divide(f, x4.w);
      if (a32) a32[i] = make_float4((float)a.x, (float)a.y, (float)a.z, 0.f);
      else F.a[i] = d4(a);
      cnt = 1;
    }
  }
  F.cf[i] = d4(f);
  F.qf[i] = qf;
  P.ccnt[i] = cnt;
}

// TriMesh_d::Move: node velocity m_v + m_w x node, then node += v dt
__global__ void k_mesh_move(MeshDev M, double dt) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= M.nn) return;
  const V3 nd = mk(M.node[q]);
  const V3 vr = cross(mk(M.mw[0], M.mw[1], M.mw[2]), nd);
  const V3 nv = mk(M.mv[0], M.mv[1], M.mv[2]) + vr;
  M.node_v[q] = d4(nv);
  const V3 moved = nd + scale(nv, dt);
  M.node[q] = d4(moved);
  if (q == 0 && M.off32)   // node 0 in FP32 for the law-1 early-out
    M.off32[0] = make_float4((float)moved.x, (float)moved.y, (float)moved.z, 0.f);
}

// CalcCentroids, CalcNormals and UpdatePlaneCoeff of one element from the
// moved nodes; the plane coefficient reads node[elnode[3e] + nfar] with
// nfar = 2, the index CalcSpheres leaves (Mesh.cu:205-231)
__global__ void k_mesh_elems(MeshDev M, int geometry) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= M.ne) return;
  if (geometry) {
    const V3 n0 = mk(M.node[M.elnode[3 * e]]), n1 = mk(M.node[M.elnode[3 * e + 1]]),
             n2 = mk(M.node[M.elnode[3 * e + 2]]);
    M.centroid[e] = d4(divide((n0 + n1) + n2, 3.));
    const V3 w = cross(n1 - n0, n2 - n0);
    M.normal[e] = d4(divide(w, len(w)));
  }
  M.pplane[e] = dot(mk(M.node[M.elnode[3 * e] + 2]), mk(M.normal[e]));
}

// UpdateContactParticles: the element's rigid particle takes the mean node
// velocity, zero acceleration and the element normal
__global__ void k_contact_particles(StepParams P, Fields F, MeshDev M, int mixed) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= M.ne) return;
  const int32_t s = P.inv[M.first + e];
  V3 vv = mk(0.0, 0.0, 0.0);
  for (int q = 0; q < 3; q++) vv = vv + mk(M.node_v[M.elnode[3 * e + q]]);
  const V3 v = divide(vv, 3.);
  const double rho = F.vd[s].w;
  F.vd[s] = d4(v, rho);
  F.a[s] = make_double4(0.0, 0.0, 0.0, 0.0);
  F.nrm[s] = M.normal[e];
  if (mixed) F.v32[s] = make_float4((float)v.x, (float)v.y, (float)v.z, (float)rho);
}

inline int blocks_for(int64_t n, int t) { return (int)((n + t - 1) / t); }

}  // namespace

void launch_contact_stage(const StepParams& P, const Fields& F, const NbBuffers& N, bool list,
                          float4* a32, cudaStream_t s) {
  if (P.contact_law == 1) {
    for (int m = 0; m < P.ncsid; m++) {   // rotating tools: bins from the current nodes
      const MeshDev& M = P.mesh[m];
      if (!M.rot) continue;
      const int64_t ncell = (int64_t)M.dims[0] * M.dims[1] * M.dims[2];
      cudaMemsetAsync(M.cstart, 0, sizeof(uint32_t) * (ncell + 1), s);
      k_bins_count<<<blocks_for(M.ne, 128), 128, 0, s>>>(M);
      device_exclusive_scan(reinterpret_cast<uint32_t*>(M.cstart), ncell + 1, M.scan_tmp, s);
      cudaMemcpyAsync(M.cursor, M.cstart, sizeof(uint32_t) * ncell, cudaMemcpyDeviceToDevice, s);
      k_bins_fill<<<blocks_for(M.ne, 128), 128, 0, s>>>(M);
    }
    k_contact_law1<<<blocks_for(P.n, 128), 128, 0, s>>>(P, F, a32);
    return;
  }
  k_surface<<<blocks_for(P.n, 128), 128, 0, s>>>(P, F, N.nb, N.cnt);
  if (list) k_contact_nb<<<blocks_for(P.n, 128), 128, 0, s>>>(P, F, N.nb, N.cnt);
  k_contact_force<<<blocks_for(P.n, 128), 128, 0, s>>>(P, F, a32);
}

void launch_mesh_update(const StepParams& P, const Fields& F, int mixed, cudaStream_t s) {
  for (int m = 0; m < P.ncsid; m++) {
    const MeshDev& M = P.mesh[m];
    k_mesh_move<<<blocks_for(M.nn, 128), 128, 0, s>>>(M, P.dt);
    k_mesh_elems<<<blocks_for(M.ne, 128), 128, 0, s>>>(M, 1);
  }
  for (int m = 0; m < P.ncsid; m++)
    k_contact_particles<<<blocks_for(P.mesh[m].ne, 128), 128, 0, s>>>(P, F, P.mesh[m], mixed);
}

void launch_mesh_plane(const StepParams& P, cudaStream_t s) {
  for (int m = 0; m < P.ncsid; m++)
    k_mesh_elems<<<blocks_for(P.mesh[m].ne, 128), 128, 0, s>>>(P.mesh[m], 0);
}
