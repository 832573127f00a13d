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

// Contact law 1 (the 2M-particle contact workload; no reference
// counterpart).  A solid particle looks up its cell in each tool's triangle
// bins (built once in the tool's frame; the frame moves with node 0) and takes
// the nearest triangle whose closest point lies within h (ties: first mesh,
// lowest triangle index).  With the gap g = (x - q).n along the face's outward
// normal and the penetration delta = dx/2 - g > 0 the normal force is
// kappa K dx delta (pressure kappa K / dx on the face dx^2); friction is
// Coulomb, regularised below v_reg: F_t = -mu F_n v_t / max(|v_t|, v_reg);
// eta of the frictional power heats the particle.  Mixed form: the
// acceleration comes from and returns to the FP32 array.
__global__ void __launch_bounds__(128) k_contact_law1(StepParams P, Fields F, float4* a32) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= P.n || F.perm[i] >= P.n_solid) return;
  const double4 x4 = F.xm[i];
  const V3 xi = mk(x4);
  double best = P.h * P.h;
  int bm = -1, be = -1;
  V3 bq = mk(0.0, 0.0, 0.0);
  for (int m = 0; m < P.ncsid; m++) {
    const MeshDev& M = P.mesh[m];
    const double4 n0 = M.node[0];
    const V3 xt = xi - (mk(n0) - mk(M.org[0], M.org[1], M.org[2]));
    // cell coordinates compared in double first: a particle far outside the
    // grid (or a NaN position) is skipped before any integer conversion
    const double fx = floor((xt.x - M.gmin[0]) / M.cs);
    const double fy = floor((xt.y - M.gmin[1]) / M.cs);
    const double fz = floor((xt.z - M.gmin[2]) / M.cs);
    if (!(fx >= 0.0 && fy >= 0.0 && fz >= 0.0 && fx < (double)M.dims[0] &&
          fy < (double)M.dims[1] && fz < (double)M.dims[2]))
      continue;
    const int cell = ((int)fz * M.dims[1] + (int)fy) * M.dims[0] + (int)fx;
    for (int t = M.cstart[cell]; t < M.cstart[cell + 1]; t++) {
      const int e = M.ctri[t];
      const int32_t* en = M.elnode + 3 * e;
      const V3 q = closest_on_tri(xi, mk(M.node[en[0]]), mk(M.node[en[1]]), mk(M.node[en[2]]));
      const V3 dv = xi - q;
      const double d2 = dot(dv, dv);
      if (d2 < best || (d2 == best && bm == m && e < be)) {
        best = d2; bm = m; be = e; bq = q;
      }
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
      const V3 vrel = mk(F.vd[i]) - mk(M.mv[0], M.mv[1], M.mv[2]);
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
  M.node[q] = d4(nd + scale(nv, dt));
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
