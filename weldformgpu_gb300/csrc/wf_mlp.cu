// wf_mlp.cu — the learned warm start of the Johnson-Cook return map:
// synthetic (state, converged increment) pairs, FP32 training kernels
// (forward, backward, Adam), BF16 tcgen05 tensor-core inference, and a kernel that
// counts Newton iterations with and without the network.
//
// No counterpart in the reference: its return map is a one-shot radial
// return (src/cuda/Mechanical.cu:503-536) with no iterative solve.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/weldform_gb300.h"
#include "wf_common.cuh"
#include "wf_mlp.cuh"
#include "wf_tensor.cuh"

namespace {

// ---- parameter packing for the tensor-core kernels ---------------------------
// The tcgen05 weight image (mlp_umma_cta): B2 = W2 in BF16, K-major core-
// matrix order, then b2, W3 and b3 in FP32 (layer 1 travels as MlpL1).
__global__ void k_mlp_pack_umma(const float* __restrict__ P, uint8_t* __restrict__ out) {
  const float* W2 = P + WF_MLP_OFF_W2;
  for (int k = threadIdx.x; k < WF_UMMA_IMAGE / 4; k += blockDim.x)
    reinterpret_cast<uint32_t*>(out)[k] = 0u;
  __syncthreads();
  for (int e = threadIdx.x; e < WF_MLP_H * WF_MLP_H; e += blockDim.x) {
    const int n = e / WF_MLP_H, k = e % WF_MLP_H;
    *reinterpret_cast<__nv_bfloat16*>(out + WF_UMMA_B2 + umma_kmajor_off(n, k, WF_MLP_H)) =
        __float2bfloat16_rn(W2[n * WF_MLP_H + k]);
  }
  for (int k = threadIdx.x; k < WF_MLP_H; k += blockDim.x) {
    reinterpret_cast<float*>(out + WF_UMMA_BIAS2)[k] = P[WF_MLP_OFF_B2 + k];
    reinterpret_cast<float*>(out + WF_UMMA_W3)[k] = P[WF_MLP_OFF_W3 + k];
  }
  if (threadIdx.x == 0) *reinterpret_cast<float*>(out + WF_UMMA_B3) = P[WF_MLP_OFF_B3];
}

// ---- standalone inference ---------------------------------------------------
__global__ void __launch_bounds__(128) k_mlp_infer_umma(const uint4* __restrict__ image,
                                                        const MlpL1 l1,
                                                        const float4* __restrict__ X, int64_t n,
                                                        float* __restrict__ Y, int* status) {
  extern __shared__ __align__(1024) uint8_t smu[];
  mlp_umma_begin(smu, image);
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const bool valid = i < n;
  float f[4] = {0.f, 0.f, 0.f, 0.f};
  if (valid) {
    const float4 x = X[i];
    f[0] = x.x; f[1] = x.y; f[2] = x.z; f[3] = x.w;
  }
  const float y = mlp_umma_cta(smu, image, f, valid, status, l1);
  if (valid) Y[i] = y;
}

__global__ void k_mlp_infer_f32(const float* __restrict__ P, const float4* __restrict__ X,
                                int64_t n, float* __restrict__ Y) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 x = X[i];
  const float f[4] = {x.x, x.y, x.z, x.w};
  float h1[WF_MLP_H];
  for (int o = 0; o < WF_MLP_H; o++) {
    float z = P[WF_MLP_OFF_B1 + o];
    for (int k = 0; k < 4; k++) z += P[WF_MLP_OFF_W1 + o * 4 + k] * f[k];
    h1[o] = mlp_silu(z);
  }
  float y = P[WF_MLP_OFF_B3];
  for (int o = 0; o < WF_MLP_H; o++) {
    float z = P[WF_MLP_OFF_B2 + o];
    for (int k = 0; k < WF_MLP_H; k++) z += P[WF_MLP_OFF_W2 + o * WF_MLP_H + k] * h1[k];
    y += P[WF_MLP_OFF_W3 + o] * mlp_silu(z);
  }
  Y[i] = y;
}

// ---- synthetic states with converged FP64 targets ------------------------------
__device__ __forceinline__ uint64_t sm64(uint64_t x) {
  uint64_t z = x + 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__device__ __forceinline__ double u01d(uint64_t x) { return (double)(sm64(x) >> 11) * (1.0 / 9007199254740992.0); }

struct JcState {
  double ratio, eps_p, rate, T;
};

// rate x thermal factor of the JC law (the rate clamp of Material.cuh:277-279)
__device__ __forceinline__ double jc_rt(const MatParams& M, double rate, double T, double* Th_out) {
  double Th = (T - M.Tt) / (M.Tm - M.Tt);
  Th = Th < 0.0 ? 0.0 : (Th > 0.999 ? 0.999 : Th);
  *Th_out = Th;
  const double sr = rate == 0.0 ? 1.e-5 : rate;
  return (1.0 + M.C * log(sr / M.eps0)) * (1.0 - pow(Th, M.m));
}

// ratio U[1,3], eps_p log-U[1e-4,2], rate log-U[1e-2,1e5] /s, T U[20,550] C
__global__ void k_mlp_synth(StepParams P, double G, int64_t n, uint64_t seed, float4* __restrict__ X,
                            float* __restrict__ Y, float4* __restrict__ S, int32_t* __restrict__ iters) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint64_t base = seed * 0x100000001B3ull + (uint64_t)i * 4ull;
  JcState s;
  s.ratio = 1.0 + 2.0 * u01d(base);
  s.eps_p = 1.0e-4 * pow(2.0e4, u01d(base + 1));
  s.rate = 1.0e-2 * pow(1.0e7, u01d(base + 2));
  s.T = 20.0 + 530.0 * u01d(base + 3);
  double Th;
  const double RT = jc_rt(P.mat, s.rate, s.T, &Th);
  double pwn = pow(s.eps_p, P.mat.n);
  const double sy0 = (P.mat.A + P.mat.B * pwn) * RT;
  const double st = s.ratio * sy0;
  double dl, sy1;
  int it = 0;
  jc_return_cached(P, st, 3.0 * G, s.eps_p, pwn, RT, -1.0, &dl, &sy1, &it);
  const double hi = (st - sy0) / (3.0 * G);
  float f[4];
  mlp_features((float)s.ratio, s.eps_p, (float)s.rate, (float)Th, f);
  X[i] = make_float4(f[0], f[1], f[2], f[3]);
  Y[i] = (float)(dl / hi);
  S[i] = make_float4((float)s.ratio, (float)s.eps_p, (float)s.rate, (float)s.T);
  iters[i] = it;
}

// Newton iterations from the radial start (image == nullptr) or the network's start
__global__ void __launch_bounds__(128) k_mlp_newton_iters(StepParams P, double G,
                                                          const uint4* __restrict__ image,
                                                          const MlpL1 l1,
                                                          const float4* __restrict__ S, int64_t n,
                                                          int32_t* __restrict__ iters,
                                                          int32_t* __restrict__ used,
                                                          float* __restrict__ dl_out, int* status) {
  extern __shared__ __align__(1024) uint8_t smu[];
  mlp_umma_begin(smu, image);
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const bool valid = i < n;
  const float4 s = valid ? S[i] : make_float4(1.f, 1e-2f, 1.f, 20.f);
  double Th;
  const double RT = jc_rt(P.mat, (double)s.z, (double)s.w, &Th);
  double pwn = pow((double)s.y, P.mat.n);
  const double sy0 = (P.mat.A + P.mat.B * pwn) * RT;
  const double st = (double)s.x * sy0;
  double ratio = -1.0;
  int use = 0;
  if (image) {
    float f[4];
    mlp_features(s.x, (double)s.y, s.z, (float)Th, f);
    const float y = mlp_umma_cta(smu, image, f, valid, status, l1);
    const float yc = mlp_accept(y);
    if (yc > 0.0f) { ratio = (double)yc; use = 1; }
  }
  if (!valid) return;
  double dl, sy1;
  int it = 0;
  jc_return_cached(P, st, 3.0 * G, (double)s.y, pwn, RT, ratio, &dl, &sy1, &it);
  iters[i] = it;
  used[i] = use;
  dl_out[i] = (float)dl;
}

// ---- training: loss and gradient of the mean squared error -------------------
// Block of 128 threads = 128 samples.  Shared memory: the parameters, the
// layer-1 pre-activations and activations, and the layer-2 gradients of the
// block's samples; weight gradients are reduced over the block's samples from
// shared memory and added to the global gradient once per block.
constexpr int TB = 128;
constexpr int LD = WF_MLP_H + 1;

__global__ void __launch_bounds__(TB) k_mlp_grad(const float* __restrict__ P,
                                                 const float4* __restrict__ X,
                                                 const float* __restrict__ Yt, int64_t n,
                                                 int64_t offset, int64_t count, float inv_total,
                                                 float* __restrict__ grad, float* __restrict__ loss) {
  extern __shared__ float sm[];
  float* Ps = sm;                                  // WF_MLP_NPARAM
  float* Z1 = Ps + ((WF_MLP_NPARAM + 3) & ~3);     // TB x LD
  float* H1 = Z1 + TB * LD;                        // TB x LD
  float* G2 = H1 + TB * LD;                        // TB x LD
  float* Xs = G2 + TB * LD;                        // TB x 4
  float* red = Xs + TB * 4;                        // 2 x WF_MLP_H + 2
  for (int k = threadIdx.x; k < WF_MLP_NPARAM; k += TB) Ps[k] = P[k];
  for (int k = threadIdx.x; k < 2 * WF_MLP_H + 2; k += TB) red[k] = 0.0f;
  __syncthreads();
  const float* W1 = Ps + WF_MLP_OFF_W1;
  const float* b1 = Ps + WF_MLP_OFF_B1;
  const float* W2 = Ps + WF_MLP_OFF_W2;
  const float* b2 = Ps + WF_MLP_OFF_B2;
  const float* w3 = Ps + WF_MLP_OFF_W3;
  const int s = threadIdx.x;
  const int64_t gi = offset + (int64_t)blockIdx.x * TB + s;
  const int nvalid = (int)min((int64_t)TB, count - (int64_t)blockIdx.x * TB);
  const bool valid = s < nvalid && gi < n;
  float* z1 = Z1 + s * LD;
  float* h1 = H1 + s * LD;
  float* g2 = G2 + s * LD;
  if (valid) {
    const float4 x4 = X[gi];
    const float x[4] = {x4.x, x4.y, x4.z, x4.w};
    Xs[s * 4 + 0] = x[0]; Xs[s * 4 + 1] = x[1]; Xs[s * 4 + 2] = x[2]; Xs[s * 4 + 3] = x[3];
    for (int o = 0; o < WF_MLP_H; o++) {
      float z = b1[o];
      for (int k = 0; k < 4; k++) z += W1[o * 4 + k] * x[k];
      z1[o] = z;
      h1[o] = z / (1.0f + expf(-z));
    }
    float y = Ps[WF_MLP_OFF_B3];
    for (int o = 0; o < WF_MLP_H; o++) {
      float z = b2[o];
      for (int k = 0; k < WF_MLP_H; k++) z += W2[o * WF_MLP_H + k] * h1[k];
      g2[o] = z;                                   // z2 for now
      y += w3[o] * (z / (1.0f + expf(-z)));
    }
    const float e = y - Yt[gi];
    atomicAdd(loss, e * e * inv_total);
    const float gy = 2.0f * e * inv_total;
    atomicAdd(red + 2 * WF_MLP_H, gy);             // gb3
    for (int o = 0; o < WF_MLP_H; o++) {
      const float z = g2[o];
      const float sg = 1.0f / (1.0f + expf(-z));
      atomicAdd(red + o, gy * z * sg);             // gW3
      g2[o] = gy * w3[o] * sg * (1.0f + z * (1.0f - sg));
    }
  } else {
    for (int o = 0; o < WF_MLP_H; o++) { z1[o] = 0.f; h1[o] = 0.f; g2[o] = 0.f; }
    Xs[s * 4 + 0] = Xs[s * 4 + 1] = Xs[s * 4 + 2] = Xs[s * 4 + 3] = 0.f;
  }
  __syncthreads();
  // gW2[o][k] = sum_s g2[s][o] h1[s][k]; gb2[o] = sum_s g2[s][o]
  for (int e = s; e < WF_MLP_H * WF_MLP_H; e += TB) {
    const int o = e / WF_MLP_H, k = e % WF_MLP_H;
    float acc = 0.0f;
    for (int q = 0; q < TB; q++) acc += G2[q * LD + o] * H1[q * LD + k];
    atomicAdd(grad + WF_MLP_OFF_W2 + e, acc);
  }
  if (s < WF_MLP_H) {
    float acc = 0.0f;
    for (int q = 0; q < TB; q++) acc += G2[q * LD + s];
    atomicAdd(grad + WF_MLP_OFF_B2 + s, acc);
    atomicAdd(grad + WF_MLP_OFF_W3 + s, red[s]);
  }
  if (s == 0) atomicAdd(grad + WF_MLP_OFF_B3, red[2 * WF_MLP_H]);
  // g1 = (W2^T g2) * silu'(z1), into z1
  float g1[WF_MLP_H];
  for (int k = 0; k < WF_MLP_H; k++) {
    float acc = 0.0f;
    for (int o = 0; o < WF_MLP_H; o++) acc += W2[o * WF_MLP_H + k] * g2[o];
    const float z = z1[k];
    const float sg = 1.0f / (1.0f + expf(-z));
    g1[k] = acc * sg * (1.0f + z * (1.0f - sg));
  }
  __syncthreads();
  for (int k = 0; k < WF_MLP_H; k++) z1[k] = g1[k];
  __syncthreads();
  // gW1[o][k] = sum_s g1[s][o] x[s][k]; gb1[o] = sum_s g1[s][o]
  for (int e = s; e < WF_MLP_H * 4; e += TB) {
    const int o = e / 4, k = e % 4;
    float acc = 0.0f;
    for (int q = 0; q < TB; q++) acc += Z1[q * LD + o] * Xs[q * 4 + k];
    atomicAdd(grad + WF_MLP_OFF_W1 + e, acc);
  }
  if (s < WF_MLP_H) {
    float acc = 0.0f;
    for (int q = 0; q < TB; q++) acc += Z1[q * LD + s];
    atomicAdd(grad + WF_MLP_OFF_B1 + s, acc);
  }
}

__global__ void k_adam(float* __restrict__ P, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, int np, float lr, float b1, float b2, float eps,
                       float c1, float c2) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= np) return;
  const float gk = g[k];
  const float mk = b1 * m[k] + (1.0f - b1) * gk;
  const float vk = b2 * v[k] + (1.0f - b2) * gk * gk;
  m[k] = mk;
  v[k] = vk;
  P[k] -= lr * (mk / c1) / (sqrtf(vk / c2) + eps);
}

size_t grad_smem_bytes() {
  return sizeof(float) * (((WF_MLP_NPARAM + 3) & ~3) + 3 * TB * LD + TB * 4 + 2 * WF_MLP_H + 2);
}

StepParams jc_params(const wf_material* m, double rtol) {
  StepParams P;
  memset(&P, 0, sizeof P);
  P.newton_max_iter = 200;
  P.newton_rtol = rtol;
  P.clamp_homologous = 1;
  MatParams& M = P.mat;
  M.model = m->model;
  M.E = m->E;
  M.A = m->A; M.B = m->B; M.n = m->n; M.C = m->C; M.eps0 = m->eps0; M.m = m->m;
  M.Tm = m->Tm; M.Tt = m->Tt;
  double c = 1.0;
  for (int k = 1; k <= 5; k++) {
    c = c * (m->n - (k - 1)) / k;
    M.bin[k - 1] = c;
  }
  return P;
}

// RAII device buffers for the standalone entry points
struct DevBufs {
  std::vector<void*> ptrs;
  ~DevBufs() {
    for (void* p : ptrs) cudaFree(p);
  }
  template <class T>
  T* get(size_t count) {
    void* p = nullptr;
    if (cudaMalloc(&p, sizeof(T) * (count ? count : 1)) != cudaSuccess) return nullptr;
    ptrs.push_back(p);
    return (T*)p;
  }
};

inline int nb(int64_t n, int t) { return (int)((n + t - 1) / t); }

}  // namespace

// packs FP32 parameters into the BF16 fragment image used by the kernels
int wf_mlp_pack_device(const float* dparams, void* dpacked, cudaStream_t s) {
  k_mlp_pack_umma<<<1, 256, 0, s>>>(dparams, (uint8_t*)dpacked);
  return cudaGetLastError() == cudaSuccess ? WF_OK : WF_ERR_CUDA;
}
size_t wf_mlp_packed_bytes() { return WF_UMMA_IMAGE; }

extern "C" {

int wf_mlp_infer(const float* params, const float* X, int64_t n, int use_tensor_cores, float* Y) {
  if (!params || !X || !Y || n <= 0) return WF_ERR_ARG;
  DevBufs B;
  float* dP = B.get<float>(WF_MLP_NPARAM);
  float4* dX = B.get<float4>(n);
  float* dY = B.get<float>(n);
  if (!dP || !dX || !dY) return WF_ERR_ALLOC;
  cudaMemcpy(dP, params, sizeof(float) * WF_MLP_NPARAM, cudaMemcpyHostToDevice);
  cudaMemcpy(dX, X, sizeof(float) * 4 * n, cudaMemcpyHostToDevice);
  if (use_tensor_cores) {
    uint4* dI = B.get<uint4>(WF_UMMA_IMAGE / 16);
    int* dS = B.get<int>(1);
    if (!dI || !dS) return WF_ERR_ALLOC;
    cudaMemset(dS, 0, sizeof(int));
    k_mlp_pack_umma<<<1, 256>>>(dP, (uint8_t*)dI);
    k_mlp_infer_umma<<<nb(n, 128), 128, WF_UMMA_SMEM>>>(dI, mlp_l1_from(params), dX, n, dY, dS);
    int st = 0;
    cudaMemcpy(&st, dS, sizeof(int), cudaMemcpyDeviceToHost);
    if (st & WF_STATUS_MMA_WAIT) return WF_ERR_CUDA;
  } else {
    k_mlp_infer_f32<<<nb(n, 128), 128>>>(dP, dX, n, dY);
  }
  if (cudaMemcpy(Y, dY, sizeof(float) * n, cudaMemcpyDeviceToHost) != cudaSuccess) return WF_ERR_CUDA;
  return cudaGetLastError() == cudaSuccess ? WF_OK : WF_ERR_CUDA;
}

int wf_mlp_grad(const float* params, const float* X, const float* Y, int64_t n, float* grad,
                float* loss) {
  if (!params || !X || !Y || !grad || !loss || n <= 0) return WF_ERR_ARG;
  DevBufs B;
  float* dP = B.get<float>(WF_MLP_NPARAM);
  float4* dX = B.get<float4>(n);
  float* dY = B.get<float>(n);
  float* dG = B.get<float>(WF_MLP_NPARAM);
  float* dL = B.get<float>(1);
  if (!dP || !dX || !dY || !dG || !dL) return WF_ERR_ALLOC;
  cudaMemcpy(dP, params, sizeof(float) * WF_MLP_NPARAM, cudaMemcpyHostToDevice);
  cudaMemcpy(dX, X, sizeof(float) * 4 * n, cudaMemcpyHostToDevice);
  cudaMemcpy(dY, Y, sizeof(float) * n, cudaMemcpyHostToDevice);
  cudaMemset(dG, 0, sizeof(float) * WF_MLP_NPARAM);
  cudaMemset(dL, 0, sizeof(float));
  const size_t smem = grad_smem_bytes();
  cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  k_mlp_grad<<<nb(n, TB), TB, smem>>>(dP, dX, dY, n, 0, n, 1.0f / (float)n, dG, dL);
  cudaMemcpy(grad, dG, sizeof(float) * WF_MLP_NPARAM, cudaMemcpyDeviceToHost);
  if (cudaMemcpy(loss, dL, sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess) return WF_ERR_CUDA;
  return cudaGetLastError() == cudaSuccess ? WF_OK : WF_ERR_CUDA;
}

int wf_mlp_train(float* params, const float* X, const float* Y, int64_t n, int64_t steps,
                 int64_t batch, float lr, float* final_loss) {
  if (!params || !X || !Y || n <= 0 || steps <= 0 || batch <= 0) return WF_ERR_ARG;
  DevBufs B;
  float* dP = B.get<float>(WF_MLP_NPARAM);
  float4* dX = B.get<float4>(n);
  float* dY = B.get<float>(n);
  float* dG = B.get<float>(WF_MLP_NPARAM);
  float* dM = B.get<float>(WF_MLP_NPARAM);
  float* dV = B.get<float>(WF_MLP_NPARAM);
  float* dL = B.get<float>(steps);
  if (!dP || !dX || !dY || !dG || !dM || !dV || !dL) return WF_ERR_ALLOC;
  cudaMemcpy(dP, params, sizeof(float) * WF_MLP_NPARAM, cudaMemcpyHostToDevice);
  cudaMemcpy(dX, X, sizeof(float) * 4 * n, cudaMemcpyHostToDevice);
  cudaMemcpy(dY, Y, sizeof(float) * n, cudaMemcpyHostToDevice);
  cudaMemset(dM, 0, sizeof(float) * WF_MLP_NPARAM);
  cudaMemset(dV, 0, sizeof(float) * WF_MLP_NPARAM);
  cudaMemset(dL, 0, sizeof(float) * steps);
  const size_t smem = grad_smem_bytes();
  cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  const float b1 = 0.9f, b2 = 0.999f;
  double p1 = 1.0, p2 = 1.0;
  int64_t off = 0;
  for (int64_t st = 0; st < steps; st++) {
    const int64_t cnt = std::min<int64_t>(batch, n - off);
    cudaMemsetAsync(dG, 0, sizeof(float) * WF_MLP_NPARAM);
    k_mlp_grad<<<nb(cnt, TB), TB, smem>>>(dP, dX, dY, n, off, cnt, 1.0f / (float)cnt, dG, dL + st);
    p1 *= b1;
    p2 *= b2;
    // cosine decay of the learning rate
    const float lr_t = lr * 0.5f * (1.0f + cosf(3.14159265f * (float)st / (float)steps));
    k_adam<<<nb(WF_MLP_NPARAM, 256), 256>>>(dP, dG, dM, dV, WF_MLP_NPARAM, lr_t, b1, b2, 1e-8f,
                                            (float)(1.0 - p1), (float)(1.0 - p2));
    off += cnt;
    if (off >= n) off = 0;
  }
  cudaMemcpy(params, dP, sizeof(float) * WF_MLP_NPARAM, cudaMemcpyDeviceToHost);
  if (final_loss) {
    std::vector<float> L(steps);
    cudaMemcpy(L.data(), dL, sizeof(float) * steps, cudaMemcpyDeviceToHost);
    const int64_t k0 = std::max<int64_t>(0, steps - 20);
    double acc = 0.0;
    for (int64_t k = k0; k < steps; k++) acc += L[k];
    *final_loss = (float)(acc / (double)(steps - k0));
  }
  return cudaGetLastError() == cudaSuccess ? WF_OK : WF_ERR_CUDA;
}

int wf_mlp_synth(const wf_material* mat, double G, int64_t n, uint64_t seed, double rtol,
                 float* X, float* Y, float* states, int32_t* iters_radial) {
  if (!mat || !X || !Y || !states || !iters_radial || n <= 0) return WF_ERR_ARG;
  if (mat->model != WF_JOHNSON_COOK) return WF_ERR_ARG;
  DevBufs B;
  float4* dX = B.get<float4>(n);
  float* dY = B.get<float>(n);
  float4* dS = B.get<float4>(n);
  int32_t* dI = B.get<int32_t>(n);
  if (!dX || !dY || !dS || !dI) return WF_ERR_ALLOC;
  StepParams P = jc_params(mat, rtol);
  k_mlp_synth<<<nb(n, 128), 128>>>(P, G, n, seed, dX, dY, dS, dI);
  cudaMemcpy(X, dX, sizeof(float) * 4 * n, cudaMemcpyDeviceToHost);
  cudaMemcpy(Y, dY, sizeof(float) * n, cudaMemcpyDeviceToHost);
  cudaMemcpy(states, dS, sizeof(float) * 4 * n, cudaMemcpyDeviceToHost);
  if (cudaMemcpy(iters_radial, dI, sizeof(int32_t) * n, cudaMemcpyDeviceToHost) != cudaSuccess)
    return WF_ERR_CUDA;
  return cudaGetLastError() == cudaSuccess ? WF_OK : WF_ERR_CUDA;
}

int wf_mlp_newton_iters(const wf_material* mat, double G, const float* params, const float* states,
                        int64_t n, double rtol, int32_t* iters, int32_t* used, float* dl) {
  if (!mat || !states || !iters || !used || !dl || n <= 0) return WF_ERR_ARG;
  DevBufs B;
  float4* dS = B.get<float4>(n);
  int32_t* dI = B.get<int32_t>(n);
  int32_t* dU = B.get<int32_t>(n);
  float* dD = B.get<float>(n);
  float* dP = B.get<float>(WF_MLP_NPARAM);
  uint4* dW = B.get<uint4>(WF_UMMA_IMAGE / 16);
  int* dSt = B.get<int>(1);
  if (!dS || !dI || !dU || !dD || !dP || !dW || !dSt) return WF_ERR_ALLOC;
  cudaMemcpy(dS, states, sizeof(float) * 4 * n, cudaMemcpyHostToDevice);
  cudaMemset(dSt, 0, sizeof(int));
  if (params) {
    cudaMemcpy(dP, params, sizeof(float) * WF_MLP_NPARAM, cudaMemcpyHostToDevice);
    k_mlp_pack_umma<<<1, 256>>>(dP, (uint8_t*)dW);
  }
  StepParams P = jc_params(mat, rtol);
  const MlpL1 l1 = params ? mlp_l1_from(params) : MlpL1{};
  k_mlp_newton_iters<<<nb(n, 128), 128, params ? WF_UMMA_SMEM : 0>>>(
      P, G, params ? dW : nullptr, l1, dS, n, dI, dU, dD, dSt);
  cudaMemcpy(iters, dI, sizeof(int32_t) * n, cudaMemcpyDeviceToHost);
  cudaMemcpy(used, dU, sizeof(int32_t) * n, cudaMemcpyDeviceToHost);
  if (cudaMemcpy(dl, dD, sizeof(float) * n, cudaMemcpyDeviceToHost) != cudaSuccess) return WF_ERR_CUDA;
  int st = 0;
  cudaMemcpy(&st, dSt, sizeof(int), cudaMemcpyDeviceToHost);
  if (st & WF_STATUS_MMA_WAIT) return WF_ERR_CUDA;
  return cudaGetLastError() == cudaSuccess ? WF_OK : WF_ERR_CUDA;
}

}  // extern "C"

static_assert(WF_MLP_NPARAM == WF_MLP_NPARAMS, "MLP parameter count mismatch between header and kernels");
