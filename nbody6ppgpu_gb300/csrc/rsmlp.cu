// Learned neighbour-radius predictor: an 8 -> 64 -> 64 -> 1 MLP with GELU,
// BF16 weight matrices, FP32 biases, activations and accumulation.
//
// No reference counterpart: the reference adjusts RS by a fixed rule after
// every regular step (src/Main/regcor_gpu.F:146-253) and shrinks it after a
// neighbour-list overflow (src/Main/util_gpu.F:81-97).  The predictor only
// proposes RS; forces are never computed here.
//
// Parameter vector (P = 4801 entries, same order in FP32 and BF16 copies):
//   W1[64][8] | b1[64] | W2[64][64] | b2[64] | W3[64] | b3
// The kernels read the weight matrices from the BF16 copy and the biases
// from the FP32 copy.  Samples are rows of X[B][8] (normalised features).
//
// Kernels use CUDA cores: a 64-wide layer is far below the size at which the
// tensor-core pipeline (TMEM allocation, descriptors, 128-wide tiles) pays
// off; one sample per thread with the weights broadcast from shared memory
// runs a 2^20-sample inference in well under a millisecond.
#include <cuda_bf16.h>

#include "common.cuh"
#include "rsrule.cuh"

namespace gpunb {

constexpr int MLP_IN = 8, MLP_H = 64;
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + MLP_H * MLP_IN, OFF_W2 = OFF_B1 + MLP_H,
              OFF_B2 = OFF_W2 + MLP_H * MLP_H, OFF_W3 = OFF_B2 + MLP_H, OFF_B3 = OFF_W3 + MLP_H,
              MLP_P = OFF_B3 + 1;
constexpr int MLP_THREADS = 128;

__device__ __forceinline__ float gelu(float x) {
  return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f));
}
__device__ __forceinline__ float gelu_grad(float x) {
  // d/dx [x Phi(x)] = Phi(x) + x phi(x)
  return 0.5f * (1.0f + erff(x * 0.70710678118654752f)) +
         x * 0.3989422804014327f * expf(-0.5f * x * x);
}

// weights (as float) and biases staged in shared memory
struct MlpSmem {
  float w1[MLP_H * MLP_IN];
  float b1[MLP_H];
  float w2[MLP_H * MLP_H];
  float b2[MLP_H];
  float w3[MLP_H];
  float b3;
};

__device__ void stage_params(MlpSmem &s, const __nv_bfloat16 *__restrict__ wq,
                             const float *__restrict__ wf) {
  for (int k = threadIdx.x; k < MLP_H * MLP_IN; k += blockDim.x)
    s.w1[k] = __bfloat162float(wq[OFF_W1 + k]);
  for (int k = threadIdx.x; k < MLP_H * MLP_H; k += blockDim.x)
    s.w2[k] = __bfloat162float(wq[OFF_W2 + k]);
  for (int k = threadIdx.x; k < MLP_H; k += blockDim.x) {
    s.w3[k] = __bfloat162float(wq[OFF_W3 + k]);
    s.b1[k] = wf[OFF_B1 + k];
    s.b2[k] = wf[OFF_B2 + k];
  }
  if (threadIdx.x == 0) s.b3 = wf[OFF_B3];
  __syncthreads();
}

__device__ __forceinline__ float mlp_eval(const MlpSmem &s, const float (&x)[MLP_IN]) {
  float h1[MLP_H];
#pragma unroll
  for (int o = 0; o < MLP_H; ++o) {
    float a = s.b1[o];
#pragma unroll
    for (int f = 0; f < MLP_IN; ++f) a = fmaf(s.w1[o * MLP_IN + f], x[f], a);
    h1[o] = gelu(a);
  }
  float out = s.b3;
  for (int o = 0; o < MLP_H; ++o) {
    float a = s.b2[o];
#pragma unroll
    for (int k = 0; k < MLP_H; ++k) a = fmaf(s.w2[o * MLP_H + k], h1[k], a);
    out = fmaf(s.w3[o], gelu(a), out);
  }
  return out;
}

__global__ void __launch_bounds__(MLP_THREADS)
    rsmlp_forward_kernel(int B, const float *__restrict__ X, const __nv_bfloat16 *__restrict__ wq,
                         const float *__restrict__ wf, float *__restrict__ y) {
  __shared__ MlpSmem s;
  stage_params(s, wq, wf);
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  float x[MLP_IN];
#pragma unroll
  for (int f = 0; f < MLP_IN; ++f) x[f] = X[(size_t)b * MLP_IN + f];
  y[b] = mlp_eval(s, x);
}

// ---------------------------------------------------------------------------
// RS update of an active block on the device: the plain rule of
// src/Main/regcor_gpu.F:120-253 (NNBOPT stabilisation, NBAVE cap, taper,
// inertial and radial-velocity factors, RSFAC limit, second-order cube root,
// shell square root, inward reduction; the zero-neighbour branch :120-143),
// optionally the few-member rule of fpoly0.F:153-158, and -- with weights --
// the learned proposal: features, MLP, and the plain rule as fallback when the
// count it implies at the current density leaves the band (default 0.5-1.5 x
// the rule's target).
__global__ void __launch_bounds__(MLP_THREADS)
    rs_update_kernel(int ni, gpunb_rs_params p, const double *__restrict__ x,
                     const double *__restrict__ v, const double *__restrict__ m_scaled,
                     const double *__restrict__ rs, const int *__restrict__ nnb,
                     const int *__restrict__ nnb0, const double *__restrict__ acc,
                     const double *__restrict__ jrk, const double *__restrict__ dtr,
                     const __nv_bfloat16 *__restrict__ wq, const float *__restrict__ wf,
                     const float *__restrict__ norm, double *__restrict__ rs_new,
                     double *__restrict__ target, int *__restrict__ used) {
  __shared__ MlpSmem s;
  if (wq) stage_params(s, wq, wf);
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ni) return;
  const double *xi = x + 3 * (size_t)i, *vi = v + 3 * (size_t)i;
  const int n = nnb[i];
  const double r0 = rs[i];
  double plain, tgt;
  rs_plain(p, r0, n, nnb0[i], xi, vi, dtr[i], -1.0, plain, tgt);
  if (p.few_nb_rule && n < 2) plain = 1.5 * r0;
  double nw = plain;
  int u = 0;
  if (wq) {
    // features (rsmlp.py): log distance to the centre, log local density,
    // count / NNBOPT, log |F_reg|, log |jerk|, log regular step, log mass N,
    // log RS; normalised with the training set's mean and spread
    const double e0 = xi[0] - p.rdens[0], e1 = xi[1] - p.rdens[1], e2 = xi[2] - p.rdens[2];
    const double nn = (double)max(n, 0);
    const double *a = acc + 3 * (size_t)i, *j = jrk + 3 * (size_t)i;
    const double f[MLP_IN] = {
        log(sqrt(e0 * e0 + e1 * e1 + e2 * e2) + 1e-6),
        log((nn + 1.0) / (4.0 / 3.0 * 3.141592653589793 * r0 * r0 * r0)),
        nn / (double)p.nnbopt,
        log(sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]) + 1e-30),
        log(sqrt(j[0] * j[0] + j[1] * j[1] + j[2] * j[2]) + 1e-30),
        log(fmax(dtr[i], 1e-12)),
        log(fmax(m_scaled[i], 1e-12)),
        log(r0)};
    float xf[MLP_IN];
#pragma unroll
    for (int q = 0; q < MLP_IN; ++q)
      xf[q] = (float)((f[q] - (double)norm[q]) / (double)norm[MLP_IN + q]);
    const float y = mlp_eval(s, xf);
    const double pc = (nn + 1.0) * exp(3.0 * (double)y) - 1.0;
    const double blo = p.band_lo > 0.0 ? p.band_lo : 0.5;
    const double bhi = p.band_hi > 0.0 ? p.band_hi : 1.5;
    if (isfinite(y) && pc >= blo * tgt && pc <= bhi * tgt) {
      nw = r0 * exp((double)y);
      u = 1;
    }
  }
  rs_new[i] = nw;
  if (target) target[i] = tgt;
  if (used) used[i] = u;
}

// Backward pass of the mean of w_b (y_b - t_b)^2 over the batch.  Each block
// writes the gradient summed over its samples to part[blockIdx][P]; a second
// kernel sums the block rows in order (deterministic).  Per-sample
// activations live in dynamic shared memory (rows padded to 65 floats):
//   sx[T][8], sh1[T][65] h1, sd1[T][65] z1 then dz1, sd2[T][65] z2 then dz2,
//   sh2[T][65] h2.
constexpr int LD = MLP_H + 1;
size_t rsmlp_backward_smem() {
  return sizeof(float) * ((size_t)MLP_THREADS * MLP_IN + 4ull * MLP_THREADS * LD + MLP_THREADS);
}

__global__ void __launch_bounds__(MLP_THREADS)
    rsmlp_backward_kernel(int B, const float *__restrict__ X, const float *__restrict__ T,
                          const float *__restrict__ Wt, const __nv_bfloat16 *__restrict__ wq,
                          const float *__restrict__ wf, float inv_norm,
                          float *__restrict__ part, float *__restrict__ loss_part) {
  __shared__ MlpSmem s;
  extern __shared__ float dyn[];
  float *sx = dyn;
  float *sh1 = sx + MLP_THREADS * MLP_IN;
  float *sd1 = sh1 + MLP_THREADS * LD;
  float *sd2 = sd1 + MLP_THREADS * LD;
  float *sh2 = sd2 + MLP_THREADS * LD;
  float *sdy = sh2 + MLP_THREADS * LD;
  __shared__ float sh_red[MLP_THREADS];
  stage_params(s, wq, wf);
  const int t = threadIdx.x;
  const int b = blockIdx.x * blockDim.x + t;
  const bool valid = b < B;
#pragma unroll
  for (int f = 0; f < MLP_IN; ++f) sx[t * MLP_IN + f] = valid ? X[(size_t)b * MLP_IN + f] : 0.f;
  // layer 1
  for (int o = 0; o < MLP_H; ++o) {
    float a = s.b1[o];
#pragma unroll
    for (int f = 0; f < MLP_IN; ++f) a = fmaf(s.w1[o * MLP_IN + f], sx[t * MLP_IN + f], a);
    sd1[t * LD + o] = a;
    sh1[t * LD + o] = gelu(a);
  }
  // layer 2 and output
  float out = s.b3;
  for (int o = 0; o < MLP_H; ++o) {
    float a = s.b2[o];
    for (int k = 0; k < MLP_H; ++k) a = fmaf(s.w2[o * MLP_H + k], sh1[t * LD + k], a);
    const float h2 = gelu(a);
    sd2[t * LD + o] = a;
    sh2[t * LD + o] = h2;
    out = fmaf(s.w3[o], h2, out);
  }
  const float w = valid ? (Wt ? Wt[b] : 1.0f) : 0.f;
  const float r = valid ? out - T[b] : 0.f;
  const float dy = 2.0f * w * r * inv_norm;
  sdy[t] = dy;
  sh_red[t] = w * r * r * inv_norm;
  // dz2 = dy W3 gelu'(z2)
  for (int o = 0; o < MLP_H; ++o) sd2[t * LD + o] = dy * s.w3[o] * gelu_grad(sd2[t * LD + o]);
  // dz1 = (W2^T dz2) gelu'(z1)
  for (int k = 0; k < MLP_H; ++k) {
    float a = 0.f;
    for (int o = 0; o < MLP_H; ++o) a = fmaf(s.w2[o * MLP_H + k], sd2[t * LD + o], a);
    sd1[t * LD + k] = a * gelu_grad(sd1[t * LD + k]);
  }
  __syncthreads();
  // block sums over the samples, each output by one thread in sample order
  float *pb = part + (size_t)blockIdx.x * MLP_P;
  for (int e = t; e < MLP_H * MLP_H; e += MLP_THREADS) {     // dW2[o][k]
    const int o = e / MLP_H, k = e % MLP_H;
    float a = 0.f;
    for (int u = 0; u < MLP_THREADS; ++u) a = fmaf(sd2[u * LD + o], sh1[u * LD + k], a);
    pb[OFF_W2 + e] = a;
  }
  for (int e = t; e < MLP_H * MLP_IN; e += MLP_THREADS) {    // dW1[k][f]
    const int k = e / MLP_IN, f = e % MLP_IN;
    float a = 0.f;
    for (int u = 0; u < MLP_THREADS; ++u) a = fmaf(sd1[u * LD + k], sx[u * MLP_IN + f], a);
    pb[OFF_W1 + e] = a;
  }
  if (t < MLP_H) {                                           // dW3, db2, db1
    float a = 0.f, c = 0.f, d = 0.f;
    for (int u = 0; u < MLP_THREADS; ++u) {
      a = fmaf(sdy[u], sh2[u * LD + t], a);
      c += sd2[u * LD + t];
      d += sd1[u * LD + t];
    }
    pb[OFF_W3 + t] = a;
    pb[OFF_B2 + t] = c;
    pb[OFF_B1 + t] = d;
  } else if (t == MLP_H) {                                   // db3
    float a = 0.f;
    for (int u = 0; u < MLP_THREADS; ++u) a += sdy[u];
    pb[OFF_B3] = a;
  } else if (t == MLP_H + 1) {                               // loss
    float a = 0.f;
    for (int u = 0; u < MLP_THREADS; ++u) a += sh_red[u];
    loss_part[blockIdx.x] = a;
  }
}

// grad[p] = sum over blocks (in order) of part[block][p]; loss likewise
__global__ void rsmlp_reduce_kernel(int nblocks, const float *__restrict__ part,
                                    const float *__restrict__ loss_part, float *__restrict__ grad,
                                    float *__restrict__ loss) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < MLP_P) {
    double a = 0.0;
    for (int k = 0; k < nblocks; ++k) a += part[(size_t)k * MLP_P + p];
    grad[p] = (float)a;
  }
  if (p == 0 && loss) {
    double a = 0.0;
    for (int k = 0; k < nblocks; ++k) a += loss_part[k];
    *loss = (float)a;
  }
}

// Adam on the FP32 master copy, then refresh the BF16 copy.
__global__ void rsmlp_adam_kernel(float *__restrict__ wf, float *__restrict__ m1,
                                  float *__restrict__ m2, const float *__restrict__ grad,
                                  float lr, float beta1, float beta2, float eps, float bc1,
                                  float bc2, __nv_bfloat16 *__restrict__ wq) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= MLP_P) return;
  const float gr = grad[p];
  const float a = beta1 * m1[p] + (1.f - beta1) * gr;
  const float b = beta2 * m2[p] + (1.f - beta2) * gr * gr;
  m1[p] = a;
  m2[p] = b;
  const float w = wf[p] - lr * (a / bc1) / (sqrtf(b / bc2) + eps);
  wf[p] = w;
  wq[p] = __float2bfloat16_rn(w);
}

__global__ void rsmlp_to_bf16_kernel(const float *__restrict__ wf, __nv_bfloat16 *__restrict__ wq) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < MLP_P) wq[p] = __float2bfloat16_rn(wf[p]);
}

}  // namespace gpunb

using namespace gpunb;

extern "C" {

int gpunb_rsmlp_num_params(void) { return MLP_P; }

int gpunb_rsmlp_to_bf16(const float *wf, void *wq, void *stream) {
  rsmlp_to_bf16_kernel<<<(MLP_P + 255) / 256, 256, 0, (cudaStream_t)stream>>>(
      wf, (__nv_bfloat16 *)wq);
  return cudaGetLastError() == cudaSuccess ? GPUNB_OK : GPUNB_E_CUDA;
}

int gpunb_rsmlp_forward(int B, const float *X, const void *wq, const float *wf, float *y,
                        void *stream) {
  if (B <= 0) return B == 0 ? GPUNB_OK : GPUNB_E_ARG;
  rsmlp_forward_kernel<<<(B + MLP_THREADS - 1) / MLP_THREADS, MLP_THREADS, 0,
                         (cudaStream_t)stream>>>(B, X, (const __nv_bfloat16 *)wq, wf, y);
  return cudaGetLastError() == cudaSuccess ? GPUNB_OK : GPUNB_E_CUDA;
}

// part: scratch of ceil(B/128)*P floats + ceil(B/128) floats
int gpunb_rsmlp_backward(int B, const float *X, const float *T, const float *W, const void *wq,
                         const float *wf, float *grad, float *loss, float *part, void *stream) {
  if (B <= 0) return GPUNB_E_ARG;
  const int nb = (B + MLP_THREADS - 1) / MLP_THREADS;
  float *loss_part = part + (size_t)nb * MLP_P;
  cudaStream_t st = (cudaStream_t)stream;
  const size_t smem = rsmlp_backward_smem();
  if (cudaFuncSetAttribute(rsmlp_backward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem) != cudaSuccess)
    return GPUNB_E_CUDA;
  rsmlp_backward_kernel<<<nb, MLP_THREADS, smem, st>>>(B, X, T, W, (const __nv_bfloat16 *)wq, wf,
                                                       1.0f / (float)B, part, loss_part);
  rsmlp_reduce_kernel<<<(MLP_P + 255) / 256, 256, 0, st>>>(nb, part, loss_part, grad, loss);
  return cudaGetLastError() == cudaSuccess ? GPUNB_OK : GPUNB_E_CUDA;
}

int gpunb_rsmlp_adam(float *wf, float *m1, float *m2, const float *grad, float lr, float beta1,
                     float beta2, float eps, int step, void *wq, void *stream) {
  const float bc1 = 1.f - powf(beta1, (float)step), bc2 = 1.f - powf(beta2, (float)step);
  rsmlp_adam_kernel<<<(MLP_P + 255) / 256, 256, 0, (cudaStream_t)stream>>>(
      wf, m1, m2, grad, lr, beta1, beta2, eps, bc1, bc2, (__nv_bfloat16 *)wq);
  return cudaGetLastError() == cudaSuccess ? GPUNB_OK : GPUNB_E_CUDA;
}

int gpunb_rs_update_device(int ni, const gpunb_rs_params *p, const double *x, const double *v,
                           const double *m_scaled, const double *rs, const int *nnb,
                           const int *nnb0, const double *acc, const double *jrk,
                           const double *dtr, const void *wq, const float *wf,
                           const float *norm, double *rs_new, double *target, int *used,
                           void *stream) {
  if (ni < 0 || !p) return GPUNB_E_ARG;
  if (ni == 0) return GPUNB_OK;
  if (wq && (!wf || !norm || !acc || !jrk || !m_scaled)) return GPUNB_E_ARG;
  rs_update_kernel<<<(ni + MLP_THREADS - 1) / MLP_THREADS, MLP_THREADS, 0,
                     (cudaStream_t)stream>>>(ni, *p, x, v, m_scaled, rs, nnb, nnb0, acc, jrk, dtr,
                                             (const __nv_bfloat16 *)wq, wf, norm, rs_new, target,
                                             used);
  return cudaGetLastError() == cudaSuccess ? GPUNB_OK : GPUNB_E_CUDA;
}

}  // extern "C"
