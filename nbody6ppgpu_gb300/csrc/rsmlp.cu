// Learned neighbour-radius predictor: an 8 -> 64 -> 64 -> 1 MLP with GELU in
// its tanh form, BF16 weight matrices, FP32 biases and accumulation.
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
// Inference (gpunb_rsmlp_forward, and the fused RS update) and training
// (gpunb_rsmlp_backward) run their matrix products on the tensor cores
// (mma.sync BF16 tiles of 16 samples, FP32 accumulation).  Inference takes
// BF16 inputs and activations and the hardware tanh approximation; training
// carries inputs and activations as two-term BF16 splits and an accurate
// tanh, so that its gradients are those of FP32 arithmetic on the same
// weights.
#include <cuda_bf16.h>

#include <algorithm>
#include <atomic>

#include "common.cuh"
#include "rsrule.cuh"

namespace gpunb {

constexpr int MLP_IN = 8, MLP_H = 64;
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + MLP_H * MLP_IN, OFF_W2 = OFF_B1 + MLP_H,
              OFF_B2 = OFF_W2 + MLP_H * MLP_H, OFF_W3 = OFF_B2 + MLP_H, OFF_B3 = OFF_W3 + MLP_H,
              MLP_P = OFF_B3 + 1;
constexpr int MLP_THREADS = 128;

// GELU in its tanh form (Hendrycks and Gimpel, 2016):
//   gelu(x) = x/2 (1 + tanh(u)),  u = sqrt(2/pi) (x + 0.044715 x^3),
//   gelu'(x) = (1 + tanh u)/2 + x/2 (1 - tanh^2 u) sqrt(2/pi) (1 + 3 0.044715 x^2).
constexpr float GELU_C = 0.7978845608028654f;           // sqrt(2/pi)
constexpr float GELU_CA = 0.7978845608028654f * 0.044715f;
__device__ __forceinline__ float gelu_arg(float x) { return x * fmaf(GELU_CA, x * x, GELU_C); }
__device__ __forceinline__ float gelu(float x) {
  const float h = 0.5f * x;
  return fmaf(h, tanhf(gelu_arg(x)), h);
}
__device__ __forceinline__ float gelu_grad(float x) {
  const float t = tanhf(gelu_arg(x));
  return fmaf(0.5f, t, 0.5f) + 0.5f * x * fmaf(-t, t, 1.0f) * fmaf(3.0f * GELU_CA, x * x, GELU_C);
}
// inference: the tanh from the hardware approximation (relative error below
// 2^-10.9, under the BF16 rounding of the activations that follows), two
// activations at a time in packed FP32
__device__ __forceinline__ float tanh_fast(float u) {
  float t;
  asm("tanh.approx.f32 %0, %1;" : "=f"(t) : "f"(u));
  return t;
}
// of the pre-activations x = acc + b, from h = x / 2 = acc / 2 + b / 2 (the
// biases staged halved): u = h (2 sqrt(2/pi) + 8 sqrt(2/pi) 0.044715 h^2),
// gelu = h + h tanh(u)
__device__ __forceinline__ f2 gelu_fast2_half(f2 acc, f2 bhalf) {
  const f2 h = fma2(acc, mk2(0.5f), bhalf);
  const f2 u = mul2(h, fma2(mk2(8.0f * GELU_CA), mul2(h, h), mk2(2.0f * GELU_C)));
  return fma2(h, make_float2(tanh_fast(u.x), tanh_fast(u.y)), h);
}

// ---------------------------------------------------------------------------
// Tensor-core building blocks (mma.sync, BF16 operands, FP32 accumulation).
//
// The D fragments of one product (rows g, g+8 of a 16-sample tile, two
// adjacent hidden columns per n8 tile) are laid out exactly as the A
// fragments of the next (n8 tiles 2s and 2s+1 form k-slice s), so hidden
// activations never leave registers.  Layer 3 (64 -> 1) is a dot product of
// each lane's hidden columns with W3, reduced over the four lanes of a quad.
// (plain asm: no side effects beyond the outputs, so the compiler may
// interleave independent products)
__device__ __forceinline__ void mma_bf16_16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0,
                                               uint32_t b1) {
  asm(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}
__device__ __forceinline__ void mma_bf16_1688(float (&d)[4], uint32_t a0, uint32_t a1,
                                              uint32_t b0) {
  asm(
      "mma.sync.aligned.m16n8k8.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5}, {%6}, "
      "{%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a0), "r"(a1), "r"(b0));
}

// two floats as one bf16x2 word (the first in the low half: the lower column)
__device__ __forceinline__ uint32_t bf16x2_bits(float x, float y) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(x, y);
  return *reinterpret_cast<const uint32_t *>(&v);
}

// the two-term BF16 split of (x, y): hi word and lo word (x = hi + lo to a
// relative 2^-17)
__device__ __forceinline__ void split_bf16x2(float x, float y, uint32_t &hi, uint32_t &lo) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(x, y);
  const float rx = x - __low2float(h), ry = y - __high2float(h);
  hi = *reinterpret_cast<const uint32_t *>(&h);
  lo = bf16x2_bits(rx, ry);
}

constexpr int TC_WARPS = 4;
#ifndef GPUNB_MLP_PAIR
#define GPUNB_MLP_PAIR 1   // inference: two 16-sample tiles per warp pass
#endif
constexpr int W2_STRIDE = MLP_H / 2 + 4;   // bf16x2 words per padded W2 row (conflict-free B loads)

// W2 row o as bf16x2 words in B-fragment order: for k-slice s and lane
// column t the two words of the fragment, (k 16s + 2t, +1) and
// (k 16s + 8 + 2t, +1), side by side at 8s + 2t, so one 64-bit load fetches
// both
__host__ __device__ constexpr int w2_frag_pos(int kk) {   // kk: word index in the row (k / 2)
  return 8 * (kk / 8) + 2 * (kk % 4) + (kk % 8) / 4;
}

struct MlpTcSmem {
  uint32_t w1[MLP_H * MLP_IN / 2];     // W1[o][f] as bf16x2 words, 4 per row
  uint32_t w2[MLP_H * W2_STRIDE];      // W2[o][k] as bf16x2 words, padded rows, fragment order
  float b1h[MLP_H], b2h[MLP_H], w3[MLP_H];   // b1 / 2, b2 / 2, W3
  float b3;
};

__device__ void stage_tc_params(MlpTcSmem &s, const __nv_bfloat16 *__restrict__ wq,
                                const float *__restrict__ wf) {
  const uint32_t *wq32 = reinterpret_cast<const uint32_t *>(wq);   // OFF_W1, OFF_W2 even
  for (int k = threadIdx.x; k < MLP_H * MLP_IN / 2; k += blockDim.x)
    s.w1[k] = wq32[OFF_W1 / 2 + k];
  for (int k = threadIdx.x; k < MLP_H * MLP_H / 2; k += blockDim.x) {
    const int o = k / (MLP_H / 2), kk = k % (MLP_H / 2);
    s.w2[o * W2_STRIDE + w2_frag_pos(kk)] = wq32[OFF_W2 / 2 + k];
  }
  for (int k = threadIdx.x; k < MLP_H; k += blockDim.x) {
    s.b1h[k] = 0.5f * wf[OFF_B1 + k];
    s.b2h[k] = 0.5f * wf[OFF_B2 + k];
    s.w3[k] = __bfloat162float(wq[OFF_W3 + k]);
  }
  if (threadIdx.x == 0) s.b3 = wf[OFF_B3];
}

// Inference of one 16-sample tile by the whole warp: lane (g = lane / 4,
// t = lane % 4) passes features 2t, 2t+1 of rows g (x0) and g + 8 (x1) and
// receives the outputs of rows g and g + 8 (every lane of the quad).  BF16
// inputs and activations, FP32 accumulation: 8 MMAs (k8) for layer 1, 32
// (k16) for layer 2.
__device__ __forceinline__ float2 mlp_tile_infer(const MlpTcSmem &s, float2 x0, float2 x1) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const uint32_t a0 = bf16x2_bits(x0.x, x0.y), a1 = bf16x2_bits(x1.x, x1.y);
  uint32_t ha[4][4];
#pragma unroll
  for (int j = 0; j < MLP_H / 8; ++j) {
    float c[4] = {0.f, 0.f, 0.f, 0.f};
    mma_bf16_1688(c, a0, a1, s.w1[(8 * j + g) * (MLP_IN / 2) + t]);
    const int col = 8 * j + 2 * t;
    const f2 bb = *reinterpret_cast<const f2 *>(&s.b1h[col]);
    const int sl = j >> 1, q = (j & 1) * 2;
    const f2 h0 = gelu_fast2_half(make_float2(c[0], c[1]), bb);
    const f2 h1 = gelu_fast2_half(make_float2(c[2], c[3]), bb);
    ha[sl][q] = bf16x2_bits(h0.x, h0.y);
    ha[sl][q + 1] = bf16x2_bits(h1.x, h1.y);
  }
  f2 p0 = mk2(0.f), p1 = mk2(0.f);   // per row: the two columns' partial dot products
#pragma unroll
  for (int j = 0; j < MLP_H / 8; ++j) {
    float c[4] = {0.f, 0.f, 0.f, 0.f};
    const uint32_t *wrow = s.w2 + (8 * j + g) * W2_STRIDE;
#pragma unroll
    for (int sl = 0; sl < MLP_H / 16; ++sl) {
      const uint2 b = *reinterpret_cast<const uint2 *>(wrow + 8 * sl + 2 * t);
      mma_bf16_16816(c, ha[sl], b.x, b.y);
    }
    const int col = 8 * j + 2 * t;
    const f2 w = *reinterpret_cast<const f2 *>(&s.w3[col]);
    const f2 bb = *reinterpret_cast<const f2 *>(&s.b2h[col]);
    p0 = fma2(gelu_fast2_half(make_float2(c[0], c[1]), bb), w, p0);
    p1 = fma2(gelu_fast2_half(make_float2(c[2], c[3]), bb), w, p1);
  }
  float q0 = p0.x + p0.y, q1 = p1.x + p1.y;
  q0 += __shfl_xor_sync(0xffffffffu, q0, 1);
  q0 += __shfl_xor_sync(0xffffffffu, q0, 2);
  q1 += __shfl_xor_sync(0xffffffffu, q1, 1);
  q1 += __shfl_xor_sync(0xffffffffu, q1, 2);
  return make_float2(q0 + s.b3, q1 + s.b3);
}

#ifndef GPUNB_MLP_MINB
#define GPUNB_MLP_MINB 1   // uncapped: 184 registers, 2 blocks per SM, 3% faster than 96 / 5
#endif
__global__ void __launch_bounds__(32 * TC_WARPS, GPUNB_MLP_MINB)
    rsmlp_forward_tc_kernel(int B, const float *__restrict__ X,
                            const __nv_bfloat16 *__restrict__ wq, const float *__restrict__ wf,
                            float *__restrict__ y) {
  __shared__ __align__(16) MlpTcSmem s;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int g = lane >> 2, t = lane & 3;
  const int ntile = (B + 15) / 16;
  const int stride = gridDim.x * TC_WARPS;
  // inputs of rows g, g + 8 of a tile (zero beyond B)
  auto load = [&](int tile, float2 &x0, float2 &x1) {
    const int r0 = tile * 16 + g, r1 = r0 + 8;
    x0 = make_float2(0.f, 0.f);
    x1 = make_float2(0.f, 0.f);
    if (tile < ntile) {
      if (r0 < B) x0 = __ldg(reinterpret_cast<const float2 *>(X + (size_t)r0 * MLP_IN + 2 * t));
      if (r1 < B) x1 = __ldg(reinterpret_cast<const float2 *>(X + (size_t)r1 * MLP_IN + 2 * t));
    }
  };
#if GPUNB_MLP_PAIR
  // two tiles per pass (independent, so their products and activations
  // interleave), the next pass's inputs in flight meanwhile
  int tile = blockIdx.x * TC_WARPS + warp;
  float2 x0, x1, z0, z1;
  load(tile, x0, x1);   // in flight while the weights are staged
  load(tile + stride, z0, z1);
  stage_tc_params(s, wq, wf);
  __syncthreads();
  for (; tile < ntile; tile += 2 * stride) {
    float2 n0, n1, m0, m1;
    load(tile + 2 * stride, n0, n1);
    load(tile + 3 * stride, m0, m1);
    const float2 oa = mlp_tile_infer(s, x0, x1);
    const float2 ob = mlp_tile_infer(s, z0, z1);
    const int ra = tile * 16 + g, rb = (tile + stride) * 16 + g;
    if (t == 0) {
      if (ra < B) y[ra] = oa.x;
      if (ra + 8 < B) y[ra + 8] = oa.y;
      if (tile + stride < ntile) {
        if (rb < B) y[rb] = ob.x;
        if (rb + 8 < B) y[rb + 8] = ob.y;
      }
    }
    x0 = n0; x1 = n1;
    z0 = m0; z1 = m1;
  }
#else
  int tile = blockIdx.x * TC_WARPS + warp;
  float2 x0, x1;
  load(tile, x0, x1);
  stage_tc_params(s, wq, wf);
  __syncthreads();
  for (; tile < ntile; tile += stride) {
    float2 n0, n1;
    load(tile + stride, n0, n1);   // the next tile's inputs, in flight during this one
    const float2 out = mlp_tile_infer(s, x0, x1);
    const int r0 = tile * 16 + g, r1 = r0 + 8;
    if (t == 0) {
      if (r0 < B) y[r0] = out.x;
      if (r1 < B) y[r1] = out.y;
    }
    x0 = n0;
    x1 = n1;
  }
#endif
}

// ---------------------------------------------------------------------------
// Training labels on the device.  For particle i with target membership k_i:
// log R with R^2 the geometric mean of the k-th and (k+1)-th smallest keys
// q_j = min(|dx|^2, |dx + dtr_i dv|^2) over the j-set (position 0: the body
// itself, q = 0), dx = x_j - x_i, dv = v_j - v_i -- the radius at which the
// kernel's own membership test min(r^2, r_p^2) < R^2 admits exactly k_i
// bodies besides i.  The keys come from the library's own neighbour rows at
// an enlarged radius (list_off/list of gpunb_regf_device): every key below
// that radius is in the row, so when the row holds at least k_i + 2 members
// the two keys are exact.  One warp per row, keys sorted in shared memory.
constexpr int LABEL_WARPS = 4;
constexpr int LABEL_MAXROW = 1024;

__global__ void __launch_bounds__(32 * LABEL_WARPS)
    rsmlp_label_kernel(int ni, const int *__restrict__ list_off, const int *__restrict__ list,
                       const int *__restrict__ nnb, const double *__restrict__ xj,
                       const double *__restrict__ vj, const double *__restrict__ xi,
                       const double *__restrict__ vi, const double *__restrict__ dtr,
                       const int *__restrict__ k, double *__restrict__ logr,
                       int *__restrict__ ok) {
  __shared__ double keys[LABEL_WARPS][LABEL_MAXROW];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int i = blockIdx.x * LABEL_WARPS + w;
  if (i >= ni) return;
  double *q = keys[w];
  const int cnt = nnb[i];
  const int ki = k[i];
  if (cnt < 0 || cnt > LABEL_MAXROW || ki < 1 || cnt < ki + 2) {
    if (lane == 0) {
      ok[i] = cnt < 0 || cnt > LABEL_MAXROW ? -1 : 0;   // -1: too many, 0: too few
      logr[i] = 0.0;
    }
    return;
  }
  const int *row = list + list_off[i];
  const double x0 = xi[3 * (size_t)i], x1 = xi[3 * (size_t)i + 1], x2 = xi[3 * (size_t)i + 2];
  const double v0 = vi[3 * (size_t)i], v1 = vi[3 * (size_t)i + 1], v2 = vi[3 * (size_t)i + 2];
  const double d = dtr[i];
  int n2 = 32;
  while (n2 < cnt) n2 <<= 1;
  for (int e = lane; e < n2; e += 32) {
    double key = INFINITY;
    if (e < cnt) {
      const int j = row[e];
      const double dx = xj[3 * (size_t)j] - x0, dy = xj[3 * (size_t)j + 1] - x1,
                   dz = xj[3 * (size_t)j + 2] - x2;
      const double px = dx + d * (vj[3 * (size_t)j] - v0);
      const double py = dy + d * (vj[3 * (size_t)j + 1] - v1);
      const double pz = dz + d * (vj[3 * (size_t)j + 2] - v2);
      key = fmin(dx * dx + dy * dy + dz * dz, px * px + py * py + pz * pz);
    }
    q[e] = key;
  }
  __syncwarp();
  // bitonic sort of n2 keys, ascending
  for (int size = 2; size <= n2; size <<= 1) {
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int e = lane; e < n2; e += 32) {
        const int p = e ^ stride;
        if (p > e) {
          const bool up = (e & size) == 0;
          const double a = q[e], b = q[p];
          if ((a > b) == up) {
            q[e] = b;
            q[p] = a;
          }
        }
      }
      __syncwarp();
    }
  }
  if (lane == 0) {
    const double lo = fmax(q[ki], 1e-300);
    const double hi = fmax(q[ki + 1], lo);
    logr[i] = 0.25 * (log(lo) + log(hi));
    ok[i] = 1;
  }
}

// ---------------------------------------------------------------------------
// RS update of an active block on the device: the plain rule of
// src/Main/regcor_gpu.F:120-253 (NNBOPT stabilisation, NBAVE cap, taper,
// inertial and radial-velocity factors, RSFAC limit, second-order cube root,
// shell square root, inward reduction; the zero-neighbour branch :120-143),
// optionally the few-member rule of fpoly0.F:153-158, and -- with weights --
// the learned proposal and the plain rule as fallback when its count leaves
// the band (default 0.5-1.5 x the rule's target).  One thread per particle
// for the rule, the features and the band check; the network runs on the
// tensor cores, each warp taking its 32 particles as two 16-sample tiles
// through shared memory.
__global__ void __launch_bounds__(MLP_THREADS)
    rs_update_kernel(int ni, gpunb_rs_params p, const double *__restrict__ x,
                     const double *__restrict__ v, const double *__restrict__ m_scaled,
                     const double *__restrict__ rs, const int *__restrict__ nnb,
                     const int *__restrict__ nnb0, const double *__restrict__ acc,
                     const double *__restrict__ jrk, const double *__restrict__ dtr,
                     const __nv_bfloat16 *__restrict__ wq, const float *__restrict__ wf,
                     const float *__restrict__ norm, double *__restrict__ rs_new,
                     double *__restrict__ target, int *__restrict__ used) {
  __shared__ __align__(16) MlpTcSmem s;
  __shared__ __align__(16) float feat[MLP_THREADS][MLP_IN];
  __shared__ float yv[MLP_THREADS];
  const int tid = threadIdx.x;
  const int i = blockIdx.x * blockDim.x + tid;
  const bool live = i < ni;
  if (wq) stage_tc_params(s, wq, wf);
  double plain = 0.0, tgt = 0.0, r0 = 0.0;
  int n = 0;
  const double *xi = x + 3 * (size_t)(live ? i : 0), *vi = v + 3 * (size_t)(live ? i : 0);
  if (live) {
    n = nnb[i];
    r0 = rs[i];
    rs_plain(p, r0, n, nnb0[i], xi, vi, dtr[i], -1.0, plain, tgt);
    if (p.few_nb_rule && n < 2) plain = 1.5 * r0;
  }
  double nw = plain;
  int u = 0;
  if (wq) {   // uniform over the grid: every warp reaches the MMAs whole
    // features (rsmlp.py): log distance to the centre, log local density,
    // count / NNBOPT, log |F_reg|, log |jerk|, log regular step, log mass N,
    // log RS; normalised with the training set's mean and spread
    const double nn = (double)max(n, 0);
    if (live) {
      const double e0 = xi[0] - p.rdens[0], e1 = xi[1] - p.rdens[1], e2 = xi[2] - p.rdens[2];
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
#pragma unroll
      for (int q = 0; q < MLP_IN; ++q)
        feat[tid][q] = (float)((f[q] - (double)norm[q]) / (double)norm[MLP_IN + q]);
    } else {
#pragma unroll
      for (int q = 0; q < MLP_IN; ++q) feat[tid][q] = 0.f;
    }
    __syncthreads();   // parameters and features staged
    {
      const int lane = tid & 31, w0 = tid & ~31, g = lane >> 2, t = lane & 3;
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int r = w0 + 16 * h + g;
        const float2 o = mlp_tile_infer(s, *reinterpret_cast<const float2 *>(&feat[r][2 * t]),
                                        *reinterpret_cast<const float2 *>(&feat[r + 8][2 * t]));
        if (t == 0) {
          yv[r] = o.x;
          yv[r + 8] = o.y;
        }
      }
      __syncwarp();
    }
    if (live) {
      const float y = yv[tid];
      const double rp = r0 * exp((double)y);
      double pc;
      if (p.list_off) {
        // the count of rp at the next regular step (see gpunb.h)
        const double dt = dtr[i], rp2 = rp * rp;
        int in = 0, members = 0;
        for (int e = p.list_off[i]; e < p.list_off[i + 1]; ++e) {
          const int jj = p.list[e];
          const double *xj = p.xj + 3 * (size_t)jj, *vj = p.vj + 3 * (size_t)jj;
          const double dv0 = vj[0] - vi[0], dv1 = vj[1] - vi[1], dv2 = vj[2] - vi[2];
          const double dx0 = xj[0] - xi[0], dx1 = xj[1] - xi[1], dx2 = xj[2] - xi[2];
          if (dx0 == 0.0 && dx1 == 0.0 && dx2 == 0.0 && dv0 == 0.0 && dv1 == 0.0 && dv2 == 0.0)
            continue;
          ++members;
          const double d0 = dx0 + dt * dv0, d1 = dx1 + dt * dv1, d2 = dx2 + dt * dv2;
          const double f0 = d0 + dt * dv0, f1 = d1 + dt * dv1, f2 = d2 + dt * dv2;
          const double k = fmin(d0 * d0 + d1 * d1 + d2 * d2, f0 * f0 + f1 * f1 + f2 * f2);
          in += k < rp2;
        }
        const double grow = (rp / r0) * (rp / r0) * (rp / r0) - 1.0;
        pc = fmax((double)in + (double)members * fmax(grow, 0.0),
                  (nn + 1.0) * exp(3.0 * (double)y) - 1.0);
      } else {
        pc = (nn + 1.0) * exp(3.0 * (double)y) - 1.0;
      }
      const double blo = p.band_lo > 0.0 ? p.band_lo : 0.5;
      const double bhi = p.band_hi > 0.0 ? p.band_hi : 1.5;
      if (isfinite(y) && pc >= blo * tgt && pc <= bhi * tgt) {
        nw = rp;
        u = 1;
      }
    }
  }
  if (!live) return;
  rs_new[i] = nw;
  if (target) target[i] = tgt;
  if (used) used[i] = u;
}

// Backward pass of the mean of w_b (y_b - t_b)^2 over the batch, on the tensor
// cores.  One block of 4 warps per 128 samples; each block writes the
// gradient summed over its samples to part[blockIdx][P] and a second kernel
// sums the block rows in order, so repeated calls give bit-identical
// gradients.
//
// Per warp, for each of its two 16-sample tiles: the forward pass with inputs
// and activations as two-term BF16 splits and the accurate tanh (the
// gradients are those of FP32 arithmetic on the BF16 weights), keeping z1, z2
// (D-fragment layout) and the layer-2 A fragments of h1; then dy, dz2 = dy W3 gelu'(z2) and
// dh1 = dz2 W2 -- again D fragments of one product reused as the A fragments
// of the next, with W2 transposed in shared memory as the B operand -- and
// dz1 = dh1 gelu'(z1).  dz2, dz1, h1 and x are staged transposed (feature
// rows of 128 samples) as two-term BF16 splits, so that the weight gradients
// dW2 = dz2^T h1 and dW1 = dz1^T x are block GEMMs over the 128 samples (warp
// w owns rows 16w..16w+15), each product of splits taken as hi*hi + hi*lo +
// lo*hi.  Bias gradients, dW3, db3 and the loss are column sums reduced over
// the lanes, then over the warps in order.
constexpr int BW_WARPS = 4;
constexpr int BW_SAMPLES = 16 * 2 * BW_WARPS;           // two 16-sample tiles per warp
constexpr int BT_STRIDE = BW_SAMPLES + 8;               // bf16 per transposed row (padded)
static_assert(BW_SAMPLES == MLP_THREADS, "one block row of partial sums per 128 samples");

struct MlpBwSmem {
  uint32_t w1[MLP_H * MLP_IN / 2];       // W1[o][f]  bf16x2 (B of layer 1)
  uint32_t w2[MLP_H * W2_STRIDE];        // W2[o][k]  bf16x2 (B of layer 2)
  uint32_t w2t[MLP_H * W2_STRIDE];       // W2[o][k] as [k][o] (B of dh1 = dz2 W2)
  float b1[MLP_H], b2[MLP_H], w3[MLP_H];
  float b3;
  __nv_bfloat16 dz2t[2][MLP_H][BT_STRIDE];   // [hi/lo][o][sample]
  __nv_bfloat16 h1t[2][MLP_H][BT_STRIDE];    // [hi/lo][k][sample]
  __nv_bfloat16 dz1t[2][MLP_H][BT_STRIDE];   // [hi/lo][k][sample]
  __nv_bfloat16 xt[2][MLP_IN][BT_STRIDE];    // [hi/lo][f][sample]
  float red[BW_WARPS][3][MLP_H];             // per warp: db1, db2, dW3 partial sums
  float redy[BW_WARPS][2];                   // per warp: db3, loss
};

template <int ROWS>
__device__ __forceinline__ void stage_split(__nv_bfloat16 (*t)[ROWS][BT_STRIDE], int row,
                                            int col, float v) {
  const __nv_bfloat16 h = __float2bfloat16_rn(v);
  t[0][row][col] = h;
  t[1][row][col] = __float2bfloat16_rn(v - __bfloat162float(h));
}

__device__ __forceinline__ uint32_t ld_pair(const __nv_bfloat16 *p) {
  return *reinterpret_cast<const uint32_t *>(p);
}

// column sums of a quad-layout value over the 8 row groups of the warp
__device__ __forceinline__ float sum_over_rows(float v) {
  v += __shfl_xor_sync(0xffffffffu, v, 4);
  v += __shfl_xor_sync(0xffffffffu, v, 8);
  v += __shfl_xor_sync(0xffffffffu, v, 16);
  return v;
}

// adds the warp's column sum of v to row[col] (one lane per column writes)
__device__ __forceinline__ void add_col_sum(float *row, int col, int g, float v) {
  v = sum_over_rows(v);
  if (g == 0) row[col] += v;
}

__global__ void __launch_bounds__(32 * BW_WARPS)
    rsmlp_backward_tc_kernel(int B, const float *__restrict__ X, const float *__restrict__ T,
                             const float *__restrict__ Wt, const __nv_bfloat16 *__restrict__ wq,
                             const float *__restrict__ wf, float inv_norm,
                             float *__restrict__ part, float *__restrict__ loss_part) {
  extern __shared__ __align__(16) unsigned char bw_smem_raw[];
  MlpBwSmem &s = *reinterpret_cast<MlpBwSmem *>(bw_smem_raw);
  const uint32_t *wq32 = reinterpret_cast<const uint32_t *>(wq);
  for (int k = threadIdx.x; k < MLP_H * MLP_IN / 2; k += blockDim.x) s.w1[k] = wq32[OFF_W1 / 2 + k];
  for (int k = threadIdx.x; k < MLP_H * MLP_H / 2; k += blockDim.x) {
    const int o = k / (MLP_H / 2), kk = k % (MLP_H / 2);
    s.w2[o * W2_STRIDE + kk] = wq32[OFF_W2 / 2 + k];
  }
  for (int e = threadIdx.x; e < MLP_H * MLP_H / 2; e += blockDim.x) {
    const int k = e / (MLP_H / 2), op = e % (MLP_H / 2);   // row k, pair (2op, 2op+1) of o
    s.w2t[k * W2_STRIDE + op] =
        bf16x2_bits(__bfloat162float(wq[OFF_W2 + (2 * op) * MLP_H + k]),
                    __bfloat162float(wq[OFF_W2 + (2 * op + 1) * MLP_H + k]));
  }
  for (int k = threadIdx.x; k < MLP_H; k += blockDim.x) {
    s.b1[k] = wf[OFF_B1 + k];
    s.b2[k] = wf[OFF_B2 + k];
    s.w3[k] = __bfloat162float(wq[OFF_W3 + k]);
  }
  if (threadIdx.x == 0) s.b3 = wf[OFF_B3];
  for (int k = threadIdx.x; k < BW_WARPS * 3 * MLP_H; k += blockDim.x) (&s.red[0][0][0])[k] = 0.f;
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int g = lane >> 2, t = lane & 3;
  const int base = blockIdx.x * BW_SAMPLES;
  float sum_dy = 0.f, sum_loss = 0.f;
  for (int tl = 0; tl < 2; ++tl) {
    const int lt = 16 * (2 * warp + tl);             // tile offset within the block
    const int r0 = base + lt + g, r1 = r0 + 8;
    const bool v0 = r0 < B, v1 = r1 < B;
    float2 x0 = make_float2(0.f, 0.f), x1 = make_float2(0.f, 0.f);
    if (v0) x0 = *reinterpret_cast<const float2 *>(X + (size_t)r0 * MLP_IN + 2 * t);
    if (v1) x1 = *reinterpret_cast<const float2 *>(X + (size_t)r1 * MLP_IN + 2 * t);
    uint32_t xa_hi[4] = {0u, 0u, 0u, 0u}, xa_lo[4] = {0u, 0u, 0u, 0u};
    split_bf16x2(x0.x, x0.y, xa_hi[0], xa_lo[0]);
    split_bf16x2(x1.x, x1.y, xa_hi[1], xa_lo[1]);
    stage_split(s.xt, 2 * t, lt + g, x0.x);
    stage_split(s.xt, 2 * t + 1, lt + g, x0.y);
    stage_split(s.xt, 2 * t, lt + g + 8, x1.x);
    stage_split(s.xt, 2 * t + 1, lt + g + 8, x1.y);
    // forward
    float z1[8][4], z2[8][4];
    uint32_t ha_hi[4][4], ha_lo[4][4];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      float c[4] = {0.f, 0.f, 0.f, 0.f};
      const uint32_t b0 = s.w1[(8 * j + g) * (MLP_IN / 2) + t];
      mma_bf16_16816(c, xa_hi, b0, 0u);
      mma_bf16_16816(c, xa_lo, b0, 0u);
      const int col = 8 * j + 2 * t;
      z1[j][0] = c[0] + s.b1[col]; z1[j][1] = c[1] + s.b1[col + 1];
      z1[j][2] = c[2] + s.b1[col]; z1[j][3] = c[3] + s.b1[col + 1];
      const float h0 = gelu(z1[j][0]), h1 = gelu(z1[j][1]);
      const float h2 = gelu(z1[j][2]), h3 = gelu(z1[j][3]);
      const int sl = j >> 1, q = (j & 1) * 2;
      split_bf16x2(h0, h1, ha_hi[sl][q], ha_lo[sl][q]);
      split_bf16x2(h2, h3, ha_hi[sl][q + 1], ha_lo[sl][q + 1]);
      stage_split(s.h1t, col, lt + g, h0);
      stage_split(s.h1t, col + 1, lt + g, h1);
      stage_split(s.h1t, col, lt + g + 8, h2);
      stage_split(s.h1t, col + 1, lt + g + 8, h3);
    }
    float p0 = 0.f, p1 = 0.f;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      float c[4] = {0.f, 0.f, 0.f, 0.f};
      const uint32_t *wrow = s.w2 + (8 * j + g) * W2_STRIDE;
#pragma unroll
      for (int sl = 0; sl < 4; ++sl) {
        const uint32_t b0 = wrow[8 * sl + t], b1 = wrow[8 * sl + 4 + t];
        mma_bf16_16816(c, ha_hi[sl], b0, b1);
        mma_bf16_16816(c, ha_lo[sl], b0, b1);
      }
      const int col = 8 * j + 2 * t;
      z2[j][0] = c[0] + s.b2[col]; z2[j][1] = c[1] + s.b2[col + 1];
      z2[j][2] = c[2] + s.b2[col]; z2[j][3] = c[3] + s.b2[col + 1];
      p0 = fmaf(gelu(z2[j][0]), s.w3[col], p0);
      p0 = fmaf(gelu(z2[j][1]), s.w3[col + 1], p0);
      p1 = fmaf(gelu(z2[j][2]), s.w3[col], p1);
      p1 = fmaf(gelu(z2[j][3]), s.w3[col + 1], p1);
    }
    p0 += __shfl_xor_sync(0xffffffffu, p0, 1);
    p0 += __shfl_xor_sync(0xffffffffu, p0, 2);
    p1 += __shfl_xor_sync(0xffffffffu, p1, 1);
    p1 += __shfl_xor_sync(0xffffffffu, p1, 2);
    // residuals of rows g and g + 8 (every lane of the quad holds them)
    const float w0 = v0 ? (Wt ? Wt[r0] : 1.0f) : 0.f, w1 = v1 ? (Wt ? Wt[r1] : 1.0f) : 0.f;
    const float e0 = v0 ? p0 + s.b3 - T[r0] : 0.f, e1 = v1 ? p1 + s.b3 - T[r1] : 0.f;
    const float dy0 = 2.0f * w0 * e0 * inv_norm, dy1 = 2.0f * w1 * e1 * inv_norm;
    if (t == 0) {
      sum_dy += dy0 + dy1;
      sum_loss += w0 * e0 * e0 * inv_norm + w1 * e1 * e1 * inv_norm;
    }
    // dz2 = dy W3 gelu'(z2) -> A fragments of dh1 = dz2 W2
    uint32_t da_hi[4][4], da_lo[4][4];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int col = 8 * j + 2 * t;
      const float d0 = dy0 * s.w3[col] * gelu_grad(z2[j][0]);
      const float d1 = dy0 * s.w3[col + 1] * gelu_grad(z2[j][1]);
      const float d2 = dy1 * s.w3[col] * gelu_grad(z2[j][2]);
      const float d3 = dy1 * s.w3[col + 1] * gelu_grad(z2[j][3]);
      add_col_sum(s.red[warp][1], col, g, d0 + d2);
      add_col_sum(s.red[warp][1], col + 1, g, d1 + d3);
      add_col_sum(s.red[warp][2], col, g, dy0 * gelu(z2[j][0]) + dy1 * gelu(z2[j][2]));
      add_col_sum(s.red[warp][2], col + 1, g, dy0 * gelu(z2[j][1]) + dy1 * gelu(z2[j][3]));
      const int sl = j >> 1, q = (j & 1) * 2;
      split_bf16x2(d0, d1, da_hi[sl][q], da_lo[sl][q]);
      split_bf16x2(d2, d3, da_hi[sl][q + 1], da_lo[sl][q + 1]);
      stage_split(s.dz2t, col, lt + g, d0);
      stage_split(s.dz2t, col + 1, lt + g, d1);
      stage_split(s.dz2t, col, lt + g + 8, d2);
      stage_split(s.dz2t, col + 1, lt + g + 8, d3);
    }
    // dh1 = dz2 W2 (B from W2 transposed), dz1 = dh1 gelu'(z1)
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      float c[4] = {0.f, 0.f, 0.f, 0.f};
      const uint32_t *wrow = s.w2t + (8 * j + g) * W2_STRIDE;
#pragma unroll
      for (int sl = 0; sl < 4; ++sl) {
        const uint32_t b0 = wrow[8 * sl + t], b1 = wrow[8 * sl + 4 + t];
        mma_bf16_16816(c, da_hi[sl], b0, b1);
        mma_bf16_16816(c, da_lo[sl], b0, b1);
      }
      const int col = 8 * j + 2 * t;
      const float d0 = c[0] * gelu_grad(z1[j][0]), d1 = c[1] * gelu_grad(z1[j][1]);
      const float d2 = c[2] * gelu_grad(z1[j][2]), d3 = c[3] * gelu_grad(z1[j][3]);
      add_col_sum(s.red[warp][0], col, g, d0 + d2);
      add_col_sum(s.red[warp][0], col + 1, g, d1 + d3);
      stage_split(s.dz1t, col, lt + g, d0);
      stage_split(s.dz1t, col + 1, lt + g, d1);
      stage_split(s.dz1t, col, lt + g + 8, d2);
      stage_split(s.dz1t, col + 1, lt + g + 8, d3);
    }
  }
  sum_dy += __shfl_xor_sync(0xffffffffu, sum_dy, 4);
  sum_dy += __shfl_xor_sync(0xffffffffu, sum_dy, 8);
  sum_dy += __shfl_xor_sync(0xffffffffu, sum_dy, 16);
  sum_loss += __shfl_xor_sync(0xffffffffu, sum_loss, 4);
  sum_loss += __shfl_xor_sync(0xffffffffu, sum_loss, 8);
  sum_loss += __shfl_xor_sync(0xffffffffu, sum_loss, 16);
  if (lane == 0) {
    s.redy[warp][0] = sum_dy;
    s.redy[warp][1] = sum_loss;
  }
  __syncthreads();
  // weight gradients over the block's samples: warp w owns rows 16w..16w+15
  float *pb = part + (size_t)blockIdx.x * MLP_P;
  {
    const int m0 = 16 * warp;
    float acc[8][4], acc1[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int n = 0; n < 8; ++n) acc[n][0] = acc[n][1] = acc[n][2] = acc[n][3] = 0.f;
#pragma unroll 2
    for (int ks = 0; ks < BW_SAMPLES / 16; ++ks) {
      const int kc = 16 * ks + 2 * t;
      uint32_t ah[4], al[4], zh[4], zl[4];
#pragma unroll
      for (int hl = 0; hl < 2; ++hl) {
        uint32_t *a = hl ? al : ah, *z = hl ? zl : zh;
        a[0] = ld_pair(&s.dz2t[hl][m0 + g][kc]);
        a[1] = ld_pair(&s.dz2t[hl][m0 + g + 8][kc]);
        a[2] = ld_pair(&s.dz2t[hl][m0 + g][kc + 8]);
        a[3] = ld_pair(&s.dz2t[hl][m0 + g + 8][kc + 8]);
        z[0] = ld_pair(&s.dz1t[hl][m0 + g][kc]);
        z[1] = ld_pair(&s.dz1t[hl][m0 + g + 8][kc]);
        z[2] = ld_pair(&s.dz1t[hl][m0 + g][kc + 8]);
        z[3] = ld_pair(&s.dz1t[hl][m0 + g + 8][kc + 8]);
      }
      const uint32_t (&ahr)[4] = *reinterpret_cast<const uint32_t(*)[4]>(ah);
      const uint32_t (&alr)[4] = *reinterpret_cast<const uint32_t(*)[4]>(al);
      const uint32_t (&zhr)[4] = *reinterpret_cast<const uint32_t(*)[4]>(zh);
      const uint32_t (&zlr)[4] = *reinterpret_cast<const uint32_t(*)[4]>(zl);
#pragma unroll
      for (int n = 0; n < 8; ++n) {
        const uint32_t bh0 = ld_pair(&s.h1t[0][8 * n + g][kc]);
        const uint32_t bh1 = ld_pair(&s.h1t[0][8 * n + g][kc + 8]);
        const uint32_t bl0 = ld_pair(&s.h1t[1][8 * n + g][kc]);
        const uint32_t bl1 = ld_pair(&s.h1t[1][8 * n + g][kc + 8]);
        mma_bf16_16816(acc[n], ahr, bh0, bh1);
        mma_bf16_16816(acc[n], ahr, bl0, bl1);
        mma_bf16_16816(acc[n], alr, bh0, bh1);
      }
      const uint32_t xh0 = ld_pair(&s.xt[0][g][kc]), xh1 = ld_pair(&s.xt[0][g][kc + 8]);
      const uint32_t xl0 = ld_pair(&s.xt[1][g][kc]), xl1 = ld_pair(&s.xt[1][g][kc + 8]);
      mma_bf16_16816(acc1, zhr, xh0, xh1);
      mma_bf16_16816(acc1, zhr, xl0, xl1);
      mma_bf16_16816(acc1, zlr, xh0, xh1);
    }
#pragma unroll
    for (int n = 0; n < 8; ++n) {
      const int k = 8 * n + 2 * t;
      pb[OFF_W2 + (m0 + g) * MLP_H + k] = acc[n][0];
      pb[OFF_W2 + (m0 + g) * MLP_H + k + 1] = acc[n][1];
      pb[OFF_W2 + (m0 + g + 8) * MLP_H + k] = acc[n][2];
      pb[OFF_W2 + (m0 + g + 8) * MLP_H + k + 1] = acc[n][3];
    }
    pb[OFF_W1 + (m0 + g) * MLP_IN + 2 * t] = acc1[0];
    pb[OFF_W1 + (m0 + g) * MLP_IN + 2 * t + 1] = acc1[1];
    pb[OFF_W1 + (m0 + g + 8) * MLP_IN + 2 * t] = acc1[2];
    pb[OFF_W1 + (m0 + g + 8) * MLP_IN + 2 * t + 1] = acc1[3];
  }
  const int tid = threadIdx.x;
  if (tid < MLP_H) {
    float a = 0.f, b = 0.f, c = 0.f;
    for (int w = 0; w < BW_WARPS; ++w) {
      a += s.red[w][0][tid];
      b += s.red[w][1][tid];
      c += s.red[w][2][tid];
    }
    pb[OFF_B1 + tid] = a;
    pb[OFF_B2 + tid] = b;
    pb[OFF_W3 + tid] = c;
  } else if (tid == MLP_H) {
    float a = 0.f, l = 0.f;
    for (int w = 0; w < BW_WARPS; ++w) {
      a += s.redy[w][0];
      l += s.redy[w][1];
    }
    pb[OFF_B3] = a;
    loss_part[blockIdx.x] = l;
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
  // one warp per 16-sample tile; one wave of resident blocks striding over
  // the tiles (a grid beyond what fits leaves a second, nearly empty wave)
  // (resident blocks per device, cached: the queries cost more host time than
  // the kernel takes for small batches; concurrent first calls store equal values)
  static std::atomic<int> wave[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return GPUNB_E_CUDA;
  int blocks = wave[dev].load(std::memory_order_relaxed);
  if (blocks == 0) {
    int n_sm = 0, per_sm = 0;
    if (cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, rsmlp_forward_tc_kernel,
                                                      32 * TC_WARPS, 0) != cudaSuccess)
      return GPUNB_E_CUDA;
    blocks = std::max(1, n_sm * per_sm);
    wave[dev].store(blocks, std::memory_order_relaxed);
  }
  const long long tiles = (B + 15) / 16;
  const long long want = (tiles + TC_WARPS - 1) / TC_WARPS;
  const int grid = (int)std::max(1ll, std::min(want, (long long)blocks));
  rsmlp_forward_tc_kernel<<<grid, 32 * TC_WARPS, 0, (cudaStream_t)stream>>>(
      B, X, (const __nv_bfloat16 *)wq, wf, y);
  return cudaGetLastError() == cudaSuccess ? GPUNB_OK : GPUNB_E_CUDA;
}

// part: scratch of ceil(B/128)*P floats + ceil(B/128) floats
int gpunb_rsmlp_backward(int B, const float *X, const float *T, const float *W, const void *wq,
                         const float *wf, float *grad, float *loss, float *part, void *stream) {
  if (B <= 0) return GPUNB_E_ARG;
  const int nb = (B + MLP_THREADS - 1) / MLP_THREADS;
  float *loss_part = part + (size_t)nb * MLP_P;
  cudaStream_t st = (cudaStream_t)stream;
  const size_t smem = sizeof(MlpBwSmem);
  if (cudaFuncSetAttribute(rsmlp_backward_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem) != cudaSuccess)
    return GPUNB_E_CUDA;
  rsmlp_backward_tc_kernel<<<nb, 32 * BW_WARPS, smem, st>>>(
      B, X, T, W, (const __nv_bfloat16 *)wq, wf, 1.0f / (float)B, part, loss_part);
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

int gpunb_rsmlp_label_device(int ni, const int *list_off, const int *list, const int *nnb,
                             const double *xj, const double *vj, const double *xi,
                             const double *vi, const double *dtr, const int *k, double *logr,
                             int *ok, void *stream) {
  if (ni < 0 || (ni > 0 && (!list_off || !list || !nnb || !xj || !vj || !xi || !vi || !dtr ||
                            !k || !logr || !ok)))
    return GPUNB_E_ARG;
  if (ni == 0) return GPUNB_OK;
  rsmlp_label_kernel<<<(ni + LABEL_WARPS - 1) / LABEL_WARPS, 32 * LABEL_WARPS, 0,
                       (cudaStream_t)stream>>>(ni, list_off, list, nnb, xj, vj, xi, vi, dtr, k,
                                               logr, ok);
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
