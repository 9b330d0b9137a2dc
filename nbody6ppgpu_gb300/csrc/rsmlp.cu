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
// Inference (gpunb_rsmlp_forward) and training (gpunb_rsmlp_backward) run
// their matrix products on the tensor cores (mma.sync BF16 tiles of 16
// samples, FP32 accumulation, FP32 inputs and activations as two-term BF16
// splits); the fused RS update evaluates the network per particle on the
// CUDA cores (mlp_eval).
#include <cuda_bf16.h>

#include <algorithm>

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

// ---------------------------------------------------------------------------
// Tensor-core forward pass (mma.sync m16n8k16, BF16 operands, FP32
// accumulation), 16 samples per warp tile.
//
// Layer 1 takes X (16 samples x 8 features, padded to K = 16) as the A
// operand and W1 (BF16) as B; its D fragments (rows g, g+8 of the tile, two
// adjacent hidden columns per n8 tile) are laid out exactly as the A
// fragments of layer 2 (n8 tiles 2s and 2s+1 form k-slice s), so the hidden
// activations never leave registers.  FP32 values enter as a two-term BF16
// split, v = hi + lo with hi = bf16(v), lo = bf16(v - hi) (relative error
// below 2^-17), each term in its own MMA against the exact BF16 weight: the
// result matches FP32 arithmetic on the same BF16 weights to about 1e-5.
// Layer 3 (64 -> 1) is a dot product of each lane's hidden columns with W3,
// reduced over the four lanes of a quad.
__device__ __forceinline__ void mma_bf16_16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0,
                                               uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// two floats as one bf16x2 word (the first in the low half: the lower column)
__device__ __forceinline__ uint32_t bf16x2_bits(float x, float y) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(x, y);
  return *reinterpret_cast<const uint32_t *>(&v);
}

// the two-term BF16 split of (x, y): hi word and lo word
__device__ __forceinline__ void split_bf16x2(float x, float y, uint32_t &hi, uint32_t &lo) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(x, y);
  const float rx = x - __low2float(h), ry = y - __high2float(h);
  hi = *reinterpret_cast<const uint32_t *>(&h);
  lo = bf16x2_bits(rx, ry);
}

constexpr int TC_WARPS = 4;
constexpr int W2_STRIDE = MLP_H / 2 + 4;   // bf16x2 words per padded W2 row (conflict-free B loads)

struct MlpTcSmem {
  uint32_t w1[MLP_H * MLP_IN / 2];     // W1[o][f] as bf16x2 words, 4 per row
  uint32_t w2[MLP_H * W2_STRIDE];      // W2[o][k] as bf16x2 words, padded rows
  float b1[MLP_H], b2[MLP_H], w3[MLP_H];
  float b3;
};

__global__ void __launch_bounds__(32 * TC_WARPS)
    rsmlp_forward_tc_kernel(int B, const float *__restrict__ X,
                            const __nv_bfloat16 *__restrict__ wq, const float *__restrict__ wf,
                            float *__restrict__ y) {
  __shared__ __align__(16) MlpTcSmem s;
  const uint32_t *wq32 = reinterpret_cast<const uint32_t *>(wq);   // OFF_W1, OFF_W2 even
  for (int k = threadIdx.x; k < MLP_H * MLP_IN / 2; k += blockDim.x)
    s.w1[k] = wq32[OFF_W1 / 2 + k];
  for (int k = threadIdx.x; k < MLP_H * MLP_H / 2; k += blockDim.x) {
    const int o = k / (MLP_H / 2), kk = k % (MLP_H / 2);
    s.w2[o * W2_STRIDE + kk] = wq32[OFF_W2 / 2 + k];
  }
  for (int k = threadIdx.x; k < MLP_H; k += blockDim.x) {
    s.b1[k] = wf[OFF_B1 + k];
    s.b2[k] = wf[OFF_B2 + k];
    s.w3[k] = __bfloat162float(wq[OFF_W3 + k]);
  }
  if (threadIdx.x == 0) s.b3 = wf[OFF_B3];
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int g = lane >> 2, t = lane & 3;
  const int ntile = (B + 15) / 16;
  for (int tile = blockIdx.x * TC_WARPS + warp; tile < ntile; tile += gridDim.x * TC_WARPS) {
    const int r0 = tile * 16 + g, r1 = r0 + 8;
    float2 x0 = make_float2(0.f, 0.f), x1 = make_float2(0.f, 0.f);
    if (r0 < B) x0 = *reinterpret_cast<const float2 *>(X + (size_t)r0 * MLP_IN + 2 * t);
    if (r1 < B) x1 = *reinterpret_cast<const float2 *>(X + (size_t)r1 * MLP_IN + 2 * t);
    uint32_t xa_hi[4] = {0u, 0u, 0u, 0u}, xa_lo[4] = {0u, 0u, 0u, 0u};
    split_bf16x2(x0.x, x0.y, xa_hi[0], xa_lo[0]);   // row g, features 2t, 2t+1
    split_bf16x2(x1.x, x1.y, xa_hi[1], xa_lo[1]);   // row g+8
    // layer 1 -> the A fragments of layer 2 (k-slice s from n-tiles 2s, 2s+1)
    uint32_t ha_hi[4][4], ha_lo[4][4];
#pragma unroll
    for (int j = 0; j < MLP_H / 8; ++j) {
      float c[4] = {0.f, 0.f, 0.f, 0.f};
      const uint32_t b0 = s.w1[(8 * j + g) * (MLP_IN / 2) + t];
      mma_bf16_16816(c, xa_hi, b0, 0u);
      mma_bf16_16816(c, xa_lo, b0, 0u);
      const int col = 8 * j + 2 * t;
      const float h0 = gelu(c[0] + s.b1[col]), h1 = gelu(c[1] + s.b1[col + 1]);
      const float h2 = gelu(c[2] + s.b1[col]), h3 = gelu(c[3] + s.b1[col + 1]);
      const int sl = j >> 1, q = (j & 1) * 2;
      split_bf16x2(h0, h1, ha_hi[sl][q], ha_lo[sl][q]);
      split_bf16x2(h2, h3, ha_hi[sl][q + 1], ha_lo[sl][q + 1]);
    }
    // layers 2 and 3
    float p0 = 0.f, p1 = 0.f;
#pragma unroll
    for (int j = 0; j < MLP_H / 8; ++j) {
      float c[4] = {0.f, 0.f, 0.f, 0.f};
      const uint32_t *wrow = s.w2 + (8 * j + g) * W2_STRIDE;
#pragma unroll
      for (int sl = 0; sl < MLP_H / 16; ++sl) {
        const uint32_t b0 = wrow[8 * sl + t], b1 = wrow[8 * sl + 4 + t];
        mma_bf16_16816(c, ha_hi[sl], b0, b1);
        mma_bf16_16816(c, ha_lo[sl], b0, b1);
      }
      const int col = 8 * j + 2 * t;
      p0 = fmaf(gelu(c[0] + s.b2[col]), s.w3[col], p0);
      p0 = fmaf(gelu(c[1] + s.b2[col + 1]), s.w3[col + 1], p0);
      p1 = fmaf(gelu(c[2] + s.b2[col]), s.w3[col], p1);
      p1 = fmaf(gelu(c[3] + s.b2[col + 1]), s.w3[col + 1], p1);
    }
    p0 += __shfl_xor_sync(0xffffffffu, p0, 1);
    p0 += __shfl_xor_sync(0xffffffffu, p0, 2);
    p1 += __shfl_xor_sync(0xffffffffu, p1, 1);
    p1 += __shfl_xor_sync(0xffffffffu, p1, 2);
    if (t == 0) {
      if (r0 < B) y[r0] = p0 + s.b3;
      if (r1 < B) y[r1] = p1 + s.b3;
    }
  }
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

// Backward pass of the mean of w_b (y_b - t_b)^2 over the batch, on the tensor
// cores.  One block of 4 warps per 128 samples; each block writes the
// gradient summed over its samples to part[blockIdx][P] and a second kernel
// sums the block rows in order, so repeated calls give bit-identical
// gradients.
//
// Per warp, for each of its two 16-sample tiles: the forward pass as in
// rsmlp_forward_tc_kernel, keeping z1, z2 (D-fragment layout) and the
// layer-2 A fragments of h1; then dy, dz2 = dy W3 gelu'(z2) and
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
  // one warp per 16-sample tile, a grid of a few blocks per SM
  int dev = 0, n_sm = 152;
  if (cudaGetDevice(&dev) == cudaSuccess)
    cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
  const long long tiles = (B + 15) / 16;
  const long long want = (tiles + TC_WARPS - 1) / TC_WARPS;
  const int grid = (int)std::max(1ll, std::min(want, 8ll * n_sm));
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
