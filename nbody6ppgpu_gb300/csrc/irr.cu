// Irregular (neighbour) force on the GPU: drop-in for the reference's SIMD
// library src/Main/irr.avx.cpp (entry points :565-603, semantics :162-176,
// 275-309, 437-560), with the C ABI of include/irr.h.
//
// The reference keeps every particle's predictor state and neighbour list in
// host arrays (irr_simd_set_jp_ / irr_simd_set_list_, called one particle at
// a time from OpenMP loops) and evaluates the force of an active block with
// AVX on the host cores.  Here the same calls update host mirrors and append
// the particle to a dirty list (lock-free, so the OpenMP callers stay
// parallel); the next force call uploads only the changed records and rows,
// then 8 or 32 lanes per active particle predict the particle and its listed
// neighbours to the block time (FP64) and sum the force in double-float
// arithmetic on the FP32 pipe (the default: within ~1e-11 of FP64, 4x faster
// than FP64 on GB300), in FP64, or in split FP32 (the reference's own
// precision scheme, 7.6x faster than FP64).  On systems
// where the device reads pageable memory coherently (Grace + GB300 over
// NVLink-C2C) the kernels read the mirrors, the address list and write the
// results in host memory directly; elsewhere they go through pinned staging.
#include <algorithm>
#include <atomic>
#include <climits>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>
#include <sys/time.h>

#include <cuda_runtime.h>

#include "common.cuh"
#include "gpunb.h"
#include "internal.h"
#include "irr.h"
#include "launch.h"

namespace gpunb {
namespace irr {

// particle record: 16 doubles {x0[3], m, v0[3], t0, a2[3], 0, j6[3], 0}
constexpr int REC = 16;
constexpr int IRR_WARPS = 8;   // warps per block; one active particle per warp
// per-call status on the device: the error word (int, offset 0) and the
// listed pairs of the call (unsigned long long, offset 8)
constexpr size_t kStatusBytes = 16;

// ---------------------------------------------------------------------------
// device

// predicted position and velocity at ti (irr.avx.cpp:162-176)
__device__ __forceinline__ void predict(const double *__restrict__ r, double ti, double x[3],
                                        double v[3], double &m) {
  const double2 *p = reinterpret_cast<const double2 *>(r);
  const double2 q0 = p[0], q1 = p[1], q2 = p[2], q3 = p[3];
  const double2 q4 = p[4], q5 = p[5], q6 = p[6], q7 = p[7];
  const double dt = ti - q3.y;
  const double x0[3] = {q0.x, q0.y, q1.x}, v0[3] = {q2.x, q2.y, q3.x};
  const double a2[3] = {q4.x, q4.y, q5.x}, j6[3] = {q6.x, q6.y, q7.x};
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    x[c] = x0[c] + dt * (v0[c] + dt * (a2[c] + dt * j6[c]));
    v[c] = v0[c] + 2.0 * dt * (a2[c] + 1.5 * dt * j6[c]);
  }
  m = q1.y;
}

__device__ __forceinline__ void flag(int *err, int code) {
  if (err) atomicCAS(err, 0, code);
}

// Predicted state of every particle, 8 doubles each {x[3], m, v[3], 0}, for
// the large blocks where the particles' lists cover the set many times over:
// each prediction is then made once instead of once per listing.  Same
// arithmetic as the per-pair prediction, so the same bits.
constexpr int PRED = 8;
__global__ void irr_pred_kernel(int n, const double *__restrict__ rec, double ti,
                                double *__restrict__ pred) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double x[3], v[3], m;
  predict(rec + (size_t)i * REC, ti, x, v, m);
  double2 *q = reinterpret_cast<double2 *>(pred + (size_t)i * PRED);
  q[0] = make_double2(x[0], x[1]);
  q[1] = make_double2(x[2], m);
  q[2] = make_double2(v[0], v[1]);
  q[3] = make_double2(v[2], 0.0);
}

template <bool PRE>
__device__ __forceinline__ void state(const double *__restrict__ rec,
                                      const double *__restrict__ pred, int i, double ti,
                                      double x[3], double v[3], double &m) {
  if (PRE) {
    const double2 *q = reinterpret_cast<const double2 *>(pred + (size_t)i * PRED);
    const double2 a = q[0], b = q[1], c = q[2], d = q[3];
    x[0] = a.x; x[1] = a.y; x[2] = b.x; m = b.y;
    v[0] = c.x; v[1] = c.y; v[2] = d.x;
  } else {
    predict(rec + (size_t)i * REC, ti, x, v, m);
  }
}

// Lanes per active particle G: 8 (four particles per warp) for blocks that
// fill the GPU, 32 for smaller ones.  An irregular list holds ~50-150
// bodies, so with G = 8 each lane takes 6-20 of them and the cross-lane sum
// is 3 shuffle levels shared by the warp's four particles instead of 5 per
// particle (on GB300 the FP64 adds of a per-particle 5-level butterfly cost
// as much as the pair arithmetic); a small block has too few warps to hide
// the latency of 6-20 dependent gathers per lane, and takes G = 32.  The lane
// count sets the summation order, so a particle's last bits can differ
// between a block below and a block above IRR_G_MIN_NI particles; for the
// same call the results are always the same.
constexpr int IRR_G = 8;
constexpr int IRR_G_MIN_NI = 4 * 152 * IRR_WARPS;   // about 4 blocks per SM of GB300
constexpr int IRR_U = 4;   // listings per lane in flight (split kernel)
// split kernel: ~100 registers a thread, so blocks of 4 warps (5 per SM)
// keep more warps resident than blocks of 8 (2 per SM)
constexpr int IRR32_WARPS = 4;

template <bool PRE, int G>
__global__ void __launch_bounds__(32 * IRR_WARPS)
    irr_firr_kernel(int n, const double *__restrict__ rec, const double *__restrict__ pred,
                    int lmax, const int *__restrict__ lists, double ti, int ni,
                    const int *__restrict__ addr, int base, double *__restrict__ acc,
                    double *__restrict__ jrk, int *__restrict__ nnbid, int *__restrict__ err,
                    unsigned long long *__restrict__ inter) {
  const int lane = threadIdx.x & 31, sub = lane & (G - 1);
  const int nwarps = (int)((gridDim.x * blockDim.x) >> 5);
  const int warp = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  // every lane runs every iteration (the shuffles below need all 32)
  for (int k0 = warp * (32 / G); k0 < ni; k0 += nwarps * (32 / G)) {
    const int k = k0 + lane / G;
    double ax = 0, ay = 0, az = 0, jx = 0, jy = 0, jz = 0;
    double best = INFINITY;
    int bj = INT_MAX;
    const int i = k < ni ? addr[k] - base : 0;
    if (k < ni && (i < 0 || i >= n)) {
      if (sub == 0) flag(err, GPUNB_E_ARG);
    } else if (k < ni) {
      double xi[3], vi[3], mi;
      state<PRE>(rec, pred, i, ti, xi, vi, mi);
      const int *row = lists + (size_t)i * lmax;
      int nnb = row[0];
      if (nnb < 0 || nnb > lmax - 1) {
        if (sub == 0) flag(err, GPUNB_E_ARG);
        nnb = 0;
      }
      if (inter && sub == 0 && nnb > 0) atomicAdd(inter, (unsigned long long)nnb);
      for (int q = sub; q < nnb; q += G) {
        const int j = row[1 + q];
        if (j < 0 || j >= n) {
          flag(err, GPUNB_E_ARG);
          continue;
        }
        double xj[3], vj[3], mj;
        state<PRE>(rec, pred, j, ti, xj, vj, mj);
        const double dx = xj[0] - xi[0], dy = xj[1] - xi[1], dz = xj[2] - xi[2];
        const double dvx = vj[0] - vi[0], dvy = vj[1] - vi[1], dvz = vj[2] - vi[2];
        const double r2 = dx * dx + dy * dy + dz * dz;
        if (r2 < best || (r2 == best && j < bj)) {
          best = r2;
          bj = j;
        }
        if (r2 > 0.0) {   // a listed body at zero distance adds nothing
          const double rinv = rsqrt(r2);
          const double rinv2 = rinv * rinv;
          const double mr3 = mj * rinv * rinv2;
          const double al = -3.0 * (dx * dvx + dy * dvy + dz * dvz) * rinv2;
          ax += mr3 * dx;
          ay += mr3 * dy;
          az += mr3 * dz;
          jx += mr3 * (dvx + al * dx);
          jy += mr3 * (dvy + al * dy);
          jz += mr3 * (dvz + al * dz);
        }
      }
    }
    // fixed butterfly within the particle's lanes (deterministic)
    for (int o = G / 2; o > 0; o >>= 1) {
      ax += __shfl_xor_sync(0xffffffffu, ax, o);
      ay += __shfl_xor_sync(0xffffffffu, ay, o);
      az += __shfl_xor_sync(0xffffffffu, az, o);
      jx += __shfl_xor_sync(0xffffffffu, jx, o);
      jy += __shfl_xor_sync(0xffffffffu, jy, o);
      jz += __shfl_xor_sync(0xffffffffu, jz, o);
      const double ob = __shfl_xor_sync(0xffffffffu, best, o);
      const int oj = __shfl_xor_sync(0xffffffffu, bj, o);
      if (ob < best || (ob == best && oj < bj)) {
        best = ob;
        bj = oj;
      }
    }
    if (sub == 0 && k < ni) {
      acc[3 * (size_t)k] = ax;
      acc[3 * (size_t)k + 1] = ay;
      acc[3 * (size_t)k + 2] = az;
      jrk[3 * (size_t)k] = jx;
      jrk[3 * (size_t)k + 1] = jy;
      jrk[3 * (size_t)k + 2] = jz;
      nnbid[k] = (bj == INT_MAX) ? 0 : bj + 1;
    }
  }
}

// ---------------------------------------------------------------------------
// Split precision (irr_set_precision(0)): the reference's own scheme for this force
// (irr.avx.cpp:58-176: positions as FP32 hi + lo pairs, FP32 velocities and
// force arithmetic), laid out for the GPU.  The prediction stays FP64 -- one
// Taylor step per particle (whole-set blocks) or per listing (small blocks),
// ~24 FP64 operations -- and its result is split into a double-single
// position, an FP32 mass and velocity: 3 float4 = 48 bytes per particle,
// which always span exactly two 32-byte sectors when gathered.  The pair
// arithmetic runs on the FP32 pipe, which GB300 has 64 times more of than
// FP64: double-single coordinate difference, rsqrt estimate with one Newton
// step in residual form, 1/r^3 and the jerk term in FP32.  Each lane sums at
// most IRR_U pairs in FP32 before it folds them into float-float lane sums, and
// a particle's 8 lanes are combined in float-float in a fixed butterfly, so
// the result is deterministic and the summation adds no error worth stating
// (FP64 adds would cost as much as the pair arithmetic).  What remains is
// the FP32 rounding of each pair term (a few units of 2^-24): an irregular
// force is a sum of a few dominant terms, so unlike the regular force's
// thousands these errors do not average out, and where the terms cancel the
// relative error of the sum grows with the cancellation.  A C emulation of
// the arithmetic against FP64 (Plummer N = 16384, lists of ~100) shows that
// exact arithmetic after the FP32 inputs would still leave 1.1e-6 of
// max(|Q_i|, S_i / 8) in the derivative: only double-single differences and
// velocities with float-float arithmetic throughout would reach the regular
// force's 1e-6 bound: that is the double-float mode below.
constexpr int PRED32 = 3;   // float4 per particle

__device__ __forceinline__ void split_state(const double x[3], const double v[3], double m,
                                            float4 s[PRED32]) {
  float h[3], l[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) ds_split(x[c], h[c], l[c]);
  s[0] = make_float4(h[0], h[1], h[2], (float)m);
  s[1] = make_float4(l[0], l[1], l[2], 0.f);
  s[2] = make_float4((float)v[0], (float)v[1], (float)v[2], 0.f);
}

__global__ void irr_pred32_kernel(int n, const double *__restrict__ rec, double ti,
                                  float4 *__restrict__ pred) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double x[3], v[3], m;
  predict(rec + (size_t)i * REC, ti, x, v, m);
  float4 s[PRED32];
  split_state(x, v, m, s);
#pragma unroll
  for (int u = 0; u < PRED32; ++u) pred[(size_t)i * PRED32 + u] = s[u];
}

template <bool PRE>
__device__ __forceinline__ void state32(const double *__restrict__ rec,
                                        const float4 *__restrict__ pred, int i, double ti,
                                        float4 s[PRED32]) {
  if (PRE) {
#pragma unroll
    for (int u = 0; u < PRED32; ++u) s[u] = __ldg(pred + (size_t)i * PRED32 + u);
  } else {
    double x[3], v[3], m;
    predict(rec + (size_t)i * REC, ti, x, v, m);
    split_state(x, v, m, s);
  }
}

// Same contract as irr_firr_kernel.  Bodies closer than 1e-19 (r^2 below the
// smallest normal float), the particle itself included, add nothing; the
// nearest neighbour is chosen on the FP32 r^2 (ties to the smaller id).
template <bool PRE, int G>
__global__ void __launch_bounds__(32 * IRR32_WARPS)
    irr_firr32_kernel(int n, const double *__restrict__ rec, const float4 *__restrict__ pred,
                      int lmax, const int *__restrict__ lists, double ti, int ni,
                      const int *__restrict__ addr, int base, double *__restrict__ acc,
                      double *__restrict__ jrk, int *__restrict__ nnbid, int *__restrict__ err,
                      unsigned long long *__restrict__ inter) {
  const int lane = threadIdx.x & 31, sub = lane & (G - 1);
  const int nwarps = (int)((gridDim.x * blockDim.x) >> 5);
  const int warp = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  for (int k0 = warp * (32 / G); k0 < ni; k0 += nwarps * (32 / G)) {
    const int k = k0 + lane / G;
    float hi[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f}, lo[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    float best = INFINITY;
    int bj = INT_MAX;
    const int i = k < ni ? addr[k] - base : 0;
    if (k < ni && (i < 0 || i >= n)) {
      if (sub == 0) flag(err, GPUNB_E_ARG);
    } else if (k < ni) {
      float4 si[PRED32];
      state32<PRE>(rec, pred, i, ti, si);
      const int *row = lists + (size_t)i * lmax;
      int nnb = row[0];
      if (nnb < 0 || nnb > lmax - 1) {
        if (sub == 0) flag(err, GPUNB_E_ARG);
        nnb = 0;
      }
      if (inter && sub == 0 && nnb > 0) atomicAdd(inter, (unsigned long long)nnb);
      // IRR_U listings per lane in flight: their ids, then their states, are
      // loaded before any is used, so the gathers' latencies overlap
      // ids of the lane's next IRR_U listings; loaded one chunk ahead, so the
      // row read of chunk c + 1 is in flight while chunk c computes
      int jn[IRR_U];
      auto load_ids = [&](int q0) {
#pragma unroll
        for (int u = 0; u < IRR_U; ++u) {
          const int q = q0 + u * G;
          jn[u] = q < nnb ? __ldg(row + 1 + q) : -1;
        }
      };
      load_ids(sub);
      for (int q0 = sub; q0 < nnb; q0 += IRR_U * G) {
        int jv[IRR_U];
#pragma unroll
        for (int u = 0; u < IRR_U; ++u) {
          jv[u] = jn[u];
          if (q0 + u * G < nnb && (jv[u] < 0 || jv[u] >= n)) {
            flag(err, GPUNB_E_ARG);
            jv[u] = -1;
          }
        }
        float4 sj[IRR_U][PRED32];
#pragma unroll
        for (int u = 0; u < IRR_U; ++u) {
          if (jv[u] >= 0) {
            state32<PRE>(rec, pred, jv[u], ti, sj[u]);
          } else {
#pragma unroll
            for (int w = 0; w < PRED32; ++w) sj[u][w] = make_float4(0.f, 0.f, 0.f, 0.f);
          }
        }
        load_ids(q0 + IRR_U * G);
        float f[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};   // at most IRR_U pairs in FP32
#pragma unroll
        for (int u = 0; u < IRR_U; ++u) {
          if (jv[u] < 0) continue;
          const int j = jv[u];
          // double-single difference: (hi_j - hi_i) + (lo_j - lo_i)
          const float dx =
              __fadd_rn(__fsub_rn(sj[u][0].x, si[0].x), __fsub_rn(sj[u][1].x, si[1].x));
          const float dy =
              __fadd_rn(__fsub_rn(sj[u][0].y, si[0].y), __fsub_rn(sj[u][1].y, si[1].y));
          const float dz =
              __fadd_rn(__fsub_rn(sj[u][0].z, si[0].z), __fsub_rn(sj[u][1].z, si[1].z));
          const float dvx = __fsub_rn(sj[u][2].x, si[2].x);
          const float dvy = __fsub_rn(sj[u][2].y, si[2].y);
          const float dvz = __fsub_rn(sj[u][2].z, si[2].z);
          const float r2 = fmaf(dz, dz, fmaf(dy, dy, __fmul_rn(dx, dx)));
          if (r2 < best || (r2 == best && j < bj)) {
            best = r2;
            bj = j;
          }
          if (r2 >= 0x1p-126f) {
            // rsqrt estimate, one Newton step in residual form:
            // e = r2 y0^2 - 1, 1/r = y0 - y0 e / 2 (one rounding in the last FMA)
            const float y0 = rsqrt_est(r2);
            const float e = fmaf(__fmul_rn(r2, y0), y0, -1.0f);
            const float rinv = fmaf(__fmul_rn(-0.5f, y0), e, y0);
            const float rinv2 = __fmul_rn(rinv, rinv);
            const float mr3 = __fmul_rn(__fmul_rn(sj[u][0].w, rinv), rinv2);
            const float rv = fmaf(dz, dvz, fmaf(dy, dvy, __fmul_rn(dx, dvx)));
            const float al = __fmul_rn(-3.0f * rv, rinv2);
            f[0] = fmaf(mr3, dx, f[0]);
            f[1] = fmaf(mr3, dy, f[1]);
            f[2] = fmaf(mr3, dz, f[2]);
            f[3] = fmaf(mr3, fmaf(al, dx, dvx), f[3]);
            f[4] = fmaf(mr3, fmaf(al, dy, dvy), f[4]);
            f[5] = fmaf(mr3, fmaf(al, dz, dvz), f[5]);
          }
        }
#pragma unroll
        for (int c = 0; c < 6; ++c) ff_accum(hi[c], lo[c], f[c]);
      }
    }
    // fixed float-float butterfly within the particle's lanes (deterministic)
    for (int o = G / 2; o > 0; o >>= 1) {
#pragma unroll
      for (int c = 0; c < 6; ++c) {
        const float oh = __shfl_xor_sync(0xffffffffu, hi[c], o);
        const float ol = __shfl_xor_sync(0xffffffffu, lo[c], o);
        ff_add(hi[c], lo[c], oh, ol);
      }
      const float ob = __shfl_xor_sync(0xffffffffu, best, o);
      const int oj = __shfl_xor_sync(0xffffffffu, bj, o);
      if (ob < best || (ob == best && oj < bj)) {
        best = ob;
        bj = oj;
      }
    }
    // every lane of the particle now holds its sums: lane c < 6 converts and
    // stores component c (one warp-wide conversion instead of six per
    // particle on the FP64 pipe), lane 6 the nearest neighbour
    if (k < ni) {
      float h = hi[0], l = lo[0];
#pragma unroll
      for (int c = 1; c < 6; ++c)
        if (sub == c) {
          h = hi[c];
          l = lo[c];
        }
      if (sub < 3) acc[3 * (size_t)k + sub] = (double)h + (double)l;
      else if (sub < 6) jrk[3 * (size_t)k + sub - 3] = (double)h + (double)l;
      else if (sub == 6) nnbid[k] = (bj == INT_MAX) ? 0 : bj + 1;
    }
  }
}

// ---------------------------------------------------------------------------
// Double-float precision (irr_set_precision(2), the default): FP64-class results from the
// FP32 pipe.  Every quantity is an unevaluated sum hi + lo of two floats
// (about 48 significant bits) and every operation an error-free transform
// (Knuth's TwoSum, the FMA product error) followed by renormalisation, the
// classic double-single arithmetic of Dekker (1971; df_* in common.cuh), so
// that a pair costs ~530 instructions on the FP32 pipe instead of ~40 on the
// FP64 pipe: on GB300, whose FP64 pipe runs at 1/64 of the FP32 rate, 4.2x
// faster, at a relative error near 1e-13 per term.  Positions, velocities and masses are the
// double-single split of the FP64 prediction (4 float4 = 64 bytes per
// particle, two sectors when gathered); 1/r is the hardware estimate refined
// by one Newton step carried in double-float (error ~2^-45).
constexpr int PREDDF = 4;   // float4 per particle
constexpr int IRRDF_U = 2;  // listings per lane in flight

__device__ __forceinline__ void split_state_df(const double x[3], const double v[3], double m,
                                               float4 s[PREDDF]) {
  float xh[3], xl[3], vh[3], vl[3], mh, ml;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    ds_split(x[c], xh[c], xl[c]);
    ds_split(v[c], vh[c], vl[c]);
  }
  ds_split(m, mh, ml);
  s[0] = make_float4(xh[0], xh[1], xh[2], mh);
  s[1] = make_float4(xl[0], xl[1], xl[2], ml);
  s[2] = make_float4(vh[0], vh[1], vh[2], 0.f);
  s[3] = make_float4(vl[0], vl[1], vl[2], 0.f);
}

__global__ void irr_preddf_kernel(int n, const double *__restrict__ rec, double ti,
                                  float4 *__restrict__ pred) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double x[3], v[3], m;
  predict(rec + (size_t)i * REC, ti, x, v, m);
  float4 s[PREDDF];
  split_state_df(x, v, m, s);
#pragma unroll
  for (int u = 0; u < PREDDF; ++u) pred[(size_t)i * PREDDF + u] = s[u];
}

template <bool PRE>
__device__ __forceinline__ void statedf(const double *__restrict__ rec,
                                        const float4 *__restrict__ pred, int i, double ti,
                                        float4 s[PREDDF]) {
  if (PRE) {
#pragma unroll
    for (int u = 0; u < PREDDF; ++u) s[u] = __ldg(pred + (size_t)i * PREDDF + u);
  } else {
    double x[3], v[3], m;
    predict(rec + (size_t)i * REC, ti, x, v, m);
    split_state_df(x, v, m, s);
  }
}

// Same contract as irr_firr_kernel.  Bodies closer than 1e-19 (r^2 below the
// smallest normal float), the particle itself included, add nothing; the
// nearest neighbour is chosen on the double-float r^2 (ties to the smaller
// id).
template <bool PRE, int G>
__global__ void __launch_bounds__(32 * IRR32_WARPS)
    irr_firrdf_kernel(int n, const double *__restrict__ rec, const float4 *__restrict__ pred,
                      int lmax, const int *__restrict__ lists, double ti, int ni,
                      const int *__restrict__ addr, int base, double *__restrict__ acc,
                      double *__restrict__ jrk, int *__restrict__ nnbid, int *__restrict__ err,
                      unsigned long long *__restrict__ inter) {
  const int lane = threadIdx.x & 31, sub = lane & (G - 1);
  const int nwarps = (int)((gridDim.x * blockDim.x) >> 5);
  const int warp = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  for (int k0 = warp * (32 / G); k0 < ni; k0 += nwarps * (32 / G)) {
    const int k = k0 + lane / G;
    dfl sum[6];
#pragma unroll
    for (int c = 0; c < 6; ++c) sum[c] = {0.f, 0.f};
    dfl best = {INFINITY, 0.f};
    int bj = INT_MAX;
    const int i = k < ni ? addr[k] - base : 0;
    if (k < ni && (i < 0 || i >= n)) {
      if (sub == 0) flag(err, GPUNB_E_ARG);
    } else if (k < ni) {
      float4 si[PREDDF];
      statedf<PRE>(rec, pred, i, ti, si);
      const int *row = lists + (size_t)i * lmax;
      int nnb = row[0];
      if (nnb < 0 || nnb > lmax - 1) {
        if (sub == 0) flag(err, GPUNB_E_ARG);
        nnb = 0;
      }
      if (inter && sub == 0 && nnb > 0) atomicAdd(inter, (unsigned long long)nnb);
      for (int q0 = sub; q0 < nnb; q0 += IRRDF_U * G) {
        int jv[IRRDF_U];
#pragma unroll
        for (int u = 0; u < IRRDF_U; ++u) {
          const int q = q0 + u * G;
          jv[u] = q < nnb ? __ldg(row + 1 + q) : -1;
          if (q < nnb && (jv[u] < 0 || jv[u] >= n)) {
            flag(err, GPUNB_E_ARG);
            jv[u] = -1;
          }
        }
        float4 sj[IRRDF_U][PREDDF];
#pragma unroll
        for (int u = 0; u < IRRDF_U; ++u) {
          if (jv[u] >= 0) {
            statedf<PRE>(rec, pred, jv[u], ti, sj[u]);
          } else {
#pragma unroll
            for (int w = 0; w < PREDDF; ++w) sj[u][w] = make_float4(0.f, 0.f, 0.f, 0.f);
          }
        }
#pragma unroll
        for (int u = 0; u < IRRDF_U; ++u) {
          if (jv[u] < 0) continue;
          const int j = jv[u];
          const dfl dx = df_diff(sj[u][0].x, sj[u][1].x, si[0].x, si[1].x);
          const dfl dy = df_diff(sj[u][0].y, sj[u][1].y, si[0].y, si[1].y);
          const dfl dz = df_diff(sj[u][0].z, sj[u][1].z, si[0].z, si[1].z);
          const dfl r2 = df_add(df_add(df_sqr(dx), df_sqr(dy)), df_sqr(dz));
          if (r2.h < best.h || (r2.h == best.h && (r2.l < best.l || (r2.l == best.l && j < bj)))) {
            best = r2;
            bj = j;
          }
          if (r2.h < 0x1p-126f) continue;
          const dfl dvx = df_diff(sj[u][2].x, sj[u][3].x, si[2].x, si[3].x);
          const dfl dvy = df_diff(sj[u][2].y, sj[u][3].y, si[2].y, si[3].y);
          const dfl dvz = df_diff(sj[u][2].z, sj[u][3].z, si[2].z, si[3].z);
          // 1/r: estimate y0, then y0 (1 + (1 - r2 y0^2) / 2) with r2 y0^2 in double-float
          const float y0 = rsqrt_est(r2.h);
          const float q = __fmul_rn(y0, y0);
          const dfl t = df_mul(r2, {q, fmaf(y0, y0, -q)});
          const float e = __fsub_rn(__fsub_rn(1.0f, t.h), t.l);
          const dfl rinv = df_fast(y0, __fmul_rn(__fmul_rn(0.5f, y0), e));
          const dfl rinv2 = df_sqr(rinv);
          const dfl mr3 = df_mul(df_mul({sj[u][0].w, sj[u][1].w}, rinv), rinv2);
          const dfl rv = df_add(df_add(df_mul(dx, dvx), df_mul(dy, dvy)), df_mul(dz, dvz));
          const dfl al = df_mulf(df_mul(rv, rinv2), -3.0f);
          sum[0] = df_add(sum[0], df_mul(mr3, dx));
          sum[1] = df_add(sum[1], df_mul(mr3, dy));
          sum[2] = df_add(sum[2], df_mul(mr3, dz));
          sum[3] = df_add(sum[3], df_mul(mr3, df_add(dvx, df_mul(al, dx))));
          sum[4] = df_add(sum[4], df_mul(mr3, df_add(dvy, df_mul(al, dy))));
          sum[5] = df_add(sum[5], df_mul(mr3, df_add(dvz, df_mul(al, dz))));
        }
      }
    }
    // fixed double-float butterfly within the particle's lanes (deterministic)
    for (int o = G / 2; o > 0; o >>= 1) {
#pragma unroll
      for (int c = 0; c < 6; ++c) {
        const dfl other = {__shfl_xor_sync(0xffffffffu, sum[c].h, o),
                           __shfl_xor_sync(0xffffffffu, sum[c].l, o)};
        sum[c] = df_add(sum[c], other);
      }
      const float obh = __shfl_xor_sync(0xffffffffu, best.h, o);
      const float obl = __shfl_xor_sync(0xffffffffu, best.l, o);
      const int oj = __shfl_xor_sync(0xffffffffu, bj, o);
      if (obh < best.h || (obh == best.h && (obl < best.l || (obl == best.l && oj < bj)))) {
        best = {obh, obl};
        bj = oj;
      }
    }
    // lane c < 6 converts and stores component c, lane 6 the nearest neighbour
    if (k < ni) {
      dfl v = sum[0];
#pragma unroll
      for (int c = 1; c < 6; ++c)
        if (sub == c) v = sum[c];
      if (sub < 3) acc[3 * (size_t)k + sub] = (double)v.h + (double)v.l;
      else if (sub < 6) jrk[3 * (size_t)k + sub - 3] = (double)v.h + (double)v.l;
      else if (sub == 6) nnbid[k] = (bj == INT_MAX) ? 0 : bj + 1;
    }
  }
}

// changed records: rec[idx[r]] = src record r (thread per double)
__global__ void irr_put_rec_kernel(int k, const int *__restrict__ idx,
                                   const double *__restrict__ src, int src_by_index,
                                   double *__restrict__ rec) {
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (size_t)k * REC) return;
  const int r = (int)(t / REC), f = (int)(t % REC);
  const int a = idx[r];
  rec[(size_t)a * REC + f] = src_by_index ? src[(size_t)a * REC + f] : src[t];
}

// changed list rows: warp per row; staged rows are packed (count + ids, at
// off[r]), mirrored rows are read at a * lmax
__global__ void irr_put_rows_kernel(int k, const int *__restrict__ idx,
                                    const int *__restrict__ off, const int *__restrict__ src,
                                    int src_by_index, int lmax, int *__restrict__ lists) {
  const int lane = threadIdx.x & 31;
  const int r = (int)(((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  if (r >= k) return;
  const int a = idx[r];
  const int *s = src_by_index ? src + (size_t)a * lmax : src + off[r];
  const int len = 1 + s[0];
  int *d = lists + (size_t)a * lmax;
  for (int u = lane; u < len && u < lmax; u += 32) d[u] = s[u];
}

// Predicted positions and velocities of particles a0 .. a0+n-1 at ti, in the
// arrays of a j-set upload (xbpredall.f:16-27: X = ((FDOT S + F) S + X0DOT) S
// + X0, XDOT = (1.5 FDOT S + F) 2 S + X0DOT, with F and FDOT as stored).
__global__ void irr_predict_all_kernel(const double *__restrict__ rec, int a0, int n, double ti,
                                       double *__restrict__ x, double *__restrict__ v) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  double xp[3], vp[3], m;
  predict(rec + (size_t)(a0 + k) * REC, ti, xp, vp, m);
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    x[3 * (size_t)k + c] = xp[c];
    v[3 * (size_t)k + c] = vp[c];
  }
}

// ---------------------------------------------------------------------------
// host

struct DevBuf {
  void *p = nullptr;
  size_t bytes = 0;
  bool ensure(size_t b) {
    if (b <= bytes) return true;
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
    if (cudaMalloc(&p, b) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    bytes = b;
    return true;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  template <class T> T *as() const { return (T *)p; }
};

struct PinBuf {
  void *p = nullptr;
  size_t bytes = 0;
  bool ensure(size_t b) {
    if (b <= bytes) return true;
    if (p) cudaFreeHost(p);
    p = nullptr;
    bytes = 0;
    if (cudaHostAlloc(&p, b, cudaHostAllocDefault) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    bytes = b;
    return true;
  }
  void release() {
    if (p) cudaFreeHost(p);
    p = nullptr;
    bytes = 0;
  }
  template <class T> T *as() const { return (T *)p; }
};

struct State {
  std::mutex mu;                 // open/close/force calls
  bool open = false;
  int nmax = 0, lmax = 0, rank = 0;
  int direct = 0;                // device reads/writes host memory coherently
  int precision = 2;             // 2 = double-float (default), 1 = FP64, 0 = split FP32
  cudaStream_t st = nullptr;
  std::vector<double> rec_h;     // host mirror of the records
  std::vector<int> list_h;       // host mirror of the rows (0-based ids)
  std::vector<int> dirty_rec, dirty_row;
  std::atomic<long long> n_rec{0}, n_row{0};
  std::vector<unsigned> seen;    // epoch stamps for de-duplication
  unsigned epoch = 0;
  std::vector<int> uniq;
  DevBuf rec_d, list_d, addr_d, out_d, nid_d, idx_d, stage_d, off_d, err_d, pm_d, px_d, pv_d;
  DevBuf pred_d;   // predicted states of all particles (large blocks; 64 B each)
  DevBuf pred_dev_d;   // the same for the device-resident form
  PinBuf stage_h, idx_h, off_h, err_h;
  double time_grav = 0.0;
  unsigned long long num_inter = 0, num_fcall = 0, num_steps = 0;
};

static State S;
static std::mutex s_err_mu;

static void failf(int code, const char *fmt, ...) {
  char buf[384];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  std::lock_guard<std::mutex> lk(s_err_mu);
  report_failure(code, buf);
}

#define IRR_CUDA(call, ret)                                                         \
  do {                                                                              \
    cudaError_t e_ = (call);                                                        \
    if (e_ != cudaSuccess) {                                                        \
      failf(GPUNB_E_CUDA, "irr: %s failed: %s", #call, cudaGetErrorString(e_));     \
      return ret;                                                                   \
    }                                                                               \
  } while (0)

static double wtime() {
  struct timeval tv;
  gettimeofday(&tv, nullptr);
  return tv.tv_sec + 1.e-6 * tv.tv_usec;
}

static void release_all() {
  for (DevBuf *b : {&S.rec_d, &S.list_d, &S.addr_d, &S.out_d, &S.nid_d, &S.idx_d, &S.stage_d,
                    &S.off_d, &S.err_d, &S.pm_d, &S.px_d, &S.pv_d, &S.pred_d, &S.pred_dev_d})
    b->release();
  for (PinBuf *b : {&S.stage_h, &S.idx_h, &S.off_h, &S.err_h}) b->release();
  S.rec_h.clear();
  S.rec_h.shrink_to_fit();
  S.list_h.clear();
  S.list_h.shrink_to_fit();
}

// the distinct particles of a dirty list (the mirror holds their last values)
static int dedup(const std::vector<int> &dirty, long long count) {
  if (++S.epoch == 0) {
    std::fill(S.seen.begin(), S.seen.end(), 0u);
    S.epoch = 1;
  }
  S.uniq.clear();
  for (long long q = 0; q < count; ++q) {
    const int a = dirty[(size_t)q];
    if (S.seen[a] != S.epoch) {
      S.seen[a] = S.epoch;
      S.uniq.push_back(a);
    }
  }
  return (int)S.uniq.size();
}

// upload what set_jp / set_list changed since the last force call
static bool upload() {
  cudaStream_t st = S.st;
  const size_t cap = S.dirty_rec.size();
  const long long nr = S.n_rec.exchange(0), nl = S.n_row.exchange(0);
  if (nr > 0) {
    if ((size_t)nr > cap) {
      IRR_CUDA(cudaMemcpyAsync(S.rec_d.p, S.rec_h.data(), S.rec_h.size() * sizeof(double),
                               cudaMemcpyHostToDevice, st), false);
    } else {
      const int k = dedup(S.dirty_rec, nr);
      if (!S.idx_d.ensure((size_t)k * sizeof(int)) || !S.idx_h.ensure((size_t)k * sizeof(int))) {
        failf(GPUNB_E_ALLOC, "irr: staging allocation failed");
        return false;
      }
      memcpy(S.idx_h.p, S.uniq.data(), (size_t)k * sizeof(int));
      IRR_CUDA(cudaMemcpyAsync(S.idx_d.p, S.idx_h.p, (size_t)k * sizeof(int),
                               cudaMemcpyHostToDevice, st), false);
      const double *src;
      int by_index;
      if (S.direct) {
        src = S.rec_h.data();   // read in place through the coherent host path
        by_index = 1;
      } else {
        if (!S.stage_h.ensure((size_t)k * REC * sizeof(double)) ||
            !S.stage_d.ensure((size_t)k * REC * sizeof(double))) {
          failf(GPUNB_E_ALLOC, "irr: staging allocation failed");
          return false;
        }
        double *h = S.stage_h.as<double>();
        for (int r = 0; r < k; ++r)
          memcpy(h + (size_t)r * REC, S.rec_h.data() + (size_t)S.uniq[r] * REC,
                 REC * sizeof(double));
        IRR_CUDA(cudaMemcpyAsync(S.stage_d.p, h, (size_t)k * REC * sizeof(double),
                                 cudaMemcpyHostToDevice, st), false);
        src = S.stage_d.as<double>();
        by_index = 0;
      }
      const size_t threads = (size_t)k * REC;
      irr_put_rec_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(
          k, S.idx_d.as<int>(), src, by_index, S.rec_d.as<double>());
      IRR_CUDA(cudaGetLastError(), false);
      // the index buffer is reused below: wait until this kernel has read it
      if (nl > 0) IRR_CUDA(cudaStreamSynchronize(st), false);
    }
  }
  if (nl > 0) {
    if ((size_t)nl > cap) {
      IRR_CUDA(cudaMemcpyAsync(S.list_d.p, S.list_h.data(), S.list_h.size() * sizeof(int),
                               cudaMemcpyHostToDevice, st), false);
    } else {
      const int k = dedup(S.dirty_row, nl);
      if (!S.idx_d.ensure((size_t)k * sizeof(int)) || !S.idx_h.ensure((size_t)k * sizeof(int)) ||
          !S.off_d.ensure((size_t)(k + 1) * sizeof(int)) ||
          !S.off_h.ensure((size_t)(k + 1) * sizeof(int))) {
        failf(GPUNB_E_ALLOC, "irr: staging allocation failed");
        return false;
      }
      memcpy(S.idx_h.p, S.uniq.data(), (size_t)k * sizeof(int));
      IRR_CUDA(cudaMemcpyAsync(S.idx_d.p, S.idx_h.p, (size_t)k * sizeof(int),
                               cudaMemcpyHostToDevice, st), false);
      const int *src;
      int by_index;
      if (S.direct) {
        src = S.list_h.data();
        by_index = 1;
      } else {
        int *off = S.off_h.as<int>();
        size_t tot = 0;
        for (int r = 0; r < k; ++r) {
          off[r] = (int)tot;
          tot += 1 + (size_t)S.list_h[(size_t)S.uniq[r] * S.lmax];
        }
        off[k] = (int)tot;
        if (!S.stage_h.ensure(tot * sizeof(int)) || !S.stage_d.ensure(tot * sizeof(int))) {
          failf(GPUNB_E_ALLOC, "irr: staging allocation failed");
          return false;
        }
        int *h = S.stage_h.as<int>();
        for (int r = 0; r < k; ++r) {
          const int *row = S.list_h.data() + (size_t)S.uniq[r] * S.lmax;
          memcpy(h + off[r], row, (size_t)(1 + row[0]) * sizeof(int));
        }
        IRR_CUDA(cudaMemcpyAsync(S.off_d.p, off, (size_t)(k + 1) * sizeof(int),
                                 cudaMemcpyHostToDevice, st), false);
        IRR_CUDA(cudaMemcpyAsync(S.stage_d.p, h, tot * sizeof(int), cudaMemcpyHostToDevice, st),
                 false);
        src = S.stage_d.as<int>();
        by_index = 0;
      }
      const size_t threads = (size_t)k * 32;
      irr_put_rows_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(
          k, S.idx_d.as<int>(), S.off_d.as<int>(), src, by_index, S.lmax, S.list_d.as<int>());
      IRR_CUDA(cudaGetLastError(), false);
    }
  }
  return true;
}

// pred: scratch of n * PRED doubles (64 bytes per particle, which also holds
// the 48-byte split and 64-byte double-float states).  Blocks of at least n/32 particles predict every
// particle once first (with ~100 neighbours each, the lists then name every
// particle several times); smaller ones predict per listing.  prec: 0 = split
// FP32, 1 = FP64.
static int launch_firr(int n, const double *rec, double *pred, int prec, int lmax,
                       const int *lists, double ti, int ni, const int *addr, int base,
                       double *acc, double *jrk, int *nnbid, int *err,
                       unsigned long long *inter, cudaStream_t st) {
  if (ni <= 0) return GPUNB_OK;
  const bool wide = ni < IRR_G_MIN_NI;   // 32 lanes per particle
  const int warps = prec == 1 ? IRR_WARPS : IRR32_WARPS;
  const int per_block = warps * (wide ? 1 : 32 / IRR_G);   // particles per block and pass
  const unsigned blocks =
      (unsigned)std::min<long long>((ni + per_block - 1) / per_block, 1ll << 20);
  const unsigned th = 32 * warps;
  const bool whole = pred && 32ll * ni >= n;
  if (prec == 1) {
    if (whole) irr_pred_kernel<<<(n + 255) / 256, 256, 0, st>>>(n, rec, ti, pred);
    const double *p = whole ? pred : nullptr;
    if (whole && wide)
      irr_firr_kernel<true, 32><<<blocks, th, 0, st>>>(n, rec, p, lmax, lists, ti, ni, addr,
                                                        base, acc, jrk, nnbid, err, inter);
    else if (whole)
      irr_firr_kernel<true, IRR_G><<<blocks, th, 0, st>>>(n, rec, p, lmax, lists, ti, ni, addr,
                                                           base, acc, jrk, nnbid, err, inter);
    else if (wide)
      irr_firr_kernel<false, 32><<<blocks, th, 0, st>>>(n, rec, p, lmax, lists, ti, ni, addr,
                                                         base, acc, jrk, nnbid, err, inter);
    else
      irr_firr_kernel<false, IRR_G><<<blocks, th, 0, st>>>(n, rec, p, lmax, lists, ti, ni, addr,
                                                            base, acc, jrk, nnbid, err, inter);
  } else if (prec == 2) {
    float4 *pdf = whole ? reinterpret_cast<float4 *>(pred) : nullptr;
    if (whole) irr_preddf_kernel<<<(n + 255) / 256, 256, 0, st>>>(n, rec, ti, pdf);
    if (whole && wide)
      irr_firrdf_kernel<true, 32><<<blocks, th, 0, st>>>(n, rec, pdf, lmax, lists, ti, ni, addr,
                                                          base, acc, jrk, nnbid, err, inter);
    else if (whole)
      irr_firrdf_kernel<true, IRR_G><<<blocks, th, 0, st>>>(n, rec, pdf, lmax, lists, ti, ni,
                                                             addr, base, acc, jrk, nnbid, err,
                                                             inter);
    else if (wide)
      irr_firrdf_kernel<false, 32><<<blocks, th, 0, st>>>(n, rec, pdf, lmax, lists, ti, ni,
                                                           addr, base, acc, jrk, nnbid, err,
                                                           inter);
    else
      irr_firrdf_kernel<false, IRR_G><<<blocks, th, 0, st>>>(n, rec, pdf, lmax, lists, ti, ni,
                                                              addr, base, acc, jrk, nnbid, err,
                                                              inter);
  } else {
    float4 *p32 = whole ? reinterpret_cast<float4 *>(pred) : nullptr;
    if (whole) irr_pred32_kernel<<<(n + 255) / 256, 256, 0, st>>>(n, rec, ti, p32);
    if (whole && wide)
      irr_firr32_kernel<true, 32><<<blocks, th, 0, st>>>(n, rec, p32, lmax, lists, ti, ni, addr,
                                                          base, acc, jrk, nnbid, err, inter);
    else if (whole)
      irr_firr32_kernel<true, IRR_G><<<blocks, th, 0, st>>>(n, rec, p32, lmax, lists, ti, ni,
                                                             addr, base, acc, jrk, nnbid, err,
                                                             inter);
    else if (wide)
      irr_firr32_kernel<false, 32><<<blocks, th, 0, st>>>(n, rec, p32, lmax, lists, ti, ni,
                                                           addr, base, acc, jrk, nnbid, err,
                                                           inter);
    else
      irr_firr32_kernel<false, IRR_G><<<blocks, th, 0, st>>>(n, rec, p32, lmax, lists, ti, ni,
                                                              addr, base, acc, jrk, nnbid, err,
                                                              inter);
  }
  return cudaGetLastError() == cudaSuccess ? GPUNB_OK : GPUNB_E_CUDA;
}

static void open_lib(int nmax, int lmax, int rank) {
  std::lock_guard<std::mutex> lk(S.mu);
  if (S.open) {
    fprintf(stderr, "irr_simd: it is already open\n");
    return;
  }
  if (nmax < 0 || lmax < 1 || lmax > (1 << 16)) {
    failf(GPUNB_E_ARG, "irr_simd_open_: need nmax >= 0 and 1 <= lmax <= 65536 (got %d, %d)",
          nmax, lmax);
    return;
  }
  int r = rank;
  gpunb_devinit_(&r);
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    failf(GPUNB_E_NO_DEVICE, "irr_simd_open_: no CUDA device");
    return;
  }
  if (!S.st) IRR_CUDA(cudaStreamCreateWithFlags(&S.st, cudaStreamNonBlocking), );
  int pageable = 0, host_tables = 0;
  if (cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables,
                             dev) != cudaSuccess) {
    cudaGetLastError();
    pageable = host_tables = 0;
  }
  S.direct = (pageable && host_tables) ? 1 : 0;
  if (const char *p = getenv("GPUNB_HOST_DIRECT")) S.direct &= (atoi(p) != 0);
  if (const char *p = getenv("GPUNB_IRR_PRECISION")) {
    const int v = atoi(p);
    S.precision = (v == 0 || v == 1) ? v : 2;
  }
  const size_t n = (size_t)std::max(nmax, 1);
  S.nmax = nmax;
  S.lmax = lmax;
  S.rank = rank;
  S.rec_h.assign(n * REC, 0.0);
  S.list_h.assign(n * (size_t)lmax, 0);
  S.dirty_rec.assign(2 * n, 0);
  S.dirty_row.assign(2 * n, 0);
  S.n_rec = 0;
  S.n_row = 0;
  S.seen.assign(n, 0u);
  S.epoch = 0;
  if (!S.rec_d.ensure(n * REC * sizeof(double)) ||
      !S.list_d.ensure(n * (size_t)lmax * sizeof(int)) || !S.err_d.ensure(kStatusBytes) ||
      !S.err_h.ensure(kStatusBytes)) {
    failf(GPUNB_E_ALLOC, "irr_simd_open_: device allocation for nmax = %d, lmax = %d failed",
          nmax, lmax);
    release_all();
    return;
  }
  IRR_CUDA(cudaMemsetAsync(S.rec_d.p, 0, n * REC * sizeof(double), S.st), );
  IRR_CUDA(cudaMemsetAsync(S.list_d.p, 0, n * (size_t)lmax * sizeof(int), S.st), );
  IRR_CUDA(cudaStreamSynchronize(S.st), );
  S.time_grav = 0.0;
  S.num_inter = S.num_fcall = S.num_steps = 0;
  S.open = true;
  fprintf(stderr, "# Opening IRR_simd lib. GPU ver. - rank: %d; nmax: %d, lmax: %d\n", rank, nmax,
          lmax);
}

static void close_lib(int rank) {
  std::lock_guard<std::mutex> lk(S.mu);
  if (!S.open) {
    fprintf(stderr, "irr_simd: it is already close\n");
    return;
  }
  if (S.st) cudaStreamSynchronize(S.st);
  release_all();
  S.open = false;
  fprintf(stderr, "Closing IRR_simd lib. GPU ver. - rank: %d\n", rank);
}

static void profile(int rank) {
  std::lock_guard<std::mutex> lk(S.mu);
  if (!S.open) return;
  const double gflops = S.time_grav > 0 ? 60.0 * (double)S.num_inter * 1.e-9 / S.time_grav : 0.0;
  const double usec = S.num_fcall ? 1.e6 * (S.time_grav / (double)S.num_fcall) : 0.0;
  const double nnb_avr = S.num_steps ? (double)S.num_inter / (double)S.num_steps : 0.0;
  const int ni_avr = S.num_fcall ? (int)(S.num_inter / S.num_fcall) : 0;
  fprintf(stderr,
          "[R.%d GPU Irr.F ] Ncall: %llu <NI>: %d <NB>: %f grav: %f s, %f Gflops, %f usec\n",
          rank, S.num_fcall, ni_avr, nnb_avr, S.time_grav, gflops, usec);
  S.time_grav = 0.0;
  S.num_inter = S.num_fcall = S.num_steps = 0;
}

static void set_jp(int addr, const double *pos, const double *vel, const double *acc2,
                   const double *jrk6, double mass, double time) {
  if (!S.open) {
    failf(GPUNB_E_NOT_OPEN, "irr_simd_set_jp_ called before irr_simd_open_");
    return;
  }
  const int a = addr - 1;
  if (a < 0 || a >= S.nmax) {
    failf(GPUNB_E_ARG, "irr_simd_set_jp_: address %d outside [1, %d]", addr, S.nmax);
    return;
  }
  double *r = S.rec_h.data() + (size_t)a * REC;
  r[0] = pos[0]; r[1] = pos[1]; r[2] = pos[2]; r[3] = mass;
  r[4] = vel[0]; r[5] = vel[1]; r[6] = vel[2]; r[7] = time;
  r[8] = acc2[0]; r[9] = acc2[1]; r[10] = acc2[2]; r[11] = 0.0;
  r[12] = jrk6[0]; r[13] = jrk6[1]; r[14] = jrk6[2]; r[15] = 0.0;
  const long long q = S.n_rec.fetch_add(1);
  if ((size_t)q < S.dirty_rec.size()) S.dirty_rec[(size_t)q] = a;
}

static void set_list(int addr, const int *nblist) {
  if (!S.open) {
    failf(GPUNB_E_NOT_OPEN, "irr_simd_set_list_ called before irr_simd_open_");
    return;
  }
  const int a = addr - 1;
  if (a < 0 || a >= S.nmax) {
    failf(GPUNB_E_ARG, "irr_simd_set_list_: address %d outside [1, %d]", addr, S.nmax);
    return;
  }
  const int nnb = nblist[0];
  if (nnb < 0 || nnb > S.lmax - 1) {
    failf(GPUNB_E_ARG, "irr_simd_set_list_: %d neighbours for lmax = %d", nnb, S.lmax);
    return;
  }
  int *row = S.list_h.data() + (size_t)a * S.lmax;
  row[0] = nnb;
  for (int k = 0; k < nnb; ++k) row[1 + k] = nblist[1 + k] - 1;
  const long long q = S.n_row.fetch_add(1);
  if ((size_t)q < S.dirty_row.size()) S.dirty_row[(size_t)q] = a;
}

static void firr_vec(double ti, int ni, const int *addr, double (*acc)[3], double (*jrk)[3],
                     int *nnbid) {
  std::lock_guard<std::mutex> lk(S.mu);
  if (!S.open) {
    failf(GPUNB_E_NOT_OPEN, "irr_simd_firr_vec_ called before irr_simd_open_");
    return;
  }
  if (ni <= 0) return;
  const double t0 = wtime();
  cudaStream_t st = S.st;
  if (!upload()) return;
  IRR_CUDA(cudaMemsetAsync(S.err_d.p, 0, kStatusBytes, st), );
  unsigned long long *inter_d = (unsigned long long *)((char *)S.err_d.p + 8);
  double *pred = nullptr;
  if (32ll * ni >= S.nmax) {
    if (!S.pred_d.ensure((size_t)S.nmax * PRED * sizeof(double))) {
      failf(GPUNB_E_ALLOC, "irr: prediction buffer allocation failed");
      return;
    }
    pred = S.pred_d.as<double>();
  }
  if (!S.addr_d.ensure((size_t)ni * sizeof(int)) ||
      !S.out_d.ensure((size_t)ni * 6 * sizeof(double)) ||
      !S.nid_d.ensure((size_t)ni * sizeof(int))) {
    failf(GPUNB_E_ALLOC, "irr: output allocation failed");
    return;
  }
  double *o = S.out_d.as<double>();
  int *herr = S.err_h.as<int>();
  if (S.direct) {
    // the device reads the address list and writes the results in host
    // memory itself, each with one coalesced copy kernel (the force kernel's
    // scattered per-particle stores would cross the host link one by one)
    HostCopyJobs in;
    in.count = 1;
    in.j[0] = HostCopyJob{addr, S.addr_d.p, ni, 4};
    IRR_CUDA(launch_host_copy(in, st), );
  } else {
    IRR_CUDA(cudaMemcpyAsync(S.addr_d.p, addr, (size_t)ni * sizeof(int), cudaMemcpyHostToDevice,
                             st), );
  }
  if (launch_firr(S.nmax, S.rec_d.as<double>(), pred, S.precision, S.lmax, S.list_d.as<int>(),
                  ti, ni, S.addr_d.as<int>(), 1, o, o + 3 * (size_t)ni, S.nid_d.as<int>(),
                  S.err_d.as<int>(), inter_d, st) != GPUNB_OK) {
    failf(GPUNB_E_CUDA, "irr: force kernel launch failed");
    return;
  }
  // results, the error word and the call's listed pairs (for
  // irr_simd_profile_)
  if (S.direct) {
    HostCopyJobs out;
    out.count = 4;
    out.j[0] = HostCopyJob{o, &acc[0][0], 3ll * ni, 8};
    out.j[1] = HostCopyJob{o + 3 * (size_t)ni, &jrk[0][0], 3ll * ni, 8};
    out.j[2] = HostCopyJob{S.nid_d.p, nnbid, ni, 4};
    out.j[3] = HostCopyJob{S.err_d.p, herr, (long long)(kStatusBytes / 8), 8};
    IRR_CUDA(launch_host_copy(out, st), );
  } else {
    IRR_CUDA(cudaMemcpyAsync(&acc[0][0], o, (size_t)ni * 3 * sizeof(double),
                             cudaMemcpyDeviceToHost, st), );
    IRR_CUDA(cudaMemcpyAsync(&jrk[0][0], o + 3 * (size_t)ni, (size_t)ni * 3 * sizeof(double),
                             cudaMemcpyDeviceToHost, st), );
    IRR_CUDA(cudaMemcpyAsync(nnbid, S.nid_d.p, (size_t)ni * sizeof(int), cudaMemcpyDeviceToHost,
                             st), );
    IRR_CUDA(cudaMemcpyAsync(herr, S.err_d.p, kStatusBytes, cudaMemcpyDeviceToHost, st), );
  }
  IRR_CUDA(cudaStreamSynchronize(st), );
  if (*herr) failf(*herr, "irr_simd_firr_vec_: an address or a listed id is out of range");
  const unsigned long long inter = *(const unsigned long long *)((const char *)S.err_h.p + 8);
  S.num_inter += inter;
  S.num_fcall++;
  S.num_steps += (unsigned long long)ni;
  S.time_grav += wtime() - t0;
}

static void send_predicted(int ifirst, int ntot, double ti, const double *body, double (*x)[3],
                           double (*xdot)[3]) {
  std::lock_guard<std::mutex> lk(S.mu);
  if (!S.open) {
    failf(GPUNB_E_NOT_OPEN, "gpunb_send_predicted_ needs the particle state of irr_simd_open_ "
                            "and irr_simd_set_jp_");
    return;
  }
  const int n = ntot - ifirst + 1;
  if (ifirst < 1 || n < 0 || ntot > S.nmax) {
    failf(GPUNB_E_ARG, "gpunb_send_predicted_: bodies %d..%d outside [1, %d]", ifirst, ntot,
          S.nmax);
    return;
  }
  cudaStream_t st = S.st;
  if (!upload()) return;
  if (!S.pm_d.ensure((size_t)std::max(n, 1) * sizeof(double)) ||
      !S.px_d.ensure((size_t)std::max(n, 1) * 3 * sizeof(double)) ||
      !S.pv_d.ensure((size_t)std::max(n, 1) * 3 * sizeof(double))) {
    failf(GPUNB_E_ALLOC, "gpunb_send_predicted_: device allocation failed");
    return;
  }
  if (n > 0) {
    IRR_CUDA(cudaMemcpyAsync(S.pm_d.p, body, (size_t)n * sizeof(double), cudaMemcpyHostToDevice,
                             st), );
    irr_predict_all_kernel<<<(n + 255) / 256, 256, 0, st>>>(S.rec_d.as<double>(), ifirst - 1, n,
                                                           ti, S.px_d.as<double>(),
                                                           S.pv_d.as<double>());
    IRR_CUDA(cudaGetLastError(), );
  }
  if (gpunb_send_device(n, S.pm_d.as<double>(), S.px_d.as<double>(), S.pv_d.as<double>(), st) !=
      GPUNB_OK)
    return;   // the engine has recorded the reason
  if (n > 0) {
    IRR_CUDA(cudaMemcpyAsync(&x[0][0], S.px_d.p, (size_t)n * 3 * sizeof(double),
                             cudaMemcpyDeviceToHost, st), );
    IRR_CUDA(cudaMemcpyAsync(&xdot[0][0], S.pv_d.p, (size_t)n * 3 * sizeof(double),
                             cudaMemcpyDeviceToHost, st), );
  }
  IRR_CUDA(cudaStreamSynchronize(st), );
}

}  // namespace irr
}  // namespace gpunb

using namespace gpunb::irr;

extern "C" {

void irr_simd_open_(int *nmax, int *lmax, int *rank) {
  open_lib(*nmax, *lmax, rank ? *rank : 0);
}

void irr_simd_close_(int *rank) { close_lib(rank ? *rank : 0); }

void irr_simd_profile_(int *rank) { profile(rank ? *rank : 0); }

void irr_simd_set_jp_(int *addr, double pos[3], double vel[3], double acc2[3], double jrk6[3],
                      double *mass, double *time) {
  set_jp(*addr, pos, vel, acc2, jrk6, *mass, *time);
}

void irr_simd_set_list_(int *addr, int *nblist) { set_list(*addr, nblist); }

void irr_simd_firr_vec_(double *ti, int *ni, int addr[], double acc[][3], double jrk[][3],
                        int nnbid[]) {
  firr_vec(*ti, *ni, addr, acc, jrk, nnbid);
}

void gpunb_send_predicted_(int *ifirst, int *ntot, double *time, double body[], double x[][3],
                           double xdot[][3]) {
  send_predicted(*ifirst, *ntot, *time, body, x, xdot);
}

int irr_set_host_path(int mode) {
  std::lock_guard<std::mutex> lk(S.mu);
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return -1;
  }
  int pageable = 0, host_tables = 0;
  if (cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables,
                             dev) != cudaSuccess) {
    cudaGetLastError();
    pageable = host_tables = 0;
  }
  S.direct = (mode != 0 && pageable && host_tables) ? 1 : 0;
  return S.direct;
}

int irr_firr_device(int n, const double *rec, int lmax, const int *lists, double ti, int ni,
                    const int *addr, double *acc, double *jrk, int *nnbid, void *stream) {
  if (n < 0 || lmax < 1 || ni < 0) return GPUNB_E_ARG;
  std::lock_guard<std::mutex> lk(S.mu);
  cudaStream_t st = stream ? (cudaStream_t)stream : S.st;
  // whole-set prediction into the library's buffer where it pays (as the
  // host form); without the buffer, per-listing prediction (the same bits)
  double *pred = nullptr;
  if (32ll * ni >= n && n > 0 && S.pred_dev_d.ensure((size_t)n * PRED * sizeof(double)))
    pred = S.pred_dev_d.as<double>();
  return launch_firr(n, rec, pred, S.precision, lmax, lists, ti, ni, addr, 0, acc, jrk, nnbid,
                     nullptr, nullptr, st);
}

int irr_set_precision(int mode) {
  std::lock_guard<std::mutex> lk(S.mu);
  S.precision = (mode == 0 || mode == 1) ? mode : 2;
  return S.precision;
}

}  // extern "C"
