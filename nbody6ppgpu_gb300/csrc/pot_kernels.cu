// Potential kernels for the energy check (gpupot_).
//
// Reference replaced: src/Main/gpupot.gpu.cu:32-57 (pot_kernel) and the
// host side of gpupot.gpu.cu:61-114.  Semantics: pot_i = sum over all j with
// r_ij^2 > 0 of m_j / r_ij (positive sign, no neighbour exclusion).
#include "common.cuh"
#include "launch.h"
#include "regf_kernels.cuh"

namespace gpunb {

constexpr int PJT = 128;
enum PField { P_XH = 0, P_YH, P_ZH, P_XL, P_YL, P_ZL, P_MN, P_NFIELD };
constexpr int PTILE_FLOATS = P_NFIELD * PJT;
constexpr int PTILE_BYTES = PTILE_FLOATS * 4;
static_assert(PTILE_BYTES % 16 == 0, "tile must be a multiple of 16 bytes");

__global__ void __launch_bounds__(PJT) pack_pot_tiles_kernel(const double *__restrict__ m,
                                                             const double *__restrict__ x, int n,
                                                             float *__restrict__ tiles,
                                                             int *err) {
  const int t = blockIdx.x, l = threadIdx.x, j = t * PJT + l;
  float *T = tiles + (size_t)t * PTILE_FLOATS;
  if (j < n) {
    const double x0 = x[3 * j], x1 = x[3 * j + 1], x2 = x[3 * j + 2], mj = m[j];
    if (isnan(x0) || isnan(x1) || isnan(x2) || isnan(mj)) raise_error(err, GPUNB_E_NAN);
    float h, lo;
    ds_split(x0, h, lo); T[P_XH * PJT + l] = h; T[P_XL * PJT + l] = lo;
    ds_split(x1, h, lo); T[P_YH * PJT + l] = h; T[P_YL * PJT + l] = lo;
    ds_split(x2, h, lo); T[P_ZH * PJT + l] = h; T[P_ZL * PJT + l] = lo;
    T[P_MN * PJT + l] = (float)(-0.5 * mj);
  } else {
    T[P_XH * PJT + l] = 1.0e15f; T[P_XL * PJT + l] = 0.f;
    T[P_YH * PJT + l] = 1.0e15f; T[P_YL * PJT + l] = 0.f;
    T[P_ZH * PJT + l] = 1.0e15f; T[P_ZL * PJT + l] = 0.f;
    T[P_MN * PJT + l] = -0.f;
  }
}

constexpr int PSTAGE = 4;

// Grid (ceil(ni / (32*IPT*WI)), S).  i = istart0 + local index (0-based).
template <int IPT, int WI>
__global__ void __launch_bounds__(32 * WI) pot_ds_kernel(const float *__restrict__ tiles,
                                                         int ntile, const double *__restrict__ x,
                                                         int istart0, int ni,
                                                         double *__restrict__ part, int ni_pad,
                                                         int *err) {
  constexpr int ITILE = 32 * IPT * WI;
  extern __shared__ __align__(128) float smem[];
  __shared__ __align__(8) uint64_t bar[PSTAGE];
  __shared__ int s_abort;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int ns = gridDim.y, sy = blockIdx.y;
  const int t0 = (int)(((long long)ntile * sy) / ns);
  const int t1 = (int)(((long long)ntile * (sy + 1)) / ns);
  const int nt = t1 - t0;
  if (tid == 0) {
    for (int s = 0; s < PSTAGE; ++s) mbar_init(&bar[s], 1);
    fence_mbar_init();
    s_abort = 0;
  }
  __syncthreads();
  if (tid == 0)
    for (int s = 0; s < PSTAGE && s < nt; ++s) {
      mbar_expect_tx(&bar[s], PTILE_BYTES);
      bulk_g2s(smem + s * PTILE_FLOATS, tiles + (size_t)(t0 + s) * PTILE_FLOATS, PTILE_BYTES,
               &bar[s]);
    }
  f2 nxh[IPT], nyh[IPT], nzh[IPT], nxl[IPT], nyl[IPT], nzl[IPT];
  f2 q[IPT];
  float hi[IPT], lo[IPT];
  int iloc[IPT];
#pragma unroll
  for (int k = 0; k < IPT; ++k) {
    const int il = blockIdx.x * ITILE + warp * 32 * IPT + k * 32 + lane;
    iloc[k] = il < ni ? il : -1;
    const int i = istart0 + (il < ni ? il : 0);
    float h, l;
    ds_split(x[3 * i], h, l); nxh[k] = mk2(-h); nxl[k] = mk2(-l);
    ds_split(x[3 * i + 1], h, l); nyh[k] = mk2(-h); nyl[k] = mk2(-l);
    ds_split(x[3 * i + 2], h, l); nzh[k] = mk2(-h); nzl[k] = mk2(-l);
    q[k] = make_float2(0.f, 0.f);
    hi[k] = lo[k] = 0.f;
  }
  int t = 0;
  for (; t < nt; ++t) {
    const int s = t % PSTAGE;
    if (!mbar_wait_bounded(&bar[s], (uint32_t)(t / PSTAGE) & 1u)) s_abort = 1;
    const float *T = smem + s * PTILE_FLOATS;
#pragma unroll 4
    for (int jj = 0; jj < PJT; jj += 2) {
      const f2 xh = *(const f2 *)(T + P_XH * PJT + jj);
      const f2 yh = *(const f2 *)(T + P_YH * PJT + jj);
      const f2 zh = *(const f2 *)(T + P_ZH * PJT + jj);
      const f2 xl = *(const f2 *)(T + P_XL * PJT + jj);
      const f2 yl = *(const f2 *)(T + P_YL * PJT + jj);
      const f2 zl = *(const f2 *)(T + P_ZL * PJT + jj);
      const f2 mn = *(const f2 *)(T + P_MN * PJT + jj);
#pragma unroll
      for (int k = 0; k < IPT; ++k) {
        const f2 dx = add2(add2(xh, nxh[k]), add2(xl, nxl[k]));
        const f2 dy = add2(add2(yh, nyh[k]), add2(yl, nyl[k]));
        const f2 dz = add2(add2(zh, nzh[k]), add2(zl, nzl[k]));
        const f2 r2 = fma2(dz, dz, fma2(dy, dy, mul2(dx, dx)));
        const f2 y0 = make_float2(rsqrt_est(r2.x), rsqrt_est(r2.y));
        f2 z = mul2(y0, fma2(mul2(r2, y0), y0, mk2(-3.0f)));   // -2/r
        z.x = r2.x >= 0x1p-126f ? z.x : 0.f;   // skip coincident bodies (r < 1e-19)
        z.y = r2.y >= 0x1p-126f ? z.y : 0.f;
        q[k] = fma2(mn, z, q[k]);                              // += m/r
      }
    }
#pragma unroll
    for (int k = 0; k < IPT; ++k) {
      ff_accum(hi[k], lo[k], __fadd_rn(q[k].x, q[k].y));
      q[k] = make_float2(0.f, 0.f);
    }
    __syncthreads();
    if (s_abort) break;
    if (tid == 0 && t + PSTAGE < nt) {
      mbar_expect_tx(&bar[s], PTILE_BYTES);
      bulk_g2s(smem + s * PTILE_FLOATS, tiles + (size_t)(t0 + t + PSTAGE) * PTILE_FLOATS,
               PTILE_BYTES, &bar[s]);
    }
  }
  if (s_abort) {
    // Copies for tiles t .. t+PSTAGE-1 may still be in flight, tile t's
    // included (its wait is the one that gave up): wait for each of them
    // before the block exits, so that no bulk copy writes into shared memory
    // the block no longer owns.  The block writes no partial sums; the
    // merge sees the error word and writes NaN.
    if (tid == 0) {
      for (int u = t; u < nt && u < t + PSTAGE; ++u)
        mbar_wait_bounded(&bar[u % PSTAGE], (uint32_t)(u / PSTAGE) & 1u, 1u << 20);
      raise_error(err, GPUNB_E_TIMEOUT);
    }
    return;
  }
#pragma unroll
  for (int k = 0; k < IPT; ++k)
    if (iloc[k] >= 0) part[(size_t)sy * ni_pad + iloc[k]] = (double)hi[k] + (double)lo[k];
}

// ---------------------------------------------------------------------------
// The potential of gpupot_ on Morton-ordered tiles: the regular force's tile
// layout (pack_jtiles_kernel; the velocity fields are unused here) with its
// centres, radii and boxes, so that, as in the regular force's pair loop,
// tiles far from every i of a warp take the tile-relative difference
// dx = (x_j - O) + (O - x_i) -- one addition per component instead of three
// -- and the bare product-form Newton step: 10 packed FP32 operations per
// pair of j against 17 on double-single coordinates.  Near tiles keep the
// double-single path.  A tile is far only when |O - x_i| >= 2R, so a far
// body lies at least |O - x_i| / 2 from x_i, and a tile counts as near
// whenever |O - x_i|^2 < 2^-120, so a far pair never meets the
// coincident-body case (r^2 below 2^-126) that the near path skips.  i runs in processing slots: slot s is the i-particle
// istart0 + iorder[s] (iorder == null: s), so that the i of a warp are close
// together as well.
template <int IPT, int WI>
__global__ void __launch_bounds__(32 * WI) pot_rel_kernel(const float *__restrict__ tiles,
                                                          int ntile, const double *__restrict__ x,
                                                          const int *__restrict__ iorder,
                                                          int istart0, int ni,
                                                          double *__restrict__ part, int ni_pad,
                                                          int *err) {
  constexpr int ITILE = 32 * IPT * WI;
  extern __shared__ __align__(128) float smem[];
  __shared__ __align__(8) uint64_t bar[PSTAGE];
  __shared__ int s_abort;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int ns = gridDim.y, sy = blockIdx.y;
  const int t0 = (int)(((long long)ntile * sy) / ns);
  const int t1 = (int)(((long long)ntile * (sy + 1)) / ns);
  const int nt = t1 - t0;
  if (tid == 0) {
    for (int s = 0; s < PSTAGE; ++s) mbar_init(&bar[s], 1);
    fence_mbar_init();
    s_abort = 0;
  }
  __syncthreads();
  if (tid == 0)
    for (int s = 0; s < PSTAGE && s < nt; ++s) {
      mbar_expect_tx(&bar[s], TILE_BYTES);
      bulk_g2s(smem + s * TILE_FLOATS, tiles + (size_t)(t0 + s) * TILE_FLOATS, TILE_BYTES,
               &bar[s]);
    }
  float nh[IPT][3], nl[IPT][3];
  f2 q[IPT];
  float hi[IPT], lo[IPT];
  int slot[IPT];
#pragma unroll
  for (int k = 0; k < IPT; ++k) {
    const int il = blockIdx.x * ITILE + warp * 32 * IPT + k * 32 + lane;
    slot[k] = il < ni ? il : -1;
    const int i = istart0 + (il < ni ? (iorder ? iorder[il] : il) : 0);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      float h, l;
      ds_split(x[3 * (size_t)i + c], h, l);
      nh[k][c] = -h;
      nl[k][c] = -l;
    }
    q[k] = make_float2(0.f, 0.f);
    hi[k] = lo[k] = 0.f;
  }
  int t = 0;
  for (; t < nt; ++t) {
    const int s = t % PSTAGE;
    if (!mbar_wait_bounded(&bar[s], (uint32_t)(t / PSTAGE) & 1u)) s_abort = 1;
    const float *T = smem + s * TILE_FLOATS;
    const float *M = T + NFIELD * JT;
    const float rad = M[M_RAD];
    const float oh[3] = {M[M_OH], M[M_OH + 1], M[M_OH + 2]};
#pragma unroll
    for (int k = 0; k < IPT; ++k) {
      // O - x_i from the double-single parts, rounded once to FP32
      float o[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) o[c] = __fadd_rn(__fadd_rn(oh[c], nh[k][c]), nl[k][c]);
      // near unless |o| >= 2R (every body at least |o| / 2 away) and |o|^2 is
      // normal.  Unlike the regular force, no test against the tile's box:
      // that box is the one of the FP32-rounded positions, and where it
      // shrinks to a point (bodies within an FP32 rounding of each other) it
      // would declare far a tile holding bodies at x_i itself, which the
      // potential (no neighbour exclusion) must skip, not divide by.
      const float o2 = fmaf(o[2], o[2], fmaf(o[1], o[1], o[0] * o[0]));
      const bool near = slot[k] >= 0 && (o2 < GPUNB_NEAR_K2 * rad * rad || o2 < 0x1p-120f);
      if (__any_sync(0xffffffffu, near)) {
        const f2 xh = mk2(nh[k][0]), yh = mk2(nh[k][1]), zh = mk2(nh[k][2]);
        const f2 xl = mk2(nl[k][0]), yl = mk2(nl[k][1]), zl = mk2(nl[k][2]);
        auto near2 = [&](f2 xh_j, f2 yh_j, f2 zh_j, f2 xl_j, f2 yl_j, f2 zl_j, f2 mn) {
          const f2 dx = add2(add2(xh_j, xh), add2(xl_j, xl));
          const f2 dy = add2(add2(yh_j, yh), add2(yl_j, yl));
          const f2 dz = add2(add2(zh_j, zh), add2(zl_j, zl));
          const f2 r2 = fma2(dz, dz, fma2(dy, dy, mul2(dx, dx)));
          const f2 y0 = make_float2(rsqrt_est(r2.x), rsqrt_est(r2.y));
          f2 z = mul2(y0, fma2(mul2(r2, y0), y0, mk2(-3.0f)));   // -2/r
          z.x = r2.x >= 0x1p-126f ? z.x : 0.f;   // skip coincident bodies (r < 1e-19)
          z.y = r2.y >= 0x1p-126f ? z.y : 0.f;
          q[k] = fma2(mn, z, q[k]);                              // += m/r
        };
#pragma unroll 2
        for (int jj = 0; jj < JT; jj += 4) {   // four j per shared-memory load
          const float4 a = *(const float4 *)(T + F_XH * JT + jj);
          const float4 b = *(const float4 *)(T + F_YH * JT + jj);
          const float4 c = *(const float4 *)(T + F_ZH * JT + jj);
          const float4 d = *(const float4 *)(T + F_XL * JT + jj);
          const float4 e = *(const float4 *)(T + F_YL * JT + jj);
          const float4 f = *(const float4 *)(T + F_ZL * JT + jj);
          const float4 w = *(const float4 *)(T + F_MN * JT + jj);
          near2(make_float2(a.x, a.y), make_float2(b.x, b.y), make_float2(c.x, c.y),
                make_float2(d.x, d.y), make_float2(e.x, e.y), make_float2(f.x, f.y),
                make_float2(w.x, w.y));
          near2(make_float2(a.z, a.w), make_float2(b.z, b.w), make_float2(c.z, c.w),
                make_float2(d.z, d.w), make_float2(e.z, e.w), make_float2(f.z, f.w),
                make_float2(w.z, w.w));
        }
      } else {
        const f2 ox = mk2(o[0]), oy = mk2(o[1]), oz = mk2(o[2]);
        auto far2 = [&](f2 xr, f2 yr, f2 zr, f2 mn) {
          const f2 dx = add2(xr, ox), dy = add2(yr, oy), dz = add2(zr, oz);
          const f2 r2 = fma2(dz, dz, fma2(dy, dy, mul2(dx, dx)));
          const f2 y0 = make_float2(rsqrt_est(r2.x), rsqrt_est(r2.y));
          const f2 z = mul2(y0, fma2(mul2(r2, y0), y0, mk2(-3.0f)));   // -2/r
          q[k] = fma2(mn, z, q[k]);
        };
#pragma unroll 4
        for (int jj = 0; jj < JT; jj += 4) {   // four j per shared-memory load
          const float4 a = *(const float4 *)(T + F_XR * JT + jj);
          const float4 b = *(const float4 *)(T + F_YR * JT + jj);
          const float4 c = *(const float4 *)(T + F_ZR * JT + jj);
          const float4 w = *(const float4 *)(T + F_MN * JT + jj);
          far2(make_float2(a.x, a.y), make_float2(b.x, b.y), make_float2(c.x, c.y),
               make_float2(w.x, w.y));
          far2(make_float2(a.z, a.w), make_float2(b.z, b.w), make_float2(c.z, c.w),
               make_float2(w.z, w.w));
        }
      }
      ff_accum(hi[k], lo[k], __fadd_rn(q[k].x, q[k].y));
      q[k] = make_float2(0.f, 0.f);
    }
    __syncthreads();
    if (s_abort) break;
    if (tid == 0 && t + PSTAGE < nt) {
      mbar_expect_tx(&bar[s], TILE_BYTES);
      bulk_g2s(smem + s * TILE_FLOATS, tiles + (size_t)(t0 + t + PSTAGE) * TILE_FLOATS,
               TILE_BYTES, &bar[s]);
    }
  }
  if (s_abort) {
    // copies for tiles t .. t+PSTAGE-1 may still be in flight (tile t's
    // included): wait for each before the block exits; no partial sums are
    // written, and the merge, seeing the error word, writes NaN
    if (tid == 0) {
      for (int u = t; u < nt && u < t + PSTAGE; ++u)
        mbar_wait_bounded(&bar[u % PSTAGE], (uint32_t)(u / PSTAGE) & 1u, 1u << 20);
      raise_error(err, GPUNB_E_TIMEOUT);
    }
    return;
  }
#pragma unroll
  for (int k = 0; k < IPT; ++k)
    if (slot[k] >= 0) part[(size_t)sy * ni_pad + slot[k]] = (double)hi[k] + (double)lo[k];
}

// Sums the S partials of each i in split order.  When an earlier kernel of
// the call raised an error (a NaN input, a bounded wait that gave up and left
// its partial sums unwritten), every result is NaN: partial sums left over
// from an earlier call can never pass for this call's potentials.
// iorder (may be null): the partials are in processing slots, slot s holding
// the i-particle iorder[s].
__global__ void pot_merge_kernel(const double *__restrict__ part, int S, int ni, int ni_pad,
                                 const int *__restrict__ err, const int *__restrict__ iorder,
                                 double *__restrict__ pot) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ni) return;
  const int out = iorder ? iorder[i] : i;
  if (err && *(volatile const int *)err != 0) {
    pot[out] = __longlong_as_double(0x7ff8000000000000ll);   // quiet NaN
    return;
  }
  double s = 0.0;
  for (int k = 0; k < S; ++k) s += part[(size_t)k * ni_pad + i];
  pot[out] = s;
}

// host launchers
static_assert(PJT == POT_JT && PTILE_FLOATS == POT_TILE_FLOATS, "pot tile layout");
constexpr int POT_IPT = 2, POT_WI = 4;

int pot_itile() { return 32 * POT_IPT * POT_WI; }

int pot_blocks_per_sm() {
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, pot_ds_kernel<POT_IPT, POT_WI>,
                                                    32 * POT_WI,
                                                    (size_t)PSTAGE * PTILE_BYTES) != cudaSuccess)
    return 1;
  return n > 0 ? n : 1;
}

cudaError_t launch_pack_pot(const double *m, const double *x, int n, float *tiles, int ntile,
                            int *err, cudaStream_t st) {
  if (ntile <= 0) return cudaSuccess;
  pack_pot_tiles_kernel<<<ntile, PJT, 0, st>>>(m, x, n, tiles, err);
  return cudaGetLastError();
}

cudaError_t launch_pot(const float *tiles, int ntile, const double *x, int istart0, int ni,
                       int gx, int S, double *part, int ni_pad, int *err, cudaStream_t st) {
  pot_ds_kernel<POT_IPT, POT_WI><<<dim3(gx, S), 32 * POT_WI, (size_t)PSTAGE * PTILE_BYTES, st>>>(
      tiles, ntile, x, istart0, ni, part, ni_pad, err);
  return cudaGetLastError();
}

cudaError_t launch_pot_merge(const double *part, int S, int ni, int ni_pad, const int *err,
                             double *pot, cudaStream_t st, const int *iorder) {
  pot_merge_kernel<<<(ni + 255) / 256, 256, 0, st>>>(part, S, ni, ni_pad, err, iorder, pot);
  return cudaGetLastError();
}

int pot_rel_blocks_per_sm() {
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, pot_rel_kernel<POT_IPT, POT_WI>,
                                                    32 * POT_WI,
                                                    (size_t)PSTAGE * TILE_BYTES) != cudaSuccess) {
    cudaGetLastError();
    return 1;
  }
  return n > 0 ? n : 1;
}

cudaError_t launch_pot_rel(const float *tiles, int ntile, const double *x, const int *iorder,
                           int istart0, int ni, int gx, int S, double *part, int ni_pad, int *err,
                           cudaStream_t st) {
  static_assert(PSTAGE * TILE_BYTES <= 48 * 1024, "the tile ring fits the default shared memory");
  pot_rel_kernel<POT_IPT, POT_WI><<<dim3(gx, S), 32 * POT_WI, (size_t)PSTAGE * TILE_BYTES, st>>>(
      tiles, ntile, x, iorder, istart0, ni, part, ni_pad, err);
  return cudaGetLastError();
}

}  // namespace gpunb
