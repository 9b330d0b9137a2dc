// Regular force + jerk + potential + neighbour-list kernels for sm_103a.
//
// Reference device path replaced: src/Main/gpunb.velocity.cu:162-552
// (dev_gravity, gravity_kernel(_m), force_reduce_kernel, gather_nb_kernel) and
// the host prefix sum / merge of gpunb.velocity.cu:793-878.
//
// Pipeline for one gpunb_regf_ call (all on one stream):
//   regf_prep_kernel      FP32 i-records in Morton processing order
//   regf_ds_kernel<...>   persistent pair loop over (i-tile, j-split) work
//                         items from a device queue, partial sums per split
//   regf_merge_(wide_)kernel  FP64 sum of the j-split partials in fixed
//                         order, neighbour count -> in-band overflow flag
//   list_scan_*           exclusive scan of accepted row lengths
//   list_gather_kernel    per-row sort (ascending j) + compaction
#include "regf_kernels.cuh"
#include "launch.h"

#include <algorithm>
#include <cfloat>
#include <climits>

// The FP32 chunk sums of the pair loop are folded into the float-float
// accumulators every GPUNB_FOLD_TILES tiles (64 terms per f32x2 half per
// tile).
#ifndef GPUNB_FOLD_TILES
#define GPUNB_FOLD_TILES 1
#endif

// The warp vote on the neighbour candidates of a pair group right after r^2,
// before the rsqrt and Newton step (the accepted neighbours then drop out
// through a zero mass, with r^2 set to 1 so that 1/r stays finite), so that
// the inverse distances and the sums of the group's lane pairs follow the
// branch in one block; else after the whole geometry (they drop out through a
// zero 1/r).  Measured on GB300 (Plummer 65536): 4.522 -> 4.499 ms at
// ni = 65536, 1.258 -> 1.253 ms at ni = 16384, identical errors and lists.
#ifndef GPUNB_VOTE_EARLY
#define GPUNB_VOTE_EARLY 1
#endif

namespace gpunb {

// ---------------------------------------------------------------------------
// j packing: FP64 (as sent) -> tile-relative FP32 SoA tiles + tile metadata.
// One block of JT threads per tile.  Replaces the host-side Jparticle packing
// of gpunb.velocity.cu:716-727 (which drops positions to plain FP32).
// Tile slot p holds body perm[p] (identity when perm is null; perm[p] = -1
// marks a padding slot).

// block-wide maxima of NV floats (JT threads), results in every thread
template <int NV>
__device__ __forceinline__ void block_maxf(float (&a)[NV], float (*s)[NV]) {
#pragma unroll
  for (int q = 0; q < NV; ++q)
    for (int o = 16; o > 0; o >>= 1) a[q] = fmaxf(a[q], __shfl_xor_sync(0xffffffffu, a[q], o));
  if ((threadIdx.x & 31) == 0) {
#pragma unroll
    for (int q = 0; q < NV; ++q) s[threadIdx.x >> 5][q] = a[q];
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < NV; ++q) {
    float r = s[0][q];
    for (int w = 1; w < JT / 32; ++w) r = fmaxf(r, s[w][q]);
    a[q] = r;
  }
  __syncthreads();
}

// The tile centre O is an FP32 number (the midpoint of the tile's box of
// FP32-rounded coordinates), so its double-single form is (O, 0) and only the
// double-single split and the tile-relative difference x - O need FP64
// arithmetic (on GB300 about 1/64 of the FP32 rate).  The tile maxima are
// formed in FP32 from the rounded values and widened by 2^-18 with upward
// rounding: the FP32 evaluation of |v|, |x - O| and sqrt(m) is within 2^-21
// of the exact value, so the stored maxima stay upper bounds.
// v may be null (the potential's tiles): velocity fields and maxima are 0.
__global__ void __launch_bounds__(JT) pack_jtiles_kernel(const double *__restrict__ m,
                                                         const double *__restrict__ x,
                                                         const double *__restrict__ v, int nj,
                                                         const int *__restrict__ perm,
                                                         float *__restrict__ tiles, int *err) {
  const int t = blockIdx.x, l = threadIdx.x, p = t * JT + l;
  float *T = tiles + (size_t)t * TILE_FLOATS;
  __shared__ float s_red6[JT / 32][6];
  __shared__ float s_red4[JT / 32][4];
  const int j = perm ? perm[p] : (p < nj ? p : -1);   // -1: padding slot
  double xj[3] = {0.0, 0.0, 0.0};
  float xf[3] = {0.f, 0.f, 0.f}, vf[3] = {0.f, 0.f, 0.f}, mf = 0.f;
  if (j >= 0) {
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      xj[c] = x[3 * j + c];
      xf[c] = (float)xj[c];
      vf[c] = v ? (float)v[3 * j + c] : 0.f;
    }
    mf = (float)m[j];
    if (isnan(xf[0]) || isnan(xf[1]) || isnan(xf[2]) || isnan(vf[0]) || isnan(vf[1]) ||
        isnan(vf[2]) || isnan(mf))
      raise_error(err, GPUNB_E_NAN);
  }
  // tile centre: midpoint of the real bodies' box (FP32)
  float bb[6];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    bb[c] = j >= 0 ? xf[c] : -INFINITY;        // max
    bb[3 + c] = j >= 0 ? -xf[c] : -INFINITY;   // -min
  }
  block_maxf<6>(bb, s_red6);
  float o[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const float hi = bb[c], lo = -bb[3 + c];
    o[c] = (hi >= lo) ? 0.5f * lo + 0.5f * hi : 0.f;   // no real body: O = 0
    if (!isfinite(o[c])) o[c] = 0.f;
  }
  float r2 = 0.f, v2 = 0.f;
  if (j >= 0) {
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float d = (float)(xj[c] - (double)o[c]);
      r2 = fmaf(d, d, r2);
      v2 = fmaf(vf[c], vf[c], v2);
      T[(F_XR + c) * JT + l] = d;
      T[(F_XH + c) * JT + l] = xf[c];
      T[(F_XL + c) * JT + l] = (float)(xj[c] - (double)xf[c]);
    }
    T[F_VX * JT + l] = vf[0];
    T[F_VY * JT + l] = vf[1];
    T[F_VZ * JT + l] = vf[2];
    T[F_MN * JT + l] = -0.5f * mf;
  } else {
    // padding body: massless and far away, never a neighbour candidate
    T[F_XR * JT + l] = 1.0e15f;
    T[F_YR * JT + l] = 1.0e15f;
    T[F_ZR * JT + l] = 1.0e15f;
    T[F_XH * JT + l] = 1.0e15f; T[F_XL * JT + l] = 0.f;
    T[F_YH * JT + l] = 1.0e15f; T[F_YL * JT + l] = 0.f;
    T[F_ZH * JT + l] = 1.0e15f; T[F_ZL * JT + l] = 0.f;
    T[F_VX * JT + l] = 0.f; T[F_VY * JT + l] = 0.f; T[F_VZ * JT + l] = 0.f;
    T[F_MN * JT + l] = -0.f;
  }
  // tile maxima of |v|, m and |x - O|; body count (real slots fill from 0)
  float mx[4] = {sqrtf(v2), mf, sqrtf(r2), j >= 0 ? (float)(l + 1) : 0.f};
  block_maxf<4>(mx, s_red4);
  if (l == 0) {
    constexpr float grow = 1.0f + 0x1p-18f;
    float *M = T + NFIELD * JT;
    M[M_VMAX] = __fmul_ru(mx[0], grow);
    M[M_SMAX] = __fmul_ru(sqrtf(fmaxf(mx[1], 0.f)), grow);
    M[M_COUNT] = mx[3];
    M[M_RAD] = __fmul_ru(mx[2], grow);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      M[M_OH + c] = o[c];
      // half-extent of the box about O (0 for an empty tile)
      M[M_BOX + c] = (bb[c] >= -bb[3 + c]) ? __fmul_ru(0.5f * (bb[c] + bb[3 + c]), grow) : 0.f;
    }
    M[M_OH + 3] = 0.f;
    M[M_BOX + 3] = 0.f;
  }
}

// ---------------------------------------------------------------------------
// Exact FP64 neighbour decision, in the expression order of the FP64 oracle
// (no contraction: explicit round-to-nearest mul/add).
__device__ __forceinline__ bool nb_test_fp64(const ISet &is, int i, const JSet &js, int j,
                                             bool mflag) {
  const double xi0 = is.x[3 * i], xi1 = is.x[3 * i + 1], xi2 = is.x[3 * i + 2];
  const double vi0 = is.v[3 * i], vi1 = is.v[3 * i + 1], vi2 = is.v[3 * i + 2];
  const double dx = __dadd_rn(js.x64[3 * j], -xi0);
  const double dy = __dadd_rn(js.x64[3 * j + 1], -xi1);
  const double dz = __dadd_rn(js.x64[3 * j + 2], -xi2);
  const double dvx = __dadd_rn(js.v64[3 * j], -vi0);
  const double dvy = __dadd_rn(js.v64[3 * j + 1], -vi1);
  const double dvz = __dadd_rn(js.v64[3 * j + 2], -vi2);
  const double dtr = is.dtr[i];
  const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
  const double px = __dadd_rn(dx, __dmul_rn(dvx, dtr));
  const double py = __dadd_rn(dy, __dmul_rn(dvy, dtr));
  const double pz = __dadd_rn(dz, __dmul_rn(dvz, dtr));
  const double r2p = __dadd_rn(__dadd_rn(__dmul_rn(px, px), __dmul_rn(py, py)), __dmul_rn(pz, pz));
  const double r2min = r2 < r2p ? r2 : r2p;
  const double crit = mflag ? __dmul_rn(js.m64[j], is.h2[i]) : is.h2[i];
  return r2min < crit;
}

// ---------------------------------------------------------------------------
// Per-i register state of the split-precision kernel.
struct IState {
  float nxh, nyh, nzh, nxl, nyl, nzl;  // -(hi, lo) of the position
  f2 nvx, nvy, nvz;                 // -velocity, duplicated
  float s;                          // sqrt(h2) * (1 + 2^-12)  (filter radius)
  float dv;                         // |dtr| * (1 + 2^-12)
  float va;                         // |v_i| * (1 + 2^-12)
  float h2f, dtrf;
  int i;
};

// i-record: the FP32 state of one i-particle, 64 bytes, written once per call
// by regf_prep_kernel in processing-slot order:
//   [0..5]  -(hi, lo) of x, y, z     [6..8]  -velocity
//   [9]  filter radius sqrt(h2)(1 + 2^-12) (-1: no neighbour test)
//   [10] |dtr|(1 + 2^-12)  [11] |v|(1 + 2^-12)  [12] h2  [13] dtr
//   [14] index into the caller's i arrays (int bits)  [15] unused
__global__ void regf_prep_kernel(const ISet is, float4 *__restrict__ rec, int *err) {
  const int slot = blockIdx.x * blockDim.x + threadIdx.x;
  if (slot >= is.ni) return;
  const int i = is.perm ? is.perm[slot] : slot;
  if (i < 0) return;   // padding slot of a batched layout (never read)
  const double x0 = is.x[3 * i], x1 = is.x[3 * i + 1], x2 = is.x[3 * i + 2];
  // FP32 from here on except the double-single split (FP64 runs at about
  // 1/64 of the FP32 rate on GB300).  The bounds are formed from the rounded
  // values (within 2^-22 of the exact ones) and widened with upward rounding
  // by 2^-12 + 2^-20, so they stay above sqrt(h2)(1 + 2^-12) etc.
  const float v0 = (float)is.v[3 * i], v1 = (float)is.v[3 * i + 1], v2 = (float)is.v[3 * i + 2];
  const float h2 = (float)is.h2[i], dtr = (float)is.dtr[i];
  float xh, xl, yh, yl, zh, zl;
  ds_split(x0, xh, xl);
  ds_split(x1, yh, yl);
  ds_split(x2, zh, zl);
  if (isnan(xh) || isnan(yh) || isnan(zh) || isnan(v0) || isnan(v1) || isnan(v2) || isnan(h2) ||
      isnan(dtr))
    raise_error(err, GPUNB_E_NAN);
  constexpr float grow = 1.0f + 0x1p-12f + 0x1p-20f;
  const float va = sqrtf(fmaf(v0, v0, fmaf(v1, v1, v2 * v2)));
  float4 *r = rec + 4 * (size_t)slot;
  r[0] = make_float4(-xh, -yh, -zh, -xl);
  r[1] = make_float4(-yl, -zl, -v0, -v1);
  r[2] = make_float4(-v2, __fmul_ru(sqrtf(fmaxf(h2, 0.f)), grow), __fmul_ru(fabsf(dtr), grow),
                     __fmul_ru(va, grow));
  r[3] = make_float4(h2, dtr, __int_as_float(i), 0.f);
}

__device__ __forceinline__ void load_istate(IState &I, const float4 *__restrict__ rec, int slot,
                                            bool valid) {
  if (valid) {
    const float4 *r = rec + 4 * (size_t)slot;
    const float4 a = r[0], b = r[1], c = r[2], d = r[3];
    I.nxh = a.x; I.nyh = a.y; I.nzh = a.z;
    I.nxl = a.w; I.nyl = b.x; I.nzl = b.y;
    I.nvx = mk2(b.z); I.nvy = mk2(b.w); I.nvz = mk2(c.x);
    I.s = c.y; I.dv = c.z; I.va = c.w;
    I.h2f = d.x; I.dtrf = d.y; I.i = __float_as_int(d.z);
  } else {
    I.nxh = I.nyh = I.nzh = I.nxl = I.nyl = I.nzl = 0.f;
    I.nvx = I.nvy = I.nvz = mk2(0.f);
    I.s = -1.f; I.dv = 0.f; I.va = 0.f; I.h2f = -1.f; I.dtrf = 0.f; I.i = -1;
  }
}

// Exact FP64 decision for a pair whose FP32 criterion value fell inside the
// error band (very rare): kept out of line so that the common path carries
// no call frame.  slot: the j's tile slot (padding slots are never members).
template <bool MFLAG>
__device__ __noinline__ bool decide_pair_fp64(const ISet &is, int i, const JSet &js, int slot) {
  const int jo = js.perm[slot];
  return jo >= 0 && nb_test_fp64(is, i, js, jo, MFLAG);
}

// Decide one candidate pair (rare path).  FP32 decision, FP64 re-test when
// the FP32 value lies inside a conservative error band around the criterion.
// The band bounds the FP32 rounding of the coordinate and velocity
// differences, of h2 and of the products by 2^-14 of the magnitudes involved
// (|dv| bounded by its L1 norm), plus 2^-18 R (r + w) for the tile-relative
// coordinates (their error is below 2^-23 (R + r) per component; R = tile
// radius).
template <bool MFLAG>
__device__ __forceinline__ bool decide_pair(const IState &I, const ISet &is, const JSet &js,
                                            int slot, float dx, float dy, float dz, float dvx,
                                            float dvy, float dvz, float r2, float mneg_half,
                                            float R) {
  const float px = fmaf(I.dtrf, dvx, dx);
  const float py = fmaf(I.dtrf, dvy, dy);
  const float pz = fmaf(I.dtrf, dvz, dz);
  const float r2p = fmaf(px, px, fmaf(py, py, pz * pz));
  const float r2min = fminf(r2, r2p);
  const float crit = MFLAG ? (-2.0f * mneg_half) * I.h2f : I.h2f;
  bool in = r2min < crit;
  const float dv1 = fabsf(dvx) + fabsf(dvy) + fabsf(dvz);
  const float w = 2.0f * fabsf(I.dtrf) * (I.va + dv1);
  const float band = 0x1p-14f * (fabsf(crit) + r2 + w * w) + 0x1p-18f * R * (sqrtf(r2) + w);
  if (fabsf(r2min - crit) <= band) in = decide_pair_fp64<MFLAG>(is, I.i, js, slot);
  return in;
}

// Accepted neighbours of one (thread, i) pending in shared memory: the tile
// slots, NBUF at most, entry e at buf[e * stride].  The pair loop only writes
// them there; a flush maps the slots to the caller's ids, reserves room in
// the row with one atomic per thread and stores them.  Flushes are
// warp-collective (when a lane of the warp could overflow its buffer, and at
// the end of each work item), so the loads and atomics of the lanes overlap
// and the pair loop never waits on global memory.  Row order does not matter:
// the rows are sorted when they are gathered.
#ifndef GPUNB_NBUF
#define GPUNB_NBUF 32
#endif
constexpr int NBUF = GPUNB_NBUF;
static_assert(NBUF >= 8 && NBUF % 4 == 0, "a pair group adds up to 8 entries");

struct NbRec {
  int *buf;
  int stride;
  int n;
};

__device__ __forceinline__ void nb_flush(NbRec &r, int i, int jbase, const int *__restrict__ perm,
                                         const RegfOut &out) {
  if (r.n > 0) {
    int valid = 0;
    for (int e0 = 0; e0 < r.n; e0 += 4) {
      int jo[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) jo[u] = e0 + u < r.n ? __ldg(perm + r.buf[(e0 + u) * r.stride]) : -1;
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        if (e0 + u < r.n) r.buf[(e0 + u) * r.stride] = jo[u];
        valid += jo[u] >= 0;
      }
    }
    if (valid > 0) {
      int slot = atomicAdd(out.cnt + i, valid);
      for (int e = 0; e < r.n; ++e) {
        const int jo = r.buf[e * r.stride];
        if (jo >= 0) {
          if (slot < out.cap) out.rows[(size_t)i * out.cap + slot] = jo - jbase;
          ++slot;
        }
      }
    }
    r.n = 0;
  }
}

// warp-collective: make room for the up to 8 entries of one pair group
__device__ __forceinline__ void nb_room(NbRec &r, int i, int jbase, const JSet &js,
                                        const RegfOut &out) {
  if (__any_sync(0xffffffffu, r.n > NBUF - 8)) nb_flush(r, i, jbase, js.perm, out);
}

// Two j (one f32x2 lane pair) against one i.  The per-pair computation is
// split in three so that the kernel can run the geometry of several lane
// pairs, take one warp vote for the rare neighbour-candidate branch, and then
// accumulate: the dependent chains of the lane pairs interleave instead of
// being cut apart by a branch after every pair.
struct JPair {
  f2 v[NFIELD];   // indexed by JField
};

struct PairGeo {
  f2 dx, dy, dz, dvx, dvy, dvz, mn, r2, rv, z;
};

// Per (i, tile): the offset O - x_i of the tile centre from the i-particle
// (double-single difference rounded to FP32, duplicated for the lane pairs),
// the candidate bound H on r^2 and the tile radius R.
struct TileCtx {
  f2 ox, oy, oz;
  f2 nxh, nyh, nzh, nxl, nyl, nzl;   // -(hi, lo) of x_i, for near tiles
  float H, R;
};

template <bool REL>
__device__ __forceinline__ void pair_inv(PairGeo &g);

template <bool REL>
__device__ __forceinline__ void pair_geo(const IState &I, const TileCtx &C, const JPair &p,
                                         PairGeo &g) {
  if (REL) {
    // from the tile-relative position: (x_j - O) + (O - x_i)
    g.dx = add2(p.v[F_XR], C.ox);
    g.dy = add2(p.v[F_YR], C.oy);
    g.dz = add2(p.v[F_ZR], C.oz);
  } else {
    // double-single difference: (hi_j - hi_i) + (lo_j - lo_i)
    g.dx = add2(add2(p.v[F_XH], C.nxh), add2(p.v[F_XL], C.nxl));
    g.dy = add2(add2(p.v[F_YH], C.nyh), add2(p.v[F_YL], C.nyl));
    g.dz = add2(add2(p.v[F_ZH], C.nzh), add2(p.v[F_ZL], C.nzl));
  }
  g.dvx = add2(p.v[F_VX], I.nvx);
  g.dvy = add2(p.v[F_VY], I.nvy);
  g.dvz = add2(p.v[F_VZ], I.nvz);
  g.mn = p.v[F_MN];
  g.r2 = fma2(g.dz, g.dz, fma2(g.dy, g.dy, mul2(g.dx, g.dx)));
  g.rv = fma2(g.dz, g.dvz, fma2(g.dy, g.dvy, mul2(g.dx, g.dvx)));
  if (!GPUNB_VOTE_EARLY) pair_inv<REL>(g);
}

// Far-tile pairs (REL) take the product form y0 ((x y0) y0 - 3) of the Newton
// step, one f32x2 operation less than the residual form the near pairs keep:
// the far pairs' terms are the smaller ones, so their extra rounding hardly
// shows.  Measured on GB300 (Plummer 65536, against the FP64 kernel at
// ni = 16384): jerk p99 7.01e-7 -> 7.13e-7, max 2.76e-6 -> 2.77e-6, force p99
// 8.4e-8 -> 9.4e-8, for 4.507 -> 4.434 ms at ni = 65536.
#ifndef GPUNB_FAR_PRODUCT
#define GPUNB_FAR_PRODUCT 1
#endif
template <bool REL>
__device__ __forceinline__ void pair_inv(PairGeo &g) {
  // rsqrt estimate + one Newton step, scaled: z = y0 (x y0^2 - 3) = -2/r,
  // evaluated in residual form: e = x y0^2 - 1 is small, so its rounding is
  // negligible, and z = y0 e - 2 y0 takes a single rounding in the last FMA.
  // The product form y0 ((x y0) y0 - 3) rounds three times; measured against
  // FP64 (Plummer 65536, 16384 active) the residual form takes the jerk's
  // 99th percentile from 9.0e-7 to 6.8e-7 and the particles above 1e-6 from
  // 130 to 50, for one more f32x2 FMA per lane pair.
  const f2 y0 = make_float2(rsqrt_est(g.r2.x), rsqrt_est(g.r2.y));
  if (REL && GPUNB_FAR_PRODUCT) {
    g.z = mul2(y0, fma2(mul2(g.r2, y0), y0, mk2(-3.0f)));
    return;
  }
  const f2 e = fma2(mul2(g.r2, y0), y0, mk2(-1.0f));
  g.z = fma2(y0, e, mul2(y0, mk2(-2.0f)));
}

__device__ __forceinline__ bool pair_maybe(const PairGeo &g, float H) {
  return (g.r2.x < H) | (g.r2.y < H);
}

// Candidates of one lane pair (rare path): decide, record the tile slot, and
// drop the neighbours from the sums.  Padding slots (massless, at 1e15) are
// filtered when the slots are mapped to ids (nb_flush).
template <bool MFLAG>
__device__ __forceinline__ void pair_candidates(const IState &I, const TileCtx &C, PairGeo &g,
                                                int jg0, const JSet &js, const ISet &is,
                                                NbRec &rec) {
  const float H = C.H;
  if (g.r2.x < H && decide_pair<MFLAG>(I, is, js, jg0, g.dx.x, g.dy.x, g.dz.x, g.dvx.x, g.dvy.x,
                                       g.dvz.x, g.r2.x, g.mn.x, C.R)) {
    rec.buf[rec.n++ * rec.stride] = jg0;
    if (GPUNB_VOTE_EARLY) {
      g.mn.x = 0.f;
      g.r2.x = 1.f;
    } else {
      g.z.x = 0.f;
    }
  }
  if (g.r2.y < H && decide_pair<MFLAG>(I, is, js, jg0 + 1, g.dx.y, g.dy.y, g.dz.y, g.dvx.y,
                                       g.dvy.y, g.dvz.y, g.r2.y, g.mn.y, C.R)) {
    rec.buf[rec.n++ * rec.stride] = jg0 + 1;
    if (GPUNB_VOTE_EARLY) {
      g.mn.y = 0.f;
      g.r2.y = 1.f;
    } else {
      g.z.y = 0.f;
    }
  }
}

__device__ __forceinline__ void pair_acc(const PairGeo &g, f2 (&q)[NQ]) {
  const f2 mr = mul2(g.mn, g.z);        // m/r
  const f2 z2 = mul2(g.z, g.z);         // 4/r^2
  const f2 mr3 = mul2(mr, z2);          // 4 m/r^3
  q[6] = add2(q[6], mr);
  q[0] = fma2(mr3, g.dx, q[0]);
  q[1] = fma2(mr3, g.dy, q[1]);
  q[2] = fma2(mr3, g.dz, q[2]);
  const f2 al = mul2(mul2(g.rv, z2), mk2(-0.75f));   // -3 (r.v)/r^2
  q[3] = fma2(mr3, fma2(al, g.dx, g.dvx), q[3]);
  q[4] = fma2(mr3, fma2(al, g.dy, g.dvy), q[4]);
  q[5] = fma2(mr3, fma2(al, g.dz, g.dvz), q[5]);
}

// Four j (two lane pairs) against one i, one warp vote for both.
template <bool MFLAG, bool REL>
__device__ __forceinline__ void pair4(const IState &I, const TileCtx &C, const JPair &p0,
                                      const JPair &p1, f2 (&q)[NQ], int jg0, int jbase,
                                      const JSet &js, const ISet &is, const RegfOut &out,
                                      NbRec &rec) {
  PairGeo g0, g1;
  pair_geo<REL>(I, C, p0, g0);
  pair_geo<REL>(I, C, p1, g1);
  if (__any_sync(0xffffffffu, pair_maybe(g0, C.H) | pair_maybe(g1, C.H))) {
    nb_room(rec, I.i, jbase, js, out);
    pair_candidates<MFLAG>(I, C, g0, jg0, js, is, rec);
    pair_candidates<MFLAG>(I, C, g1, jg0 + 2, js, is, rec);
  }
  if (GPUNB_VOTE_EARLY) {
    pair_inv<REL>(g0);
    pair_inv<REL>(g1);
  }
  pair_acc(g0, q);
  pair_acc(g1, q);
}

// Eight j (four lane pairs) against one i, one warp vote for all.
template <bool MFLAG, bool REL>
__device__ __forceinline__ void pair8(const IState &I, const TileCtx &C, const JPair (&p)[4],
                                      f2 (&q)[NQ], int jg0, int jbase, const JSet &js,
                                      const ISet &is, const RegfOut &out, NbRec &rec) {
  PairGeo g[4];
#pragma unroll
  for (int u = 0; u < 4; ++u) pair_geo<REL>(I, C, p[u], g[u]);
  const float H = C.H;
  const bool any = pair_maybe(g[0], H) | pair_maybe(g[1], H) | pair_maybe(g[2], H) |
                   pair_maybe(g[3], H);
  if (__any_sync(0xffffffffu, any)) {
    nb_room(rec, I.i, jbase, js, out);
#pragma unroll
    for (int u = 0; u < 4; ++u) pair_candidates<MFLAG>(I, C, g[u], jg0 + 2 * u, js, is, rec);
  }
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    if (GPUNB_VOTE_EARLY) pair_inv<REL>(g[u]);
    pair_acc(g[u], q);
  }
}

// One warp's share [jbeg, jbeg + JW) of a tile against one i: the fields the
// path needs, JV j per shared-memory load, one warp vote per 4 (JV <= 4) or
// 8 j (JV = 8).
template <bool MFLAG, bool REL, int JV, int JW>
__device__ __forceinline__ void tile_pairs(const IState &I, const TileCtx &C,
                                           const float *__restrict__ T, int jbeg, f2 (&q)[NQ],
                                           int jg_tile, int jbase, const JSet &js,
                                           const ISet &is, const RegfOut &out, NbRec &rec) {
  constexpr int F0 = REL ? 0 : F_VX;
  constexpr int F1 = REL ? NFIELD_REL : NFIELD;
  if (JV == 8) {
    for (int jj = jbeg; jj < jbeg + JW; jj += 8) {
      JPair p[4];
#pragma unroll
      for (int f = F0; f < F1; ++f) {
        const float4 u = *(const float4 *)(T + f * JT + jj);
        const float4 w4 = *(const float4 *)(T + f * JT + jj + 4);
        p[0].v[f] = make_float2(u.x, u.y);
        p[1].v[f] = make_float2(u.z, u.w);
        p[2].v[f] = make_float2(w4.x, w4.y);
        p[3].v[f] = make_float2(w4.z, w4.w);
      }
      pair8<MFLAG, REL>(I, C, p, q, jg_tile + jj, jbase, js, is, out, rec);
    }
  } else {
    for (int jj = jbeg; jj < jbeg + JW; jj += 4) {
      JPair p0, p1;
      if (JV == 2) {
#pragma unroll
        for (int f = F0; f < F1; ++f) {
          p0.v[f] = *(const f2 *)(T + f * JT + jj);
          p1.v[f] = *(const f2 *)(T + f * JT + jj + 2);
        }
      } else {
#pragma unroll
        for (int f = F0; f < F1; ++f) {
          const float4 u = *(const float4 *)(T + f * JT + jj);
          p0.v[f] = make_float2(u.x, u.y);
          p1.v[f] = make_float2(u.z, u.w);
        }
      }
      pair4<MFLAG, REL>(I, C, p0, p1, q, jg_tile + jj, jbase, js, is, out, rec);
    }
  }
}

// ---------------------------------------------------------------------------
// Merge of the j-split partial sums (merge kernels and the merge in the pair
// kernel).
__device__ __forceinline__ void merge_store(const double *s, int i, const int *__restrict__ cnt,
                                            int nnbmax, double *__restrict__ acc,
                                            double *__restrict__ jrk, double *__restrict__ pot,
                                            int *__restrict__ nnb, int *__restrict__ rowlen) {
  acc[3 * i + 0] = 0.25 * s[0];
  acc[3 * i + 1] = 0.25 * s[1];
  acc[3 * i + 2] = 0.25 * s[2];
  jrk[3 * i + 0] = 0.25 * s[3];
  jrk[3 * i + 1] = 0.25 * s[4];
  jrk[3 * i + 2] = 0.25 * s[5];
  pot[i] = s[6];
  const int c = cnt[i];
  const bool over = c > nnbmax;
  nnb[i] = over ? -c : c;
  rowlen[i] = over ? 0 : c;
}

// Partial sums are stored by processing slot (column); the result of slot s
// belongs to i = perm[s] (identity without a permutation).  The split kernel
// stores each partial as a float-float pair (hi, lo) in the 8-byte slot and
// the merges add those pairs exactly-rounded on the FP32 pipe (FF); the FP64
// kernel stores doubles, added in FP64.  Either way the order is fixed.
template <bool FF>
struct PartAcc {
  double d[NQ];
  float h[NQ], l[NQ];
  __device__ __forceinline__ PartAcc() {
#pragma unroll
    for (int c = 0; c < NQ; ++c) {
      d[c] = 0.0;
      h[c] = l[c] = 0.f;
    }
  }
  // adds partial c, loaded as the 8 bytes of its slot (for FF the float
  // pair (hi, lo) at the slot's low and high 4 bytes)
  __device__ __forceinline__ void add_slot(int c, double v) {
    if (FF) {
      const unsigned long long b = (unsigned long long)__double_as_longlong(v);
      ff_add(h[c], l[c], __int_as_float((int)(unsigned int)b), __int_as_float((int)(b >> 32)));
    } else {
      d[c] += v;
    }
  }
  // adds the NQ partials of one split, entry c at p[c * stride]
  __device__ __forceinline__ void add(const double *__restrict__ p, size_t stride) {
#pragma unroll
    for (int c = 0; c < NQ; ++c) add_slot(c, p[c * stride]);
  }
  __device__ __forceinline__ double value(int c) const {
    return FF ? (double)h[c] + (double)l[c] : d[c];
  }
};

// ---------------------------------------------------------------------------
// Split-precision pair kernel, persistent.
//   IPT : i-particles per thread (independent chains)
//   WI  : warps along i;  WJ : warps splitting each j tile (same i's)
// Work items are (i-tile it, j-split s) pairs, split s covering tiles
// [s*ntile/S, (s+1)*ntile/S); a block takes items from the device queue until
// it is empty.  Queue order: item = s * n_itiles + it (the i-tiles of one
// split side by side, its j tiles hot in L2), or with out.done item =
// it * S + s (an i-tile's splits side by side, finishing close together) and
// the block that completes an i-tile's last item merges the tile
// (merge_itile).  The j tiles of an item stream through a
// NSTAGE-deep shared-memory ring filled by bulk-async copies; the last warp
// to finish with a stage refills it, so warps are never held at a block-wide
// barrier inside an item.  Stage phases run on a per-block tile counter g
// that continues across items.
#ifndef GPUNB_NSTAGE
#define GPUNB_NSTAGE 4
#endif
constexpr int NSTAGE = GPUNB_NSTAGE;

struct RegfWork {
  int *queue;              // item counter, zeroed before the launch
  int n_itiles;            // single j-set: items are (i-tile, split) pairs
  int S;
  const ItemDesc *items;   // batched clusters: explicit item table (else null)
  const int *order;        // queue position -> item (largest first), or null
  int n_items;
};

// The merge of one i-tile (slots [slot0, slot0 + itile) of the partial rows,
// columns from pcol0) by the block that completed its last item: the S rows
// summed in split order per slot (float-float, then FP64 as the merge
// kernels), the results stored, and the merged rows' L2 lines discarded --
// they are dead, and would otherwise be written back to DRAM.
__device__ __forceinline__ void merge_itile(const RegfOut &out, int S, int slot0, int slot_end,
                                            int pcol0, int itile) {
  const size_t rs = (size_t)NQ * out.ni_pad;   // doubles per partial row
  for (int u = threadIdx.x; u < itile; u += blockDim.x) {
    const int slot = slot0 + u;
    if (slot >= slot_end) break;
    const double *p = out.part + pcol0 + u;
    PartAcc<true> a;
    int k = 0;
    for (; k + 4 <= S; k += 4) {   // four rows' loads in flight, added in row order
      double v[4][NQ];
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < NQ; ++c) v[r][c] = __ldcg(p + (k + r) * rs + (size_t)c * out.ni_pad);
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < NQ; ++c) a.add_slot(c, v[r][c]);
    }
    for (; k < S; ++k)
#pragma unroll
      for (int c = 0; c < NQ; ++c) a.add_slot(c, __ldcg(p + k * rs + (size_t)c * out.ni_pad));
    double sv[NQ];
#pragma unroll
    for (int c = 0; c < NQ; ++c) sv[c] = a.value(c);
    merge_store(sv, out.perm ? out.perm[slot] : slot, out.cnt, out.nnbmax, out.acc, out.jrk,
                out.pot, out.nnb, out.rowlen);
  }
  __syncthreads();   // every read of the rows done
  // 128-byte lines: the tile's columns (itile x 8 bytes, a multiple of 128
  // from a multiple of 128) in each of the S x NQ row segments
  const int lines = itile * 8 / 128;
  for (int e = threadIdx.x; e < S * NQ * lines; e += blockDim.x) {
    const int seg = e / lines, l = e - seg * lines;
    const double *a = out.part + (size_t)seg * out.ni_pad + pcol0 + l * 16;
    asm volatile("discard.global.L2 [%0], 128;" ::"l"(a) : "memory");
  }
}

// Slot within the i-tile of (warp along i, i index of the thread, lane):
// contiguous runs of 32 per warp, or with GPUNB_WARP_INTERLEAVE the tile's
// slots dealt round-robin over its warps (each warp then spans the tile).
#ifndef GPUNB_WARP_INTERLEAVE
#define GPUNB_WARP_INTERLEAVE 0
#endif
template <int IPT, int WI>
__device__ __forceinline__ int itile_slot(int wi, int k, int lane) {
  return GPUNB_WARP_INTERLEAVE ? (k * 32 + lane) * WI + wi : wi * 32 * IPT + k * 32 + lane;
}

template <int IPT, int WI, int WJ, int JV, bool MFLAG, int MINB>
__global__ void __launch_bounds__(32 * WI * WJ, MINB)
    regf_ds_kernel(const JSet js, const ISet is, const RegfOut out, const RegfWork w) {
  constexpr int NT = 32 * WI * WJ;
  constexpr int NW = NT / 32;
  constexpr int ITILE = 32 * IPT * WI;
  constexpr int JW = JT / WJ;
  static_assert(JW % JV == 0 && JW % 4 == 0 && (JV == 2 || JV == 4 || JV == 8),
                "j per warp must be a multiple of JV and of 4");
  extern __shared__ __align__(128) float smem[];
  float *ring = smem;                                   // NSTAGE * TILE_FLOATS
  float *ffs = smem + NSTAGE * TILE_FLOATS;             // [2][NQ][IPT][NT] float-float
  int *nbuf = reinterpret_cast<int *>(ffs + 2 * NQ * IPT * NT);   // [NBUF][IPT][NT]
  __shared__ __align__(8) uint64_t bar[NSTAGE];
  __shared__ int s_rel[NSTAGE];                         // warps done with the stage
  __shared__ int s_iss[NSTAGE];                         // copies issued into the stage
  __shared__ int s_item, s_abort, s_last;

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wi = warp % WI, wj = warp / WI;
  const int n_items = w.items ? w.n_items : w.n_itiles * w.S;

  if (tid == 0) {
    for (int u = 0; u < NSTAGE; ++u) {
      mbar_init(&bar[u], 1);
      s_rel[u] = 0;
      s_iss[u] = 0;
    }
    fence_mbar_init();
    s_abort = 0;
  }
  __syncthreads();

  int g = 0;   // tiles consumed by this block so far (uniform)
  for (;;) {
    if (tid == 0) s_item = atomicAdd(w.queue, 1);
    __syncthreads();
    const int qpos = s_item;
    if (qpos >= n_items || s_abort) break;
    int slot0, slot_end, t0, t1, prow, jbase, pcol0;
    if (w.items) {
      const ItemDesc d = w.items[w.order ? w.order[qpos] : qpos];
      slot0 = d.slot0; slot_end = d.slot_end; t0 = d.t0; t1 = d.t1;
      prow = d.prow; jbase = d.jbase; pcol0 = d.pcol0;
    } else {
      // with the merge in the kernel an i-tile's splits follow one another;
      // otherwise the i-tiles of one split do (the split's j tiles hot in L2)
      int it, sy;
      if (out.done) {
        it = qpos / w.S;
        sy = qpos - it * w.S;
      } else {
        sy = qpos / w.n_itiles;
        it = qpos - sy * w.n_itiles;
      }
      slot0 = it * ITILE; slot_end = is.ni;
      t0 = (int)(((long long)js.ntile * sy) / w.S);
      t1 = (int)(((long long)js.ntile * (sy + 1)) / w.S);
      prow = sy; jbase = 0; pcol0 = slot0;
    }
    const int nt = t1 - t0;
    if (tid == 0) {
      for (int u = 0; u < NSTAGE && u < nt; ++u) {
        const int st = (g + u) % NSTAGE;
        s_iss[st]++;
        mbar_expect_tx(&bar[st], TILE_BYTES);
        bulk_g2s(ring + st * TILE_FLOATS, js.tiles + (size_t)(t0 + u) * TILE_FLOATS, TILE_BYTES,
                 &bar[st]);
      }
    }

    IState I[IPT];
    f2 q[IPT][NQ];
    NbRec rec[IPT];
#pragma unroll
    for (int k = 0; k < IPT; ++k) {
      rec[k].buf = nbuf + k * NT + tid;
      rec[k].stride = IPT * NT;
      rec[k].n = 0;
      const int slot = slot0 + itile_slot<IPT, WI>(wi, k, lane);
      load_istate(I[k], is.rec, slot, slot < slot_end);
#pragma unroll
      for (int c = 0; c < NQ; ++c) {
        q[k][c] = make_float2(0.f, 0.f);
        ffs[((0 * NQ + c) * IPT + k) * NT + tid] = 0.f;
        ffs[((1 * NQ + c) * IPT + k) * NT + tid] = 0.f;
      }
    }

    for (int t = 0; t < nt; ++t) {
      const int st = (g + t) % NSTAGE;
      const uint32_t par = (uint32_t)((g + t) / NSTAGE) & 1u;
      if (!mbar_wait_bounded(&bar[st], par)) s_abort = 1;
      if (*(volatile int *)&s_abort) break;
      const float *T = ring + st * TILE_FLOATS;
      const float *M = T + NFIELD * JT;
      const float vmax = M[M_VMAX], smax = M[M_SMAX], rad = M[M_RAD];
      const float ohx = M[M_OH], ohy = M[M_OH + 1], ohz = M[M_OH + 2];
      const float bx = M[M_BOX], by = M[M_BOX + 1], bz = M[M_BOX + 2];
      const int jbeg = wj * JW;
#pragma unroll
      for (int k = 0; k < IPT; ++k) {
        TileCtx C;
        // O - x_i from the double-single parts, rounded once to FP32
        C.ox = mk2(__fadd_rn(__fadd_rn(ohx, I[k].nxh), I[k].nxl));
        C.oy = mk2(__fadd_rn(__fadd_rn(ohy, I[k].nyh), I[k].nyl));
        C.oz = mk2(__fadd_rn(__fadd_rn(ohz, I[k].nzh), I[k].nzl));
        const float base = I[k].dv * (I[k].va + vmax);
        float b = MFLAG ? fmaf(I[k].s, smax, base) : I[k].s + base;
        b = fmaf(rad, 0x1p-20f, b);   // the tile-relative rounding, 2^-22 (R + r) per axis
        C.H = (I[k].s < 0.f) ? -1.0f : b * b;
        C.R = rad;
        // The tile-relative difference (x_j - O) + o errs by less than
        // 2^-24 (R + |o| + |dx|) per component.  Every j of the tile lies at
        // least max(|o| - R, d_box) from x_i (d_box: distance to the tile's
        // box); while that bound is at least (R + |o|)/3 the error stays
        // below 2^-22 |dx|, as for every tile with |o| >= 2R.  A tile where
        // the bound fails for a lane of the warp (|o| < 2R and
        // R + |o| > 3 d_box) is near and takes the double-single path.
        const float o2 = C.ox.x * C.ox.x + C.oy.x * C.oy.x + C.oz.x * C.oz.x;
        bool near = (I[k].s >= 0.f) && (o2 < GPUNB_NEAR_K2 * rad * rad);
        if (near) {
          const float ex = fmaxf(fabsf(C.ox.x) - bx, 0.f);
          const float ey = fmaxf(fabsf(C.oy.x) - by, 0.f);
          const float ez = fmaxf(fabsf(C.oz.x) - bz, 0.f);
          const float ro = rad + sqrtf(o2);
          near = ro * ro > 9.0f * (ex * ex + ey * ey + ez * ez);
        }
        if (__any_sync(0xffffffffu, near)) {
          C.nxh = mk2(I[k].nxh); C.nyh = mk2(I[k].nyh); C.nzh = mk2(I[k].nzh);
          C.nxl = mk2(I[k].nxl); C.nyl = mk2(I[k].nyl); C.nzl = mk2(I[k].nzl);
          tile_pairs<MFLAG, false, JV, JW>(I[k], C, T, jbeg, q[k], (t0 + t) * JT, jbase, js, is,
                                           out, rec[k]);
        } else {
          tile_pairs<MFLAG, true, JV, JW>(I[k], C, T, jbeg, q[k], (t0 + t) * JT, jbase, js, is,
                                          out, rec[k]);
        }
      }
      // fold the FP32 chunk sums into the float-float accumulators
      if (GPUNB_FOLD_TILES == 1 || (t + 1) % GPUNB_FOLD_TILES == 0 || t + 1 == nt) {
#pragma unroll
        for (int k = 0; k < IPT; ++k) {
#pragma unroll
          for (int c = 0; c < NQ; ++c) {
            float &hi = ffs[((0 * NQ + c) * IPT + k) * NT + tid];
            float &lo = ffs[((1 * NQ + c) * IPT + k) * NT + tid];
            float h = hi, l = lo;
            ff_accum(h, l, __fadd_rn(q[k][c].x, q[k][c].y));
            hi = h; lo = l;
            q[k][c] = make_float2(0.f, 0.f);
          }
        }
      }
      // release the stage; the last warp out refills it with tile t + NSTAGE
      __syncwarp();
      if (lane == 0) {
        __threadfence_block();
        const int done = atomicAdd(&s_rel[st], 1);
        if (done == NW - 1) {
          s_rel[st] = 0;
          if (t + NSTAGE < nt) {
            s_iss[st]++;
            mbar_expect_tx(&bar[st], TILE_BYTES);
            bulk_g2s(ring + st * TILE_FLOATS, js.tiles + (size_t)(t0 + t + NSTAGE) * TILE_FLOATS,
                     TILE_BYTES, &bar[st]);
          }
        }
      }
    }
#pragma unroll
    for (int k = 0; k < IPT; ++k) nb_flush(rec[k], I[k].i, jbase, js.perm, out);
    g += nt;
    __syncthreads();
    if (s_abort) break;

    // fixed-order merge of the WJ j-subranges (warps wj > 0 into wj == 0)
    if (WJ > 1 && wj == 0) {
#pragma unroll
      for (int k = 0; k < IPT; ++k)
#pragma unroll
        for (int c = 0; c < NQ; ++c) {
          float h = ffs[((0 * NQ + c) * IPT + k) * NT + tid];
          float l = ffs[((1 * NQ + c) * IPT + k) * NT + tid];
          for (int u = 1; u < WJ; ++u) {
            const int src = tid + u * 32 * WI;
            ff_add(h, l, ffs[((0 * NQ + c) * IPT + k) * NT + src],
                   ffs[((1 * NQ + c) * IPT + k) * NT + src]);
          }
          ffs[((0 * NQ + c) * IPT + k) * NT + tid] = h;
          ffs[((1 * NQ + c) * IPT + k) * NT + tid] = l;
        }
    }
    if (wj == 0) {
#pragma unroll
      for (int k = 0; k < IPT; ++k) {
        if (I[k].i < 0) continue;
        const int col = pcol0 + itile_slot<IPT, WI>(wi, k, lane);
#pragma unroll
        for (int c = 0; c < NQ; ++c) {
          const float2 v = make_float2(ffs[((0 * NQ + c) * IPT + k) * NT + tid],
                                       ffs[((1 * NQ + c) * IPT + k) * NT + tid]);
          reinterpret_cast<float2 *>(out.part)[((size_t)prow * NQ + c) * out.ni_pad + col] = v;
        }
      }
    }
    if (out.done && !w.items) {
      __threadfence();   // this item's rows (and neighbour counts) visible before its count
      __syncthreads();
      if (tid == 0) s_last = atomicAdd(out.done + qpos / w.S, 1) == w.S - 1;
      __syncthreads();
      if (s_last) {
        __threadfence();   // the rows of the tile's other items, counted before, are visible
        merge_itile(out, w.S, slot0, slot_end, pcol0, ITILE);
      }
    }
    __syncthreads();   // ffs and s_item are reused by the next item
  }
  if (s_abort && tid == 0) {
    // let copies still in flight land before the block exits
    for (int u = 0; u < NSTAGE; ++u)
      if (s_iss[u] > 0) mbar_wait_bounded(&bar[u], (uint32_t)(s_iss[u] - 1) & 1u, 1u << 16);
    raise_error(out.err, GPUNB_E_TIMEOUT);
  }
}

__device__ __forceinline__ void record_neighbour(const RegfOut &out, int i, int j) {
  const int slot = atomicAdd(out.cnt + i, 1);
  if (slot < out.cap) out.rows[(size_t)i * out.cap + slot] = j;
}

// ---------------------------------------------------------------------------
// Plain FP64 pair kernel (the FP64 baseline of the metric): regint.f:39-79
// arithmetic, j in FP64 staged through shared memory, one i per thread.
template <bool MFLAG>
__global__ void __launch_bounds__(128) regf_fp64_kernel(const JSet js, const ISet is,
                                                        const RegfOut out) {
  constexpr int NT = 128;
  __shared__ double sx[JT64 * 3], sv[JT64 * 3], sm[JT64];
  const int tid = threadIdx.x;
  const int i = blockIdx.x * NT + tid;
  const bool valid = i < is.ni;
  const int ns = gridDim.y, sy = blockIdx.y;
  const int t0 = (int)(((long long)js.ntile64 * sy) / ns);
  const int t1 = (int)(((long long)js.ntile64 * (sy + 1)) / ns);
  double xi0 = 0, xi1 = 0, xi2 = 0, vi0 = 0, vi1 = 0, vi2 = 0, h2 = -1, dtr = 0;
  if (valid) {
    xi0 = is.x[3 * i]; xi1 = is.x[3 * i + 1]; xi2 = is.x[3 * i + 2];
    vi0 = is.v[3 * i]; vi1 = is.v[3 * i + 1]; vi2 = is.v[3 * i + 2];
    h2 = is.h2[i]; dtr = is.dtr[i];
    if (sy == 0 && (isnan(xi0) || isnan(xi1) || isnan(xi2) || isnan(vi0) || isnan(vi1) ||
                    isnan(vi2) || isnan(h2) || isnan(dtr)))
      raise_error(out.err, GPUNB_E_NAN);
  }
  double ax = 0, ay = 0, az = 0, jx = 0, jy = 0, jz = 0, po = 0;
  for (int t = t0; t < t1; ++t) {
    const int jb = t * JT64;
    const int n = min(JT64, js.nj - jb);
    __syncthreads();
    for (int u = tid; u < 3 * n; u += NT) { sx[u] = js.x64[3 * jb + u]; sv[u] = js.v64[3 * jb + u]; }
    for (int u = tid; u < n; u += NT) sm[u] = js.m64[jb + u];
    __syncthreads();
    if (!valid) continue;
    for (int jj = 0; jj < n; ++jj) {
      const double dx = __dadd_rn(sx[3 * jj], -xi0);
      const double dy = __dadd_rn(sx[3 * jj + 1], -xi1);
      const double dz = __dadd_rn(sx[3 * jj + 2], -xi2);
      const double dvx = __dadd_rn(sv[3 * jj], -vi0);
      const double dvy = __dadd_rn(sv[3 * jj + 1], -vi1);
      const double dvz = __dadd_rn(sv[3 * jj + 2], -vi2);
      const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
      const double px = __dadd_rn(dx, __dmul_rn(dvx, dtr));
      const double py = __dadd_rn(dy, __dmul_rn(dvy, dtr));
      const double pz = __dadd_rn(dz, __dmul_rn(dvz, dtr));
      const double r2p = __dadd_rn(__dadd_rn(__dmul_rn(px, px), __dmul_rn(py, py)), __dmul_rn(pz, pz));
      const double r2min = r2 < r2p ? r2 : r2p;
      const double crit = MFLAG ? __dmul_rn(sm[jj], h2) : h2;
      if (r2min < crit) {
        record_neighbour(out, i, jb + jj);
        continue;
      }
      // 1/r with the FP64 reciprocal square root (rsqrt), not an FP64
      // division and square root, which cost about as many FP64 instructions
      // as the rest of the pair on a part whose FP64 pipe runs at 1/64 of the
      // FP32 rate
      const double y = rsqrt(r2);
      const double dr2i = y * y;
      const double mr = sm[jj] * y;              // m/r
      const double dr3i = mr * dr2i;             // m/r^3
      const double drdp = 3.0 * (dx * dvx + dy * dvy + dz * dvz) * dr2i;
      ax += dx * dr3i; ay += dy * dr3i; az += dz * dr3i;
      jx += (dvx - dx * drdp) * dr3i;
      jy += (dvy - dy * drdp) * dr3i;
      jz += (dvz - dz * drdp) * dr3i;
      po += mr;
    }
  }
  if (valid) {
    // same partial layout as the split kernel, which stores 4x acc/jrk
    double *p = out.part + (size_t)sy * NQ * out.ni_pad + i;
    p[0 * out.ni_pad] = 4.0 * ax; p[1 * out.ni_pad] = 4.0 * ay; p[2 * out.ni_pad] = 4.0 * az;
    p[3 * out.ni_pad] = 4.0 * jx; p[4 * out.ni_pad] = 4.0 * jy; p[5 * out.ni_pad] = 4.0 * jz;
    p[6 * out.ni_pad] = po;
  }
}

// Double-float pair kernel (gpunb_set_precision(2)): the FP64 kernel's
// structure and semantics with every pair computed in double-float
// arithmetic on the FP32 pipe (df_* in common.cuh): FP64-class results --
// force, jerk and potential within ~1e-11 of FP64 -- several times faster
// than FP64 on GB300.  The j tile is split into double-single positions,
// velocities and masses once per tile in shared memory; the neighbour
// decision compares the double-float min(r^2, r_p^2) with the criterion and
// re-takes it in the oracle's FP64 expression order (nb_test_fp64) whenever
// the two lie within 2^-40 of each other, so that the lists are the FP64
// oracle's exactly.
template <bool MFLAG>
__global__ void __launch_bounds__(128) regf_df_kernel(const JSet js, const ISet is,
                                                      const RegfOut out) {
  constexpr int NT = 128;
  __shared__ float sxh[JT64 * 3], sxl[JT64 * 3], svh[JT64 * 3], svl[JT64 * 3];
  __shared__ float smh[JT64], sml[JT64];
  const int tid = threadIdx.x;
  const int i = blockIdx.x * NT + tid;
  const bool valid = i < is.ni;
  const int ns = gridDim.y, sy = blockIdx.y;
  const int t0 = (int)(((long long)js.ntile64 * sy) / ns);
  const int t1 = (int)(((long long)js.ntile64 * (sy + 1)) / ns);
  float xh[3] = {0.f, 0.f, 0.f}, xl[3] = {0.f, 0.f, 0.f};
  float vh[3] = {0.f, 0.f, 0.f}, vl[3] = {0.f, 0.f, 0.f};
  dfl h2 = {-1.f, 0.f}, dtr = {0.f, 0.f};
  if (valid) {
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      ds_split(is.x[3 * i + c], xh[c], xl[c]);
      ds_split(is.v[3 * i + c], vh[c], vl[c]);
    }
    const double h2d = is.h2[i], dtrd = is.dtr[i];
    ds_split(h2d, h2.h, h2.l);
    ds_split(dtrd, dtr.h, dtr.l);
    if (sy == 0 && (isnan(is.x[3 * i]) || isnan(is.x[3 * i + 1]) || isnan(is.x[3 * i + 2]) ||
                    isnan(is.v[3 * i]) || isnan(is.v[3 * i + 1]) || isnan(is.v[3 * i + 2]) ||
                    isnan(h2d) || isnan(dtrd)))
      raise_error(out.err, GPUNB_E_NAN);
  }
  dfl q[NQ];
#pragma unroll
  for (int c = 0; c < NQ; ++c) q[c] = {0.f, 0.f};
  for (int t = t0; t < t1; ++t) {
    const int jb = t * JT64;
    const int n = min(JT64, js.nj - jb);
    __syncthreads();
    for (int u = tid; u < 3 * n; u += NT) {
      ds_split(js.x64[3 * (size_t)jb + u], sxh[u], sxl[u]);
      ds_split(js.v64[3 * (size_t)jb + u], svh[u], svl[u]);
    }
    for (int u = tid; u < n; u += NT) ds_split(js.m64[jb + u], smh[u], sml[u]);
    __syncthreads();
    if (!valid) continue;
    for (int jj = 0; jj < n; ++jj) {
      const dfl dx = df_diff(sxh[3 * jj], sxl[3 * jj], xh[0], xl[0]);
      const dfl dy = df_diff(sxh[3 * jj + 1], sxl[3 * jj + 1], xh[1], xl[1]);
      const dfl dz = df_diff(sxh[3 * jj + 2], sxl[3 * jj + 2], xh[2], xl[2]);
      const dfl dvx = df_diff(svh[3 * jj], svl[3 * jj], vh[0], vl[0]);
      const dfl dvy = df_diff(svh[3 * jj + 1], svl[3 * jj + 1], vh[1], vl[1]);
      const dfl dvz = df_diff(svh[3 * jj + 2], svl[3 * jj + 2], vh[2], vl[2]);
      const dfl r2 = df_add(df_add(df_sqr(dx), df_sqr(dy)), df_sqr(dz));
      const dfl m = {smh[jj], sml[jj]};
      const dfl crit = MFLAG ? df_mul(m, h2) : h2;
      // r_p^2 in double-float only where it can decide: an FP32 lower bound
      // first -- each predicted component from the heads, less 2^-21 of the
      // magnitudes involved (the tails are at most 2^-24 of their heads and
      // the FMA rounds once: several times the worst case); NaN or infinite
      // inputs give a bound of 0.  Where the bound clears the criterion by
      // 2^-16, r_p^2 is no smaller than the criterion, so min(r^2, r_p^2)
      // decides exactly as r^2 alone does.
      dfl r2min = r2;
      {
        const float qx = fmaf(dvx.h, dtr.h, dx.h), qy = fmaf(dvy.h, dtr.h, dy.h),
                    qz = fmaf(dvz.h, dtr.h, dz.h);
        const float dt = fabsf(dtr.h);
        const float ax = fmaxf(fabsf(qx) - 0x1p-21f * (fabsf(qx) + fmaf(fabsf(dvx.h), dt,
                                                                        fabsf(dx.h))), 0.f);
        const float ay = fmaxf(fabsf(qy) - 0x1p-21f * (fabsf(qy) + fmaf(fabsf(dvy.h), dt,
                                                                        fabsf(dy.h))), 0.f);
        const float az = fmaxf(fabsf(qz) - 0x1p-21f * (fabsf(qz) + fmaf(fabsf(dvz.h), dt,
                                                                        fabsf(dz.h))), 0.f);
        const float lb = fmaf(ax, ax, fmaf(ay, ay, az * az));
        if (!(lb >= fmaf(crit.h, 1.0f + 0x1p-16f, 0x1p-100f))) {
          const dfl px = df_add(dx, df_mul(dvx, dtr));
          const dfl py = df_add(dy, df_mul(dvy, dtr));
          const dfl pz = df_add(dz, df_mul(dvz, dtr));
          const dfl r2p = df_add(df_add(df_sqr(px), df_sqr(py)), df_sqr(pz));
          if (r2p.h < r2.h || (r2p.h == r2.h && r2p.l < r2.l)) r2min = r2p;
        }
      }
      const dfl diff = df_add(r2min, {-crit.h, -crit.l});
      bool in;
      if (fabsf(diff.h) <= 0x1p-40f * fabsf(crit.h))
        in = nb_test_fp64(is, i, js, jb + jj, MFLAG);   // the oracle's own decision
      else
        in = diff.h < 0.f;
      if (in) {
        record_neighbour(out, i, jb + jj);
        continue;
      }
      if (r2.h < 0x1p-126f) continue;   // a body closer than 1e-19 that is no neighbour
      // 1/r: estimate y0, then y0 (1 + (1 - r2 y0^2) / 2) with r2 y0^2 in double-float
      const float y0 = rsqrt_est(r2.h);
      const float y2 = __fmul_rn(y0, y0);
      const dfl tq = df_mul(r2, {y2, fmaf(y0, y0, -y2)});
      const float e = __fsub_rn(__fsub_rn(1.0f, tq.h), tq.l);
      const dfl rinv = df_fast(y0, __fmul_rn(__fmul_rn(0.5f, y0), e));
      const dfl rinv2 = df_sqr(rinv);
      const dfl mr = df_mul(m, rinv);                     // m/r
      const dfl mr3 = df_mul(mr, rinv2);                  // m/r^3
      const dfl rv = df_add(df_add(df_mul(dx, dvx), df_mul(dy, dvy)), df_mul(dz, dvz));
      const dfl al = df_mulf(df_mul(rv, rinv2), -3.0f);  // -3 (r.v)/r^2
      q[0] = df_add(q[0], df_mul(mr3, dx));
      q[1] = df_add(q[1], df_mul(mr3, dy));
      q[2] = df_add(q[2], df_mul(mr3, dz));
      q[3] = df_add(q[3], df_mul(mr3, df_add(dvx, df_mul(al, dx))));
      q[4] = df_add(q[4], df_mul(mr3, df_add(dvy, df_mul(al, dy))));
      q[5] = df_add(q[5], df_mul(mr3, df_add(dvz, df_mul(al, dz))));
      q[6] = df_add(q[6], mr);
    }
  }
  if (valid) {
    // the FP64 kernel's partial layout (4x acc and jrk, as the split kernel)
    double *p = out.part + (size_t)sy * NQ * out.ni_pad + i;
#pragma unroll
    for (int c = 0; c < NQ; ++c)
      p[c * out.ni_pad] = (c < 6 ? 4.0 : 1.0) * ((double)q[c].h + (double)q[c].l);
  }
}

// ---------------------------------------------------------------------------
// Merge of the S j-split partials, fixed order s = 0..S-1 (the
// deterministic replacement of force_reduce_kernel + the host sum over GPUs,
// gpunb.velocity.cu:441-496,822-845).  Also turns counts into the in-band
// overflow flag of gpunb.velocity.cu:872-877 / reg.avx.cpp:320-321.
//
// Many j-splits (small active blocks): one block of MERGE_THREADS per slot,
// each thread summing a strided subset of the splits (four splits' loads in
// flight at a time, added in split order), then a fixed shared-memory tree,
// so the order of the FP64 additions is the same in every run.
constexpr int MERGE_THREADS = 128;
constexpr int MERGE_UNROLL = 4;
template <bool FF>
__global__ void __launch_bounds__(MERGE_THREADS)
    regf_merge_wide_kernel(const double *__restrict__ part, int S, int ni, int ni_pad,
                           const int *__restrict__ perm, const int *__restrict__ cnt, int nnbmax,
                           double *__restrict__ acc, double *__restrict__ jrk,
                           double *__restrict__ pot, int *__restrict__ nnb,
                           int *__restrict__ rowlen) {
  __shared__ double sh[NQ][MERGE_THREADS];
  const int slot = blockIdx.x, t = threadIdx.x;
  PartAcc<FF> acc_t;
  for (int k0 = t; k0 < S; k0 += MERGE_THREADS * MERGE_UNROLL) {
    // four splits' loads in flight, then added in split order
    double a[MERGE_UNROLL][NQ];
#pragma unroll
    for (int u = 0; u < MERGE_UNROLL; ++u) {
      const int k = k0 + u * MERGE_THREADS;
      const double *p = part + (size_t)k * NQ * ni_pad + slot;
#pragma unroll
      for (int c = 0; c < NQ; ++c) a[u][c] = (k < S) ? p[(size_t)c * ni_pad] : 0.0;
    }
#pragma unroll
    for (int u = 0; u < MERGE_UNROLL; ++u)
#pragma unroll
      for (int c = 0; c < NQ; ++c) acc_t.add_slot(c, a[u][c]);
  }
  double s[NQ];
#pragma unroll
  for (int c = 0; c < NQ; ++c) sh[c][t] = acc_t.value(c);
  __syncthreads();
  for (int w = MERGE_THREADS / 2; w > 0; w >>= 1) {
    if (t < w) {
#pragma unroll
      for (int c = 0; c < NQ; ++c) sh[c][t] += sh[c][t + w];
    }
    __syncthreads();
  }
  if (t == 0) {
#pragma unroll
    for (int c = 0; c < NQ; ++c) s[c] = sh[c][0];
    merge_store(s, perm ? perm[slot] : slot, cnt, nnbmax, acc, jrk, pot, nnb, rowlen);
  }
}

// Large blocks: a block of MERGE_KW warps per 32 consecutive slots, lane =
// slot, warp w summing the splits w, w + MERGE_KW, ... in order (reads
// coalesced across the warp), then the MERGE_KW partial sums of a slot added
// in warp order: the same FP64 order in every run, with MERGE_KW times the
// memory parallelism of a thread per slot.
constexpr int MERGE_KW = 8;
template <bool FF>
__global__ void __launch_bounds__(32 * MERGE_KW)
    regf_merge_kernel(const double *__restrict__ part, int S, int ni, int ni_pad,
                      const int *__restrict__ perm, const int *__restrict__ cnt, int nnbmax,
                      double *__restrict__ acc, double *__restrict__ jrk, double *__restrict__ pot,
                      int *__restrict__ nnb, int *__restrict__ rowlen) {
  __shared__ double sh[MERGE_KW][NQ][32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int slot = blockIdx.x * 32 + lane;
  PartAcc<FF> acc_t;
  if (slot < ni) {
    for (int k = w; k < S; k += MERGE_KW)
      acc_t.add(part + (size_t)k * NQ * ni_pad + slot, (size_t)ni_pad);
  }
  double s[NQ];
#pragma unroll
  for (int c = 0; c < NQ; ++c) sh[w][c][lane] = acc_t.value(c);
  __syncthreads();
  if (w == 0 && slot < ni) {
#pragma unroll
    for (int c = 0; c < NQ; ++c) {
      double t = sh[0][c][lane];
      for (int u = 1; u < MERGE_KW; ++u) t += sh[u][c][lane];
      s[c] = t;
    }
    merge_store(s, perm ? perm[slot] : slot, cnt, nnbmax, acc, jrk, pot, nnb, rowlen);
  }
}

// Batched clusters: one block per i-tile; the tile's splits are the partial
// rows row0 .. row0+nrow-1 (stride itile), summed in row order.
__global__ void regf_merge_batch_kernel(const double *__restrict__ part,
                                        const int4 *__restrict__ tiles, int itile,
                                        const int *__restrict__ perm,
                                        const int *__restrict__ cnt, int nnbmax,
                                        double *__restrict__ acc, double *__restrict__ jrk,
                                        double *__restrict__ pot, int *__restrict__ nnb,
                                        int *__restrict__ rowlen) {
  const int4 td = tiles[blockIdx.x];   // slot0, nslots, row0, nrow
  for (int u = threadIdx.x; u < td.y; u += blockDim.x) {
    PartAcc<true> acc_t;   // the batched pair is always the split kernel
    for (int k = 0; k < td.w; ++k)
      acc_t.add(part + (size_t)(td.z + k) * NQ * itile + u, (size_t)itile);
    double s[NQ];
#pragma unroll
    for (int c = 0; c < NQ; ++c) s[c] = acc_t.value(c);
    merge_store(s, perm[td.x + u], cnt, nnbmax, acc, jrk, pot, nnb, rowlen);
  }
}

// ---------------------------------------------------------------------------
// Exclusive scan of row lengths: per-block scan (SCAN_ITEMS per block) with
// block totals, then one block scanning the totals.  The gather adds the
// block offset, so no third pass is needed.
constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_PER_THREAD = 4;
constexpr int SCAN_ITEMS = SCAN_THREADS * SCAN_PER_THREAD;

__device__ __forceinline__ int block_exclusive_scan(int v, int *sh, int &total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int x = v;
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sh[warp] = x;
  __syncthreads();
  if (warp == 0) {
    int w = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    sh[lane] = w;
  }
  __syncthreads();
  const int before = (warp > 0) ? sh[warp - 1] : 0;
  total = sh[(blockDim.x >> 5) - 1];
  __syncthreads();
  return before + x - v;
}

__global__ void __launch_bounds__(SCAN_THREADS) list_scan_blocks_kernel(
    const int *__restrict__ len, int n, int *__restrict__ off, int *__restrict__ btotal) {
  __shared__ int sh[32];
  const int base = blockIdx.x * SCAN_ITEMS + threadIdx.x * SCAN_PER_THREAD;
  int v[SCAN_PER_THREAD], sum = 0;
#pragma unroll
  for (int u = 0; u < SCAN_PER_THREAD; ++u) {
    v[u] = (base + u < n) ? len[base + u] : 0;
    sum += v[u];
  }
  int total;
  int ex = block_exclusive_scan(sum, sh, total);
#pragma unroll
  for (int u = 0; u < SCAN_PER_THREAD; ++u) {
    if (base + u < n) off[base + u] = ex;
    ex += v[u];
  }
  if (threadIdx.x == 0) btotal[blockIdx.x] = total;
}

// scans up to SCAN_THREADS*SCAN_PER_THREAD block totals in place; writes the
// grand total to btotal[nb]
__global__ void __launch_bounds__(SCAN_THREADS) list_scan_totals_kernel(int *btotal, int nb) {
  __shared__ int sh[32];
  const int base = threadIdx.x * SCAN_PER_THREAD;
  int v[SCAN_PER_THREAD], sum = 0;
#pragma unroll
  for (int u = 0; u < SCAN_PER_THREAD; ++u) {
    v[u] = (base + u < nb) ? btotal[base + u] : 0;
    sum += v[u];
  }
  int total;
  int ex = block_exclusive_scan(sum, sh, total);
  __syncthreads();
#pragma unroll
  for (int u = 0; u < SCAN_PER_THREAD; ++u) {
    if (base + u < nb) btotal[base + u] = ex;
    ex += v[u];
  }
  if (threadIdx.x == 0) btotal[nb] = total;
}

// One warp per row: sort the row's ids ascending (bitonic, in shared memory)
// and write them at the row's offset of the dense list.  Rows longer than
// GATHER_SMEM_IDS are sorted in place in global memory by the same network.
constexpr int GATHER_WARPS = 8;
constexpr int GATHER_SMEM_IDS = 1024;

// Bitonic sort of 32*E ints held by one warp, element u = lane*E + r in
// v[r]: exchanges at distance >= E between lanes (shuffles), below E inside
// a lane.  Ascending.
template <int E>
__device__ __forceinline__ void warp_bitonic_sort(int (&v)[E], int lane) {
  constexpr int P2 = 32 * E;
#pragma unroll
  for (int k = 2; k <= P2; k <<= 1) {
#pragma unroll
    for (int jd = k >> 1; jd > 0; jd >>= 1) {
      if (jd >= E) {
#pragma unroll
        for (int r = 0; r < E; ++r) {
          const int u = lane * E + r;
          const int other = __shfl_xor_sync(0xffffffffu, v[r], jd / E);
          const bool keep_min = ((u & jd) == 0) == ((u & k) == 0);
          v[r] = keep_min ? min(v[r], other) : max(v[r], other);
        }
      } else {
#pragma unroll
        for (int r = 0; r < E; ++r) {
          const int p = r ^ jd;
          if (p > r) {
            const int u = lane * E + r;
            const bool up = (u & k) == 0;
            const int x = v[r], y = v[p];
            if ((x > y) == up) {
              v[r] = y;
              v[p] = x;
            }
          }
        }
      }
    }
  }
}

template <int E>
__device__ __forceinline__ void gather_row_regs(const int *__restrict__ row, int n, int lane,
                                                int *__restrict__ out) {
  int v[E];
#pragma unroll
  for (int r = 0; r < E; ++r) {
    const int u = lane * E + r;
    v[r] = (u < n) ? row[u] : INT_MAX;
  }
  warp_bitonic_sort<E>(v, lane);
#pragma unroll
  for (int r = 0; r < E; ++r) {
    const int u = lane * E + r;
    if (u < n) out[u] = v[r];
  }
}

// Bucket sort of a row of 33..256 distinct ids by one warp: 32 buckets
// spanning [min, max] of the row, filled through shared-memory counters; each
// id's place is then its bucket's start plus the number of smaller ids in the
// bucket.  The ids are distinct, so the result does not depend on the order
// in which the counters hand out bucket slots.  Returns false, with nothing
// written, when a bucket holds more than GATHER_BUCKET_MAX ids (ids clustered
// in index): the caller then uses the sorting network.
constexpr int GATHER_BUCKET_MAX = 24;
__device__ __forceinline__ bool gather_row_buckets(const int *__restrict__ row, int n, int lane,
                                                   int *__restrict__ sb, int *__restrict__ start,
                                                   int *__restrict__ out) {
  int v[8], b[8], pos[8];
  int lo = INT_MAX, hi = INT_MIN;
#pragma unroll
  for (int r = 0; r < 8; ++r) {
    const int u = r * 32 + lane;
    v[r] = (u < n) ? row[u] : 0;
    if (u < n) {
      lo = min(lo, v[r]);
      hi = max(hi, v[r]);
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  // bucket = floor((v - lo) * 32 / (hi - lo + 1)), in FP32: a non-decreasing
  // function of v, which is all the bucket order needs
  const float scale = 32.0f / ((float)hi - (float)lo + 1.0f);
  start[lane] = 0;
  __syncwarp();
#pragma unroll
  for (int r = 0; r < 8; ++r) {
    const int u = r * 32 + lane;
    b[r] = min(31, max(0, (int)((float)(v[r] - lo) * scale)));
    if (u < n) pos[r] = atomicAdd(&start[b[r]], 1);
  }
  __syncwarp();
  const int c = start[lane];
  if (__any_sync(0xffffffffu, c > GATHER_BUCKET_MAX)) return false;
  int ex = c;   // inclusive scan of the bucket sizes
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, ex, o);
    if (lane >= o) ex += y;
  }
  start[lane] = ex - c;
  if (lane == 31) start[32] = ex;
  __syncwarp();
#pragma unroll
  for (int r = 0; r < 8; ++r) {
    const int u = r * 32 + lane;
    if (u < n) sb[start[b[r]] + pos[r]] = v[r];
  }
  __syncwarp();
#pragma unroll
  for (int r = 0; r < 8; ++r) {
    if (r * 32 >= n) break;
    const int u = r * 32 + lane;
    if (u < n) {
      const int s0 = start[b[r]], s1 = start[b[r] + 1];
      int rank = s0;
      for (int k = s0; k < s1; ++k) rank += sb[k] < v[r];
      out[rank] = v[r];
    }
  }
  return true;
}

// Row i (its accepted neighbours, appended in any order by the pair kernel)
// -> ascending, into the compacted list at off[i] + boff[i / SCAN_ITEMS].
// Rows of up to 32 ids are sorted in registers, up to 256 by buckets (or in
// registers when their ids cluster), up to GATHER_SMEM_IDS in shared memory,
// longer ones in place (odd-even transposition).
__global__ void __launch_bounds__(32 * GATHER_WARPS) list_gather_kernel(
    int *__restrict__ rows, int cap, const int *__restrict__ len, const int *__restrict__ off,
    const int *__restrict__ boff, int ni, int *__restrict__ dense) {
  __shared__ int buf[GATHER_WARPS][GATHER_SMEM_IDS];
  __shared__ int bcnt[GATHER_WARPS][33];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int i = blockIdx.x * GATHER_WARPS + warp;
  if (i >= ni) return;
  const int n = len[i];
  if (n == 0) return;
  int *row = rows + (size_t)i * cap;
  const int o = off[i] + boff[i / SCAN_ITEMS];
  if (n <= 32) { gather_row_regs<1>(row, n, lane, dense + o); return; }
  if (n <= 256 && gather_row_buckets(row, n, lane, buf[warp], bcnt[warp], dense + o)) return;
  if (n <= 64) { gather_row_regs<2>(row, n, lane, dense + o); return; }
  if (n <= 128) { gather_row_regs<4>(row, n, lane, dense + o); return; }
  if (n <= 256) { gather_row_regs<8>(row, n, lane, dense + o); return; }
  const bool in_smem = n <= GATHER_SMEM_IDS;
  int *a = in_smem ? buf[warp] : row;
  int p2 = 1;
  while (p2 < n) p2 <<= 1;
  if (in_smem) {
    for (int u = lane; u < p2; u += 32) a[u] = (u < n) ? row[u] : INT_MAX;
  }
  __syncwarp();
  if (!in_smem) p2 = n;  // global fallback: odd-even transposition below
  if (in_smem) {
    for (int k = 2; k <= p2; k <<= 1) {
      for (int jd = k >> 1; jd > 0; jd >>= 1) {
        for (int u = lane; u < p2; u += 32) {
          const int l = u ^ jd;
          if (l > u) {
            const int x = a[u], y = a[l];
            const bool up = (u & k) == 0;
            if ((x > y) == up) { a[u] = y; a[l] = x; }
          }
        }
        __syncwarp();
      }
    }
  } else {
    for (int phase = 0; phase < n; ++phase) {
      for (int u = 2 * lane + (phase & 1); u + 1 < n; u += 64) {
        const int x = a[u], y = a[u + 1];
        if (x > y) { a[u] = y; a[u + 1] = x; }
      }
      __syncwarp();
    }
  }
  for (int u = lane; u < n; u += 32) dense[o + u] = a[u];
}

// ---------------------------------------------------------------------------
// host launchers
// Finalise the list offsets for the device-resident API: off[i] += block
// offset, off[ni] = grand total.
__global__ void list_finalize_offsets_kernel(int *off, const int *btot, int ni, int nb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < ni) off[i] += btot[i / SCAN_ITEMS];
  if (i == 0) off[ni] = btot[nb];
}

// ipt, warps along i, warps along j, j per load, minimum resident blocks per
// SM (the register cap, 65536 / (threads x blocks) per thread, set to what
// each shape reaches unconstrained: a tighter cap, e.g. 80 registers for six
// blocks of variant 4, spills and measured slower)
#ifndef GPUNB_V6_MINB
#define GPUNB_V6_MINB 4
#endif
static const VariantDesc kVariants[] = {{2, 4, 1, 2, 3}, {2, 2, 2, 2, 3}, {1, 1, 8, 2, 2},
                                        {1, 4, 1, 2, 5}, {1, 4, 1, 4, 5}, {1, 8, 1, 2, 2},
                                        {1, 4, 1, 8, GPUNB_V6_MINB}};
constexpr int kNumVariants = (int)(sizeof(kVariants) / sizeof(kVariants[0]));

int regf_num_variants() { return kNumVariants; }
VariantDesc regf_variant(int v) { return kVariants[v]; }

size_t regf_ds_smem(int v) {
  const VariantDesc d = kVariants[v];
  return (size_t)NSTAGE * TILE_BYTES + 2u * NQ * d.ipt * d.threads() * sizeof(float) +
         (size_t)NBUF * d.ipt * d.threads() * sizeof(int);
}

typedef void (*regf_fn)(JSet, ISet, RegfOut, RegfWork);
static regf_fn regf_kernel_ptr(int v, bool mflag) {
#define GPUNB_RK(a, b, c, d, e) \
  (mflag ? regf_ds_kernel<a, b, c, d, true, e> : regf_ds_kernel<a, b, c, d, false, e>)
  switch (v) {
    case 0: return GPUNB_RK(2, 4, 1, 2, 3);
    case 1: return GPUNB_RK(2, 2, 2, 2, 3);
    case 2: return GPUNB_RK(1, 1, 8, 2, 2);
    case 3: return GPUNB_RK(1, 4, 1, 2, 5);
    case 4: return GPUNB_RK(1, 4, 1, 4, 5);
    case 5: return GPUNB_RK(1, 8, 1, 2, 2);
    default: return GPUNB_RK(1, 4, 1, 8, GPUNB_V6_MINB);
  }
#undef GPUNB_RK
}

// Dynamic shared memory above 48 KB needs the kernel's opt-in attribute,
// both to launch and for the occupancy calculator: queried without it, the
// calculator reports no resident block at all.
static cudaError_t allow_smem(regf_fn fn, size_t smem) {
  if (smem <= 48 * 1024) return cudaSuccess;
  return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

int regf_ds_blocks_per_sm(int v, bool mflag) {
  int n = 0;
  regf_fn fn = regf_kernel_ptr(v, mflag);
  if (allow_smem(fn, regf_ds_smem(v)) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, kVariants[v].threads(),
                                                    regf_ds_smem(v)) != cudaSuccess) {
    cudaGetLastError();
    return 1;
  }
  return n > 0 ? n : 1;
}

cudaError_t launch_pack_jtiles(const double *m, const double *x, const double *v, int nj, const int *perm,
                               float *tiles, int ntile, int *err, cudaStream_t st) {
  if (ntile <= 0) return cudaSuccess;
  pack_jtiles_kernel<<<ntile, JT, 0, st>>>(m, x, v, nj, perm, tiles, err);
  return cudaGetLastError();
}

cudaError_t launch_regf_ds(int v, bool mflag, int n_itiles, int S, int grid, int *queue,
                           const JSet &js, const ISet &is, const RegfOut &out, cudaStream_t st,
                           const ItemDesc *items, const int *order, int n_items) {
  const VariantDesc d = kVariants[v];
  regf_fn fn = regf_kernel_ptr(v, mflag);
  const size_t smem = regf_ds_smem(v);
  {
    const cudaError_t e = allow_smem(fn, smem);
    if (e != cudaSuccess) return e;
  }
  // the item counter, and with the merge in the kernel the per-i-tile counts
  // that follow it
  if (out.done && (items || out.done != queue + 1)) return cudaErrorInvalidValue;
  cudaError_t e =
      cudaMemsetAsync(queue, 0, (out.done ? 1 + (size_t)n_itiles : 1) * sizeof(int), st);
  if (e != cudaSuccess) return e;
  RegfWork w;
  w.queue = queue;
  w.n_itiles = n_itiles;
  w.S = S;
  w.items = items;
  w.order = order;
  w.n_items = n_items;
  fn<<<grid, d.threads(), smem, st>>>(js, is, out, w);
  return cudaGetLastError();
}

cudaError_t launch_regf_fp64(bool mflag, int gx, int S, const JSet &js, const ISet &is,
                             const RegfOut &out, cudaStream_t st) {
  if (mflag)
    regf_fp64_kernel<true><<<dim3(gx, S), FP64_THREADS, 0, st>>>(js, is, out);
  else
    regf_fp64_kernel<false><<<dim3(gx, S), FP64_THREADS, 0, st>>>(js, is, out);
  return cudaGetLastError();
}

cudaError_t launch_regf_df(bool mflag, int gx, int S, const JSet &js, const ISet &is,
                           const RegfOut &out, cudaStream_t st) {
  if (mflag)
    regf_df_kernel<true><<<dim3(gx, S), FP64_THREADS, 0, st>>>(js, is, out);
  else
    regf_df_kernel<false><<<dim3(gx, S), FP64_THREADS, 0, st>>>(js, is, out);
  return cudaGetLastError();
}

cudaError_t launch_regf_merge(const double *part, bool ff, int S, int ni, int ni_pad,
                              const int *perm, const int *cnt, int nnbmax, double *acc,
                              double *jrk, double *pot, int *nnb, int *rowlen, cudaStream_t st) {
  // many splits of a small block: a block per i-slot (threads over splits);
  // otherwise a thread per i-slot, whose reads are coalesced across the warp
  if (S >= 32 && ni < 8192) {
    if (ff)
      regf_merge_wide_kernel<true><<<ni, MERGE_THREADS, 0, st>>>(part, S, ni, ni_pad, perm, cnt,
                                                                 nnbmax, acc, jrk, pot, nnb,
                                                                 rowlen);
    else
      regf_merge_wide_kernel<false><<<ni, MERGE_THREADS, 0, st>>>(part, S, ni, ni_pad, perm, cnt,
                                                                  nnbmax, acc, jrk, pot, nnb,
                                                                  rowlen);
  } else {
    const int nb = (ni + 31) / 32;
    if (ff)
      regf_merge_kernel<true><<<nb, 32 * MERGE_KW, 0, st>>>(part, S, ni, ni_pad, perm, cnt,
                                                            nnbmax, acc, jrk, pot, nnb, rowlen);
    else
      regf_merge_kernel<false><<<nb, 32 * MERGE_KW, 0, st>>>(part, S, ni, ni_pad, perm, cnt,
                                                             nnbmax, acc, jrk, pot, nnb, rowlen);
  }
  return cudaGetLastError();
}

cudaError_t launch_regf_merge_batch(const double *part, const int4 *tiles, int ntiles, int itile,
                                    const int *perm, const int *cnt, int nnbmax, double *acc,
                                    double *jrk, double *pot, int *nnb, int *rowlen,
                                    cudaStream_t st) {
  if (ntiles <= 0) return cudaSuccess;
  regf_merge_batch_kernel<<<ntiles, 128, 0, st>>>(part, tiles, itile, perm, cnt, nnbmax, acc,
                                                  jrk, pot, nnb, rowlen);
  return cudaGetLastError();
}

cudaError_t launch_regf_prep(const ISet &is, float4 *rec, int *err, cudaStream_t st) {
  if (is.ni <= 0) return cudaSuccess;
  regf_prep_kernel<<<(is.ni + 127) / 128, 128, 0, st>>>(is, rec, err);
  return cudaGetLastError();
}

int list_scan_blocks(int ni) { return (ni + SCAN_ITEMS - 1) / SCAN_ITEMS; }

cudaError_t launch_list_scan(const int *rowlen, int ni, int *off, int *btot, cudaStream_t st) {
  const int nb = list_scan_blocks(ni);
  list_scan_blocks_kernel<<<nb, SCAN_THREADS, 0, st>>>(rowlen, ni, off, btot);
  list_scan_totals_kernel<<<1, SCAN_THREADS, 0, st>>>(btot, nb);
  return cudaGetLastError();
}

cudaError_t launch_list_gather(int *rows, int cap, const int *rowlen, const int *off,
                               const int *btot, int ni, int *dense, cudaStream_t st) {
  list_gather_kernel<<<(ni + GATHER_WARPS - 1) / GATHER_WARPS, 32 * GATHER_WARPS, 0, st>>>(
      rows, cap, rowlen, off, btot, ni, dense);
  return cudaGetLastError();
}

// Host-visible rows (the gpunb_regf_ LISTGP layout) written by the device:
// one warp per row, row[0] = the signed count, row[1..count] = the ids of the
// compacted list (row i starts at off[i] + boff[i / SCAN_ITEMS], the scan's
// in-block offset plus its block's base).  `rows` is the caller's host array, reached through the
// coherent host-memory path (the caller checks that the device may access
// pageable memory through the host's page tables before using this).
__global__ void list_rows_kernel(const int *__restrict__ dense, const int *__restrict__ off,
                                 const int *__restrict__ boff, const int *__restrict__ nnb, int ni,
                                 int lmax, int *__restrict__ rows) {
  const int lane = threadIdx.x & 31;
  const int i = (int)(((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  if (i >= ni) return;
  const int c = nnb[i];
  int *row = rows + (size_t)i * lmax;
  if (lane == 0) row[0] = c;
  if (c > 0) {
    const int *src = dense + off[i] + boff[i / SCAN_ITEMS];
    for (int u = lane; u < c; u += 32) row[1 + u] = src[u];
  }
}

cudaError_t launch_list_rows(const int *dense, const int *off, const int *boff, const int *nnb,
                             int ni, int lmax, int *rows, cudaStream_t st) {
  if (ni <= 0) return cudaSuccess;
  const int threads = 256;
  const long long blocks = ((long long)ni * 32 + threads - 1) / threads;
  list_rows_kernel<<<(unsigned)blocks, threads, 0, st>>>(dense, off, boff, nnb, ni, lmax, rows);
  return cudaGetLastError();
}

// Copies between the caller's host arrays and device buffers done by the
// device itself over the coherent host path (one launch for up to
// HOSTCOPY_MAX arrays instead of one pageable cudaMemcpy each, whose fixed
// cost is ~11 us); 8-byte or 4-byte elements, coalesced across the warp.
__global__ void host_copy_kernel(HostCopyJobs jobs) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  const long long t0 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  for (int q = 0; q < jobs.count; ++q) {
    const HostCopyJob J = jobs.j[q];
    if (J.esize == 8) {
      const double *src = (const double *)J.src;
      double *dst = (double *)J.dst;
      for (long long e = t0; e < J.n; e += stride) dst[e] = src[e];
    } else {
      const int *src = (const int *)J.src;
      int *dst = (int *)J.dst;
      for (long long e = t0; e < J.n; e += stride) dst[e] = src[e];
    }
  }
}

cudaError_t launch_host_copy(const HostCopyJobs &jobs, cudaStream_t st) {
  long long tot = 0;
  for (int q = 0; q < jobs.count; ++q) tot += jobs.j[q].n;
  if (tot <= 0) return cudaSuccess;
  const long long blocks = std::min<long long>((tot + 255) / 256, 2048);
  host_copy_kernel<<<(unsigned)blocks, 256, 0, st>>>(jobs);
  return cudaGetLastError();
}

cudaError_t launch_list_finalize_offsets(int *off, const int *btot, int ni, cudaStream_t st) {
  list_finalize_offsets_kernel<<<(ni + 255) / 256, 256, 0, st>>>(off, btot, ni,
                                                                 list_scan_blocks(ni));
  return cudaGetLastError();
}

}  // namespace gpunb
