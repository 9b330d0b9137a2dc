// Device-side building blocks shared by the regular-force and potential
// kernels: packed FP32 pairs, double-single splitting, compensated sums,
// bulk-async (TMA) copies with bounded mbarrier waits, and the error word.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "gpunb.h"  // error codes

namespace gpunb {

// ---------------------------------------------------------------------------
// Packed FP32 pairs: one sm_100-family f32x2 instruction does two FP32 ops.
// The two halves always hold two different j for the same i.
typedef float2 f2;

__device__ __forceinline__ f2 mk2(float a) { return make_float2(a, a); }
__device__ __forceinline__ f2 add2(f2 a, f2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ f2 mul2(f2 a, f2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ f2 fma2(f2 a, f2 b, f2 c) { return __ffma2_rn(a, b, c); }

// Hardware reciprocal square root estimate (about 2^-22 relative error; the
// pair loops refine it with one Newton step).  The .ftz form is the bare
// estimate instruction: inputs below 2^-126 (distances below 1e-19) read as
// zero and give +inf, exactly like coincident bodies.
__device__ __forceinline__ float rsqrt_est(float x) {
  float y;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// ---------------------------------------------------------------------------
// Double-single: x = hi + lo with hi = fl32(x), lo = fl32(x - hi).
// Round-to-nearest split (valid for any |x| in float range), unlike the
// truncating fixed-point split of the reference potential code.
__host__ __device__ __forceinline__ void ds_split(double x, float &hi, float &lo) {
  hi = (float)x;
  lo = (float)(x - (double)hi);
}

// Error-free sum of two floats (Knuth TwoSum, 6 flops, no ordering needed).
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
  s = __fadd_rn(a, b);
  const float bb = __fadd_rn(s, -a);
  const float aa = __fadd_rn(s, -bb);
  e = __fadd_rn(__fadd_rn(a, -aa), __fadd_rn(b, -bb));
}

// Fold an FP32 chunk sum c into a float-float accumulator (hi, lo).
__device__ __forceinline__ void ff_accum(float &hi, float &lo, float c) {
  float s, e;
  two_sum(hi, c, s, e);
  hi = s;
  lo = __fadd_rn(lo, e);
}

// float-float + float-float (used for fixed-order intra-CTA merges).
__device__ __forceinline__ void ff_add(float &hi, float &lo, float bhi, float blo) {
  float s, e;
  two_sum(hi, bhi, s, e);
  e = __fadd_rn(e, __fadd_rn(lo, blo));
  float s2, e2;
  two_sum(s, e, s2, e2);
  hi = s2;
  lo = e2;
}

// ---------------------------------------------------------------------------
// Double-float arithmetic: a value is the unevaluated sum hi + lo of two
// floats (about 48 significant bits); each operation is an error-free
// transform (Knuth's TwoSum, the FMA product error) followed by
// renormalisation -- the double-single arithmetic of Dekker (1971).  On a
// part whose FP64 pipe runs at 1/64 of the FP32 rate it gives FP64-class
// results several times faster than FP64 itself.
struct dfl {
  float h, l;
};
__device__ __forceinline__ dfl df_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}
__device__ __forceinline__ dfl df_fast(float a, float b) {   // |a| >= |b| or a == 0
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ dfl df_add(dfl a, dfl b) {
  const dfl s = df_two_sum(a.h, b.h);
  return df_fast(s.h, __fadd_rn(s.l, __fadd_rn(a.l, b.l)));
}
__device__ __forceinline__ dfl df_mul(dfl a, dfl b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = fmaf(a.h, b.h, -p);
  e = fmaf(a.h, b.l, e);
  e = fmaf(a.l, b.h, e);
  return df_fast(p, e);
}
__device__ __forceinline__ dfl df_mulf(dfl a, float b) {
  const float p = __fmul_rn(a.h, b);
  return df_fast(p, fmaf(a.l, b, fmaf(a.h, b, -p)));
}
__device__ __forceinline__ dfl df_sqr(dfl a) {
  const float p = __fmul_rn(a.h, a.h);
  return df_fast(p, fmaf(__fmul_rn(2.0f, a.h), a.l, fmaf(a.h, a.h, -p)));
}
// difference of two double-single values b - a
__device__ __forceinline__ dfl df_diff(float bh, float bl, float ah, float al) {
  const dfl s = df_two_sum(bh, -ah);
  return df_fast(s.h, __fadd_rn(s.l, __fsub_rn(bl, al)));
}

// ---------------------------------------------------------------------------
// Bulk-async global->shared copies completing on an mbarrier (TMA engine).
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

// 1-D bulk copy: both addresses 16-byte aligned, size a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void *dst_smem, const void *src_gmem, uint32_t bytes,
                                         uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cta.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst_smem)),
      "l"(src_gmem), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, "
      "1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait: gives up after `limit` polls (each try_wait itself suspends
// for a hardware-defined time slice) and reports false.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity,
                                                  uint32_t limit = (1u << 22)) {
  for (uint32_t it = 0; it < limit; ++it)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// ---------------------------------------------------------------------------
// Global error word: first error wins; the host reads it after each call.
__device__ __forceinline__ void raise_error(int *err, int code) {
  if (err) atomicCAS(err, 0, code);
}

}  // namespace gpunb
