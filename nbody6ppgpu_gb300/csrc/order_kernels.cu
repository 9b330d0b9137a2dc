// Spatial ordering of bodies along a Morton (Z-order) curve.
//
// No reference counterpart: the reference packs j in the caller's order and
// runs i in the caller's order (gpunb.velocity.cu:716-727,757-762).  Ordering
// both sets spatially makes the neighbour-candidate branch of the pair kernel
// coherent: the i-particles of one warp are close to each other, so the j
// bodies that can be their neighbours arrive in the same few tiles and the
// warp enters the branch rarely and with many lanes active.  Results do not
// depend on the order beyond FP32 summation order; the order itself is a pure
// function of the positions (deterministic bounding box, stable radix sort).
#include <algorithm>
#include <climits>
#include <cub/device/device_radix_sort.cuh>

#include "common.cuh"
#include "launch.h"

namespace gpunb {

// order-preserving float <-> int mapping for deterministic atomic min/max
__device__ __forceinline__ int f2ord(float f) {
  const int i = __float_as_int(f);
  return i >= 0 ? i : i ^ 0x7fffffff;
}
__device__ __forceinline__ float ord2f(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff); }

// bb[0..2] = min, bb[3..5] = max of the FP32-rounded coordinates (as
// order-preserving ints).  Each block reduces its share and writes one
// partial box; the last block to finish (ticket bb[BBOX_TICKET]) reduces the
// partials and resets the ticket, so one launch does the whole reduction and
// needs no initialisation.  The ticket is zeroed when the buffer is created.
__global__ void __launch_bounds__(BBOX_THREADS) bbox_kernel(const double *__restrict__ x, int n,
                                                            int *bb) {
  __shared__ float s[BBOX_THREADS / 32][6];
  __shared__ bool last;
  float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float v = (float)x[3 * i + c];
      lo[c] = fminf(lo[c], v);
      hi[c] = fmaxf(hi[c], v);
    }
  }
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    for (int o = 16; o > 0; o >>= 1) {
      lo[c] = fminf(lo[c], __shfl_xor_sync(0xffffffffu, lo[c], o));
      hi[c] = fmaxf(hi[c], __shfl_xor_sync(0xffffffffu, hi[c], o));
    }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      s[warp][c] = lo[c];
      s[warp][3 + c] = hi[c];
    }
  }
  __syncthreads();
  if (threadIdx.x < 6) {
    const int q = threadIdx.x;
    float r = s[0][q];
    for (int w = 1; w < BBOX_THREADS / 32; ++w) r = q < 3 ? fminf(r, s[w][q]) : fmaxf(r, s[w][q]);
    bb[BBOX_PART + 6 * blockIdx.x + q] = f2ord(r);
    __threadfence();
  }
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(bb + BBOX_TICKET, 1) == (int)gridDim.x - 1;
  __syncthreads();
  if (!last) return;
  // last block: thread b reads partial b (all loads in flight at once), then
  // the same warp + shared-memory reduction (on order-preserving ints)
  __shared__ int si[BBOX_THREADS / 32][6];
  int r[6];
#pragma unroll
  for (int q = 0; q < 6; ++q) r[q] = q < 3 ? INT_MAX : INT_MIN;
  for (int b = threadIdx.x; b < (int)gridDim.x; b += BBOX_THREADS) {
#pragma unroll
    for (int q = 0; q < 6; ++q) {
      const int u = __ldcg(bb + BBOX_PART + 6 * b + q);
      r[q] = q < 3 ? min(r[q], u) : max(r[q], u);
    }
  }
#pragma unroll
  for (int q = 0; q < 6; ++q)
    for (int o = 16; o > 0; o >>= 1) {
      const int u = __shfl_xor_sync(0xffffffffu, r[q], o);
      r[q] = q < 3 ? min(r[q], u) : max(r[q], u);
    }
  if (lane == 0) {
#pragma unroll
    for (int q = 0; q < 6; ++q) si[warp][q] = r[q];
  }
  __syncthreads();
  if (threadIdx.x < 6) {
    const int q = threadIdx.x;
    int t = si[0][q];
    for (int w = 1; w < BBOX_THREADS / 32; ++w) t = q < 3 ? min(t, si[w][q]) : max(t, si[w][q]);
    bb[q] = t;
  }
  if (threadIdx.x == 0) bb[BBOX_TICKET] = 0;
}

// spread the low 16 bits of v to every third bit
__device__ __forceinline__ unsigned long long spread3(unsigned int v) {
  unsigned long long x = v & 0xffffu;
  x = (x | (x << 32)) & 0x001f00000000ffffull;
  x = (x | (x << 16)) & 0x001f0000ff0000ffull;
  x = (x | (x << 8)) & 0x100f00f00f00f00full;
  x = (x | (x << 4)) & 0x10c30c30c30c30c3ull;
  x = (x | (x << 2)) & 0x1249249249249249ull;
  return x;
}

// Morton keys: MORTON_BITS per axis inside the bounding box.  10 bits (a
// 1024^3 grid) keep a tile of 128 bodies compact even in a 2^20-body core,
// and the 30-bit key sorts in four 8-bit radix passes instead of six.
constexpr int MORTON_BITS = 10;
constexpr int KEY_BITS = 3 * MORTON_BITS;
constexpr float MORTON_MAX = (float)((1 << MORTON_BITS) - 1);

// Morton key and identity values for the sort.
__global__ void morton_kernel(const double *__restrict__ x, int n, const int *__restrict__ bb,
                              unsigned long long *__restrict__ key, int *__restrict__ val) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  unsigned int q[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const float lo = ord2f(bb[c]), hi = ord2f(bb[3 + c]);
    const float span = hi - lo;
    const float s = span > 0.f ? MORTON_MAX / span : 0.f;
    float u = ((float)x[3 * i + c] - lo) * s;
    u = fminf(fmaxf(u, 0.f), MORTON_MAX);
    q[c] = (unsigned int)u;
  }
  key[i] = spread3(q[0]) | (spread3(q[1]) << 1) | (spread3(q[2]) << 2);
  val[i] = i;
}

// owning set of element e: the c with off[c] <= e < off[c+1]
__device__ __forceinline__ int owner_of(const int *__restrict__ off, int nset, int e) {
  int lo = 0, hi = nset;   // invariant off[lo] <= e < off[hi]
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (off[mid] <= e) lo = mid;
    else hi = mid;
  }
  return lo;
}

// Batched sets: key = (set index << KEY_BITS) | Morton key, so that one stable sort
// groups the bodies by set and orders each set along the curve.
__global__ void morton_batch_kernel(const double *__restrict__ x, int n, const int *__restrict__ bb,
                                    const int *__restrict__ off, int nset,
                                    unsigned long long *__restrict__ key, int *__restrict__ val) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  unsigned int q[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const float lo = ord2f(bb[c]), hi = ord2f(bb[3 + c]);
    const float span = hi - lo;
    const float s = span > 0.f ? MORTON_MAX / span : 0.f;
    float u = ((float)x[3 * i + c] - lo) * s;
    u = fminf(fmaxf(u, 0.f), MORTON_MAX);
    q[c] = (unsigned int)u;
  }
  const unsigned long long set = (unsigned long long)owner_of(off, nset, i);
  key[i] = (set << KEY_BITS) | spread3(q[0]) | (spread3(q[1]) << 1) | (spread3(q[2]) << 2);
  val[i] = i;
}

// sorted position q (grouped by set, off[] = set boundaries) -> slot in a
// layout where set c starts at slot_off[c]; slots not written keep -1.
__global__ void scatter_slots_kernel(const int *__restrict__ sorted, int n,
                                     const int *__restrict__ off, const int *__restrict__ slot_off,
                                     int nset, int *__restrict__ perm) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const int c = owner_of(off, nset, q);
  perm[slot_off[c] + (q - off[c])] = sorted[q];
}

cudaError_t launch_order_batch(const double *x, int n, const int *bb, const int *off, int nset,
                               const int *slot_off, int nslots, unsigned long long *keys,
                               unsigned long long *keys_alt, int *vals_alt, int *sorted,
                               int *perm, void *temp, size_t temp_bytes, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(perm, 0xff, (size_t)nslots * sizeof(int), st);
  if (e != cudaSuccess || n <= 0) return e;
  morton_batch_kernel<<<(n + 255) / 256, 256, 0, st>>>(x, n, bb, off, nset, keys, vals_alt);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  int end_bit = KEY_BITS;
  while ((1ll << (end_bit - KEY_BITS)) < nset) ++end_bit;
  size_t tb = temp_bytes;
  e = cub::DeviceRadixSort::SortPairs(temp, tb, keys, keys_alt, vals_alt, sorted, n, 0, end_bit,
                                      st);
  if (e != cudaSuccess) return e;
  scatter_slots_kernel<<<(n + 255) / 256, 256, 0, st>>>(sorted, n, off, slot_off, nset, perm);
  return cudaGetLastError();
}

size_t order_batch_temp_bytes(int n, int nset) {
  int end_bit = KEY_BITS;
  while ((1ll << (end_bit - KEY_BITS)) < nset) ++end_bit;
  size_t tb = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, tb, (const unsigned long long *)nullptr,
                                  (unsigned long long *)nullptr, (const int *)nullptr,
                                  (int *)nullptr, n, 0, end_bit);
  return tb;
}

size_t order_temp_bytes(int n) {
  size_t tb = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, tb, (const unsigned long long *)nullptr,
                                  (unsigned long long *)nullptr, (const int *)nullptr,
                                  (int *)nullptr, n, 0, KEY_BITS);
  return tb;
}

cudaError_t launch_bbox(const double *x, int n, int *bb, cudaStream_t st) {
  // two bodies per thread at least; an empty set still runs one block (box
  // of +inf / -inf, as for the FP32 coordinates of no body)
  const int per_block = 2 * BBOX_THREADS;
  const int blocks = std::max(1, std::min(BBOX_MAX_BLOCKS, (std::max(n, 0) + per_block - 1) /
                                                              per_block));
  bbox_kernel<<<blocks, BBOX_THREADS, 0, st>>>(x, std::max(n, 0), bb);
  return cudaGetLastError();
}

// perm[0..n) = indices of x sorted by Morton key within bounding box bb.
cudaError_t launch_order(const double *x, int n, const int *bb, unsigned long long *keys,
                         unsigned long long *keys_alt, int *vals_alt, int *perm, void *temp,
                         size_t temp_bytes, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  morton_kernel<<<(n + 255) / 256, 256, 0, st>>>(x, n, bb, keys, vals_alt);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  size_t tb = temp_bytes;
  return cub::DeviceRadixSort::SortPairs(temp, tb, keys, keys_alt, vals_alt, perm, n, 0, KEY_BITS,
                                         st);
}

}  // namespace gpunb
