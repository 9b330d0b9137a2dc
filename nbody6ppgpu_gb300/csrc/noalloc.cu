// gpupot_device_noalloc: the potential of gpupot_ for callers that cannot
// allocate device memory.
//
// Some callers of this library must not call cudaMalloc: an integrator that
// checks the energy from inside a CUDA-graph-captured step (allocation is not
// allowed while a stream is being captured), and host programs that have
// handed all free device memory to their own caching allocator before the
// library is first used (cudaMalloc then fails, and cudaFree would also
// synchronise the whole device in the middle of their step).  This entry point
// therefore uses a fixed scratch area that is part of the library image: a
// file-scope device array of NOALLOC_SCRATCH_BYTES (4 MiB), present on every
// GPU that loads the library until the process exits.  It calls no
// cudaMalloc, cudaFree or other allocating routine.
//
// Limits: n <= NOALLOC_MAX_N bodies (65536); 1 <= istart, istart-1+ni <= n.
// The caller passes device pointers for m[n], x[n][3] and pot[ni] and a stream.
//
// The scratch is shared by all calls and keeps the last call's contents; the
// parts that must start at zero are cleared at the start of every call.  Calls
// that overlap on the GPU (on different streams, or from different threads)
// race on the scratch: serialise them on one stream.
#include <algorithm>
#include <cstdio>
#include <mutex>

#include "common.cuh"
#include "launch.h"

namespace gpunb {

constexpr int NOALLOC_MAX_N = 65536;
constexpr size_t NOALLOC_ERR_BYTES = 256;
constexpr size_t NOALLOC_TILE_BYTES =
    (size_t)((NOALLOC_MAX_N + POT_JT - 1) / POT_JT) * POT_TILE_FLOATS * sizeof(float);
constexpr size_t NOALLOC_PART_DOUBLES = (size_t)1 << 18;
constexpr size_t NOALLOC_SCRATCH_BYTES =
    NOALLOC_ERR_BYTES + NOALLOC_TILE_BYTES + NOALLOC_PART_DOUBLES * sizeof(double);
static_assert(NOALLOC_TILE_BYTES % 256 == 0, "keep the partials 256-byte aligned");
static_assert(NOALLOC_SCRATCH_BYTES <= ((size_t)4 << 20), "scratch stays within 4 MiB");

static __device__ __align__(256) unsigned char noalloc_scratch[NOALLOC_SCRATCH_BYTES];

// Device address of the scratch, looked up once per device with that device
// current (in host code the array's name is only a host-side stand-in).
static constexpr int kMaxDevices = 64;
static unsigned char *g_scratch_ptr[kMaxDevices] = {nullptr};
static std::mutex g_scratch_mutex;

static int scratch_for_current_device(unsigned char **ptr) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return GPUNB_E_NO_DEVICE;
  }
  std::lock_guard<std::mutex> lk(g_scratch_mutex);
  if (!g_scratch_ptr[dev]) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, noalloc_scratch);
    if (e != cudaSuccess || p == nullptr) {
      cudaGetLastError();
      fprintf(stderr, "gpupot_device_noalloc: cudaGetSymbolAddress failed: %s\n",
              cudaGetErrorString(e));
      return GPUNB_E_CUDA;
    }
    g_scratch_ptr[dev] = (unsigned char *)p;
  }
  *ptr = g_scratch_ptr[dev];
  return GPUNB_OK;
}

}  // namespace gpunb

using namespace gpunb;

extern "C" int gpupot_device_noalloc(int istart, int ni, int n, const double *m, const double *x,
                                     double *pot, void *stream) {
  if (n < 1 || n > NOALLOC_MAX_N || ni < 1 || istart < 1 || istart - 1 + ni > n || !m || !x ||
      !pot) {
    fprintf(stderr,
            "gpupot_device_noalloc: need 1 <= n <= %d, 1 <= istart, istart-1+ni <= n and "
            "non-null pointers (istart %d ni %d n %d)\n",
            NOALLOC_MAX_N, istart, ni, n);
    return GPUNB_E_ARG;
  }
  unsigned char *base = nullptr;
  const int rc = scratch_for_current_device(&base);
  if (rc != GPUNB_OK) return rc;
  int *err = (int *)base;
  float *tiles = (float *)(base + NOALLOC_ERR_BYTES);
  double *part = (double *)(base + NOALLOC_ERR_BYTES + NOALLOC_TILE_BYTES);

  int dev = 0, n_sm = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
  const int ntile = (n + POT_JT - 1) / POT_JT;
  const int itile = pot_itile();
  const int gx = (ni + itile - 1) / itile;
  const int ni_pad = gx * itile;
  long long S = (2ll * n_sm * pot_blocks_per_sm() + gx - 1) / gx;
  S = std::min<long long>(S, std::max(1, ntile / 2));
  S = std::min<long long>(S, (long long)(NOALLOC_PART_DOUBLES / (size_t)ni_pad));
  if (S < 1) S = 1;

  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e = cudaMemsetAsync(err, 0, sizeof(int), st);
  if (e == cudaSuccess) e = launch_pack_pot(m, x, n, tiles, ntile, err, st);
  if (e == cudaSuccess)
    e = launch_pot(tiles, ntile, x, istart - 1, ni, gx, (int)S, part, ni_pad, err, st);
  if (e == cudaSuccess) e = launch_pot_merge(part, (int)S, ni, ni_pad, pot, st);
  if (e != cudaSuccess) {
    fprintf(stderr, "gpupot_device_noalloc: launch failed: %s\n", cudaGetErrorString(e));
    return GPUNB_E_CUDA;
  }
  return GPUNB_OK;
}
