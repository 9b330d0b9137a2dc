// gpupot_device_noalloc: the potential of gpupot_ for callers that cannot
// allocate device memory.
//
// Some callers of this library cannot call cudaMalloc.  A host program that
// has handed all free device memory to its own caching allocator before the
// library is first used (a PyTorch- or pool-managed integrator) gets an
// out-of-memory error from cudaMalloc; a step loop that must not stall the
// device cannot afford cudaFree, which synchronises the whole device.  This
// entry point therefore uses a fixed scratch area that is part of the
// library image: a file-scope device array of NOALLOC_SCRATCH_BYTES (4 MiB),
// present on every GPU that loads the library until the process exits.  It
// calls no cudaMalloc, cudaFree or other allocating routine.
//
// Limits: n <= NOALLOC_MAX_N bodies (65536); 1 <= istart, istart-1+ni <= n.
// The caller passes device pointers for m[n], x[n][3] and pot[ni] and a stream.
//
// The call waits for its own work on that stream and returns the error word
// that its kernels wrote into the scratch: a NaN input gives GPUNB_E_NAN, a
// bounded wait that gave up GPUNB_E_TIMEOUT.  Whenever that word is set the
// potentials are all NaN, so partial sums left in the scratch by an earlier
// call can never pass for this call's results.
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

// Per device, filled on the first call with that device current: the
// scratch's device address (in host code the array's name is only a
// host-side stand-in) and the launch figures of the potential kernel.
struct NoallocDevice {
  unsigned char *scratch = nullptr;
  int n_sm = 0;
  int blocks_per_sm = 0;
};
static constexpr int kMaxDevices = 64;
static NoallocDevice g_noalloc_dev[kMaxDevices];
static std::mutex g_scratch_mutex;

static int noalloc_device(NoallocDevice *out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return GPUNB_E_NO_DEVICE;
  }
  std::lock_guard<std::mutex> lk(g_scratch_mutex);
  NoallocDevice &d = g_noalloc_dev[dev];
  if (!d.scratch) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, noalloc_scratch);
    if (e != cudaSuccess || p == nullptr) {
      cudaGetLastError();
      fprintf(stderr, "gpupot_device_noalloc: cudaGetSymbolAddress failed: %s\n",
              cudaGetErrorString(e));
      return GPUNB_E_CUDA;
    }
    int n_sm = 0;
    if (cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        n_sm < 1) {
      cudaGetLastError();
      return GPUNB_E_CUDA;
    }
    d.n_sm = n_sm;
    d.blocks_per_sm = pot_blocks_per_sm();
    d.scratch = (unsigned char *)p;
  }
  *out = d;
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
  NoallocDevice dev;
  const int rc = noalloc_device(&dev);
  if (rc != GPUNB_OK) return rc;
  unsigned char *base = dev.scratch;
  int *err = (int *)base;
  float *tiles = (float *)(base + NOALLOC_ERR_BYTES);
  double *part = (double *)(base + NOALLOC_ERR_BYTES + NOALLOC_TILE_BYTES);

  const int ntile = (n + POT_JT - 1) / POT_JT;
  const int itile = pot_itile();
  const int gx = (ni + itile - 1) / itile;
  const int ni_pad = gx * itile;
  long long S = (2ll * dev.n_sm * dev.blocks_per_sm + gx - 1) / gx;
  S = std::min<long long>(S, std::max(1, ntile / 2));
  S = std::min<long long>(S, (long long)(NOALLOC_PART_DOUBLES / (size_t)ni_pad));
  if (S < 1) S = 1;

  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e = cudaMemsetAsync(err, 0, sizeof(int), st);
  if (e == cudaSuccess) e = launch_pack_pot(m, x, n, tiles, ntile, err, st);
  if (e == cudaSuccess)
    e = launch_pot(tiles, ntile, x, istart - 1, ni, gx, (int)S, part, ni_pad, err, st);
  if (e == cudaSuccess) e = launch_pot_merge(part, (int)S, ni, ni_pad, err, pot, st);
  // the kernels' error word, read once this call's work on the stream is done
  int herr = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    fprintf(stderr, "gpupot_device_noalloc: %s\n", cudaGetErrorString(e));
    cudaGetLastError();
    return GPUNB_E_CUDA;
  }
  if (herr != 0)
    fprintf(stderr, "gpupot_device_noalloc: %s (potentials set to NaN)\n",
            herr == GPUNB_E_NAN ? "NaN in an input array"
            : herr == GPUNB_E_TIMEOUT ? "a device wait timed out" : "device error");
  return herr;
}
