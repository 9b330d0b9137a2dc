// Host runtime of libgpunb.so: device state, buffers, launch planning,
// autotuning, CUDA-graph replay, and the C ABI of include/gpunb.h.
//
// Reference host code replaced: src/Main/gpunb.velocity.cu:555-939 (static
// state, GPUNB_devinit/open/close/send/regf/profile, extern "C" exports),
// include/cuda_pointer.h (synchronous pinned/device pairs) and
// src/Main/gpupot.gpu.cu:59-127.  Differences by design: one GPU per process,
// j-set resident in HBM in a split-precision tiled layout built on the device,
// one stream, asynchronous copies from pinned staging, device-side reductions
// and list compaction (no host prefix sum and no second upload of offsets).
#include <cerrno>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <algorithm>
#include <map>
#include <vector>
#include <mutex>
#include <string>
#include <sys/time.h>
#include <unistd.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "gpunb.h"
#include "launch.h"

namespace gpunb {

// ---------------------------------------------------------------------------
// errors
static int g_err_code = 0;
static std::string g_err_msg;
static int g_abort_on_error = 1;

static void fail(int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (g_err_code == 0) {
    g_err_code = code;
    g_err_msg = buf;
  }
  fprintf(stderr, "gpunb: error %d: %s\n", code, buf);
  if (g_abort_on_error) abort();
}

// errors raised by the other translation units of the library (irregular
// force): same record, same abort policy
void report_failure(int code, const char *msg) { fail(code, "%s", msg); }

#define CUDA_OR(call, ret)                                                          \
  do {                                                                              \
    cudaError_t e_ = (call);                                                        \
    if (e_ != cudaSuccess) {                                                        \
      fail(GPUNB_E_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_));            \
      return ret;                                                                   \
    }                                                                               \
  } while (0)

static double wtime() {
  struct timeval tv;
  gettimeofday(&tv, nullptr);
  return tv.tv_sec + 1.e-6 * tv.tv_usec;
}

// ---------------------------------------------------------------------------
// grow-only buffers
// Incremented whenever a device buffer moves: captured CUDA graphs hold raw
// addresses and are replayed only while this count is unchanged.
static unsigned long long g_alloc_gen = 0;
// gpunb_test_fail_allocs: the next n device allocations report failure
static int g_fail_allocs = 0;

struct DevBuf {
  void *p = nullptr;
  size_t bytes = 0;
  bool ensure(size_t n) {
    if (n <= bytes) return true;
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
    ++g_alloc_gen;
    size_t want = n + n / 4 + 256;
    if (g_fail_allocs > 0) {
      --g_fail_allocs;
      fail(GPUNB_E_ALLOC, "cudaMalloc of %zu bytes failed (test hook)", want);
      return false;
    }
    if (cudaMalloc(&p, want) != cudaSuccess) {
      cudaGetLastError();
      fail(GPUNB_E_ALLOC, "cudaMalloc of %zu bytes failed", want);
      return false;
    }
    bytes = want;
    return true;
  }
  // as ensure, and a newly created buffer is zero-filled
  bool ensure_zero(size_t n) {
    if (n <= bytes) return true;
    if (!ensure(n)) return false;
    if (cudaMemset(p, 0, bytes) != cudaSuccess) {
      cudaGetLastError();
      fail(GPUNB_E_CUDA, "cudaMemset of %zu bytes failed", bytes);
      return false;
    }
    return true;
  }
  void release() {
    if (p) {
      cudaFree(p);
      ++g_alloc_gen;
    }
    p = nullptr;
    bytes = 0;
  }
  template <class T> T *as() const { return (T *)p; }
};

// A captured CUDA graph of one call shape.  The first call of a shape runs
// eagerly (allocating what it needs), then the same launch sequence is
// captured; later calls of that shape replay it while no buffer has moved.
struct GraphEntry {
  cudaGraphExec_t exec = nullptr;
  unsigned long long gen = 0;
};

static void graph_drop(GraphEntry &e) {
  if (e.exec) cudaGraphExecDestroy(e.exec);
  e.exec = nullptr;
}

// issue(st) queues the device work of one call and returns an error code;
// it must not touch host memory that changes between calls.
template <class F>
static int run_graphed(GraphEntry &e, bool enabled, cudaStream_t st, F issue) {
  if (enabled && e.exec && e.gen == g_alloc_gen) {
    CUDA_OR(cudaGraphLaunch(e.exec, st), GPUNB_E_CUDA);
    return GPUNB_OK;
  }
  int rc = issue(st);
  if (rc != GPUNB_OK || !enabled) return rc;
  graph_drop(e);
  const unsigned long long gen0 = g_alloc_gen;
  CUDA_OR(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), GPUNB_E_CUDA);
  rc = issue(st);
  cudaGraph_t graph = nullptr;
  const cudaError_t ec = cudaStreamEndCapture(st, &graph);
  if (rc == GPUNB_OK && ec == cudaSuccess && graph && gen0 == g_alloc_gen) {
    if (cudaGraphInstantiate(&e.exec, graph, 0) != cudaSuccess) {
      cudaGetLastError();
      e.exec = nullptr;
    }
    e.gen = g_alloc_gen;
  } else {
    cudaGetLastError();
  }
  if (graph) cudaGraphDestroy(graph);
  return rc;
}

// CUDA-graph replay (gpunb_set_graphs): the batched entry points keep one
// graph per plan; the single-set device entry points keep one per call key
// (sizes, caller pointers, stream and launch plan), at most kMaxDevGraphs.
static bool g_use_graphs = false;
static std::map<std::vector<long long>, GraphEntry> g_dev_graphs;
constexpr size_t kMaxDevGraphs = 64;

static void dev_graphs_drop() {
  for (auto &kv : g_dev_graphs) graph_drop(kv.second);
  g_dev_graphs.clear();
}

static GraphEntry &dev_graph(const std::vector<long long> &key) {
  if (g_dev_graphs.size() >= kMaxDevGraphs && g_dev_graphs.find(key) == g_dev_graphs.end())
    dev_graphs_drop();
  return g_dev_graphs[key];
}

struct PinBuf {
  void *p = nullptr;
  size_t bytes = 0;
  bool ensure(size_t n) {
    if (n <= bytes) return true;
    if (p) cudaFreeHost(p);
    p = nullptr;
    bytes = 0;
    ++g_alloc_gen;   // pinned buffers appear in captured graphs too
    size_t want = n + n / 4 + 256;
    if (cudaMallocHost(&p, want) != cudaSuccess) {
      cudaGetLastError();
      fail(GPUNB_E_ALLOC, "cudaMallocHost of %zu bytes failed", want);
      return false;
    }
    bytes = want;
    return true;
  }
  void release() {
    if (p) {
      cudaFreeHost(p);
      ++g_alloc_gen;
    }
    p = nullptr;
    bytes = 0;
  }
  template <class T> T *as() const { return (T *)p; }
};

// parallel host copy for large staging transfers
static void hcopy(void *dst, const void *src, size_t bytes) {
#ifdef _OPENMP
  if (bytes >= (4u << 20)) {
    const int nt = omp_get_max_threads();
    const size_t chunk = (bytes + nt - 1) / nt;
#pragma omp parallel for schedule(static)
    for (int t = 0; t < nt; ++t) {
      const size_t b = (size_t)t * chunk;
      if (b < bytes) memcpy((char *)dst + b, (const char *)src + b, std::min(chunk, bytes - b));
    }
    return;
  }
#endif
  memcpy(dst, src, bytes);
}

// ---------------------------------------------------------------------------
struct TuneEntry {
  int variant, splits;
  float ms;
};

struct Engine {
  bool devinit = false, is_open = false;
  int device = 0, n_sm = 0;
  char devname[256] = {0};
  cudaStream_t stream = nullptr;
  cudaEvent_t ek0 = nullptr, ek1 = nullptr;   // autotuner timing
  std::vector<cudaEvent_t> evpool;            // per-launch timing pairs
  int evused = 0;
  int nbodymax = 0;
  // j-set
  int nj = 0;
  DevBuf jraw;     // m[nj] | x[nj][3] | v[nj][3]  (FP64 as sent)
  DevBuf jtiles;   // split-precision tiles
  PinBuf hj;
  // i-set and work buffers
  DevBuf iraw;     // h2[ni] | dtr[ni] | x[ni][3] | v[ni][3]
  DevBuf part, cnt, rows, rowlen, off, btot, dense, outblk, err;
  // spatial ordering: j permutation (tile slot -> sent index), i permutation,
  // bounding box of the j-set, sort scratch
  DevBuf jperm, iperm, bbox, okeys, okeys_alt, ovals_alt, otemp;
  DevBuf queue;    // work-item counter of the persistent pair kernel
  DevBuf irec;     // FP32 i-records of the current active block
  PinBuf hin, hout, hlist;
  std::vector<size_t> host_offs;  // row offsets of the compacted list (host)
  // configuration
  int precision = 0;
  int force_variant = -1, force_splits = 0;
  int timing = 0;
  float last_kernel_ms = 0.f;
  int last_variant = -1, last_splits = 0, last_gx = 0;
  bool last_fused = false;   // the last pair pass merged its partials itself
  std::map<long long, TuneEntry> tune;
  int autotune_on = 0;
  // host arrays of the gpunb_* calls: 1 = copied straight from/to the
  // caller's (pageable) arrays and list rows written by the device, which
  // needs coherent access to pageable memory through the host's page tables
  // (Grace + GB300 over NVLink-C2C); 0 = staged through pinned buffers
  int host_direct = 0;
  int host_direct_supported = 0;
  // j-set ordering: re-sorted along the Morton curve when nj changes and on
  // every resort_every-th send; the sends between reuse the permutation
  int resort_every = 8;
  int sends_since_sort = 0;
  int sorted_nj = -1;
  long long sorts = 0;
  // profile counters (GPUNB_profile)
  double time_send = 0, time_grav = 0, time_reduce = 0, time_out = 0;
  long long num_inter = 0;
  long long icall = 0, ini = 0, isend = 0;
  // potential
  DevBuf praw, ptiles, ppart, pout, pperm, piperm, pbbox;
  PinBuf hp;
};

static Engine g;
static std::mutex g_mutex;

// largest active block per call: the two-level list scan covers
// SCAN_ITEMS * SCAN_ITEMS rows (4096 * 4096)
constexpr int kMaxNi = 4096 * 4096;

// Replaces the tuning cache with the entries of a saved file; -1 (cache
// unchanged) when the file cannot be opened.  Caller holds g_mutex.
static int tune_load(const char *path) {
  FILE *f = path ? fopen(path, "r") : nullptr;
  if (!f) return -1;
  g.tune.clear();   // the file's entries replace the cache
  int n = 0;
  long long key;
  int v, s;
  float ms;
  while (fscanf(f, "%lld %d %d %f", &key, &v, &s, &ms) == 4) {
    if (v >= 0 && v < regf_num_variants() && s > 0) {
      g.tune[key] = TuneEntry{v, s, ms};
      ++n;
    }
  }
  fclose(f);
  return n;
}

static bool devinit(int irank) {
  if (g.devinit) return true;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) {
    cudaGetLastError();
    fail(GPUNB_E_NO_DEVICE, "no CUDA device visible");
    return false;
  }
  int dev = 0;
  if (const char *gl = getenv("GPU_LIST")) dev = atoi(gl);
  if (dev < 0 || dev >= ndev) dev = 0;
  CUDA_OR(cudaSetDevice(dev), false);
  cudaDeviceProp prop;
  CUDA_OR(cudaGetDeviceProperties(&prop, dev), false);
  g.device = dev;
  g.n_sm = prop.multiProcessorCount;
  snprintf(g.devname, sizeof(g.devname), "%s", prop.name);
  CUDA_OR(cudaStreamCreateWithFlags(&g.stream, cudaStreamNonBlocking), false);
  CUDA_OR(cudaEventCreate(&g.ek0), false);
  CUDA_OR(cudaEventCreate(&g.ek1), false);
  if (!g.err.ensure(sizeof(int)) || !g.bbox.ensure_zero(BBOX_INTS * sizeof(int)) ||
      !g.queue.ensure(sizeof(int)))
    return false;
  char host[150] = {0};
  gethostname(host, sizeof(host) - 1);
  fprintf(stderr, "# GPU initialization - rank: %d; HOST %s; NGPU 1; device: %d %s\n", irank,
          host, dev, prop.name);
  int pageable = 0, host_tables = 0;
  if (cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables,
                             dev) != cudaSuccess) {
    cudaGetLastError();
    pageable = host_tables = 0;
  }
  g.host_direct_supported = (pageable && host_tables) ? 1 : 0;
  g.host_direct = g.host_direct_supported;
  if (const char *p = getenv("GPUNB_HOST_DIRECT")) g.host_direct &= (atoi(p) != 0);
  g.devinit = true;
  if (const char *p = getenv("GPUNB_TUNE_CACHE")) tune_load(p);
  if (const char *p = getenv("GPUNB_AUTOTUNE")) g.autotune_on = atoi(p);
  if (const char *p = getenv("GPUNB_GRAPHS")) g_use_graphs = atoi(p) != 0;
  if (const char *p = getenv("GPUNB_RESORT_EVERY")) g.resort_every = std::max(1, atoi(p));
  return true;
}

// device error word -> host error
static bool check_device_error(int code_from_device) {
  if (code_from_device == 0) return true;
  const char *what = code_from_device == GPUNB_E_NAN       ? "NaN in an input array"
                     : code_from_device == GPUNB_E_TIMEOUT ? "a device wait timed out"
                                                           : "device error";
  fail(code_from_device, "%s", what);
  return false;
}

// ---------------------------------------------------------------------------
// j-set upload: FP64 arrays on the device + split-precision tiles
// Morton ordering scratch: keys, alternate keys/values and the sort's temp.
static bool ensure_order_scratch(int n) {
  const size_t nn = (size_t)std::max(n, 1);
  return g.okeys.ensure(nn * sizeof(unsigned long long)) &&
         g.okeys_alt.ensure(nn * sizeof(unsigned long long)) &&
         g.ovals_alt.ensure(nn * sizeof(int)) && g.otemp.ensure(order_temp_bytes((int)nn));
}

// Whether the next send re-orders the j-set along the Morton curve: when nj
// differs from the last ordered set's, and on every resort_every-th send.
// The sends between keep the permutation -- bodies move little between the
// block times of consecutive sends (intgrt.F:912-944), and the tiles are
// re-packed from the current positions with their true centres, radii and
// boxes, so results do not depend on the choice; only the spatial coherence
// of the tiles, and with it the speed, would decay if bodies travelled far.
// Taken once per call, outside any captured launch sequence.
static bool send_resorts(int nj) {
  return nj != g.sorted_nj || g.resort_every <= 1 || g.sends_since_sort + 1 >= g.resort_every;
}
static void send_account(int nj, bool resorted) {
  if (resorted) {
    g.sorted_nj = nj;
    g.sends_since_sort = 0;
    ++g.sorts;
  } else {
    ++g.sends_since_sort;
  }
}

static int send_common(int nj, cudaStream_t st, bool resort) {
  const int ntile = (nj + JT - 1) / JT;
  const size_t perm_bytes = (size_t)std::max(ntile, 1) * JT * sizeof(int);
  if (perm_bytes > g.jperm.bytes) resort = true;   // a new permutation buffer
  if (!g.jtiles.ensure((size_t)std::max(ntile, 1) * TILE_BYTES) || !g.jperm.ensure(perm_bytes) ||
      !ensure_order_scratch(nj))
    return GPUNB_E_ALLOC;
  double *m = g.jraw.as<double>();
  const double *x = m + nj;
  if (resort) {
    // spatial order of the j-set: bounding box, Morton keys, stable sort
    CUDA_OR(launch_bbox(x, nj, g.bbox.as<int>(), st), GPUNB_E_CUDA);
    CUDA_OR(launch_order(x, nj, g.bbox.as<int>(), g.okeys.as<unsigned long long>(),
                         g.okeys_alt.as<unsigned long long>(), g.ovals_alt.as<int>(),
                         g.jperm.as<int>(), g.otemp.p, g.otemp.bytes, st),
            GPUNB_E_CUDA);
    // padding slots of the last tile map to -1 (never a neighbour)
    if (ntile * JT > nj)
      CUDA_OR(cudaMemsetAsync(g.jperm.as<int>() + nj, 0xff,
                              (size_t)(ntile * JT - nj) * sizeof(int), st),
              GPUNB_E_CUDA);
  }
  CUDA_OR(launch_pack_jtiles(m, x, m + 4 * (size_t)nj, nj, g.jperm.as<int>(),
                             g.jtiles.as<float>(), ntile, g.err.as<int>(), st),
          GPUNB_E_CUDA);
  g.nj = nj;
  return GPUNB_OK;
}

// Morton order of an active block (within the j-set's bounding box); blocks
// too small to gain from it keep the caller's order (perm = null).
constexpr int kOrderMinNi = 256;
// Prepares an active block for the split-precision kernel: Morton order
// (skipped for small blocks) and the FP32 i-records in that order.
static int order_iset(ISet &is, cudaStream_t st) {
  is.perm = nullptr;
  is.rec = nullptr;
  if (is.ni >= kOrderMinNi && g.nj > 0) {
    if (!g.iperm.ensure((size_t)is.ni * sizeof(int)) || !ensure_order_scratch(is.ni))
      return GPUNB_E_ALLOC;
    CUDA_OR(launch_order(is.x, is.ni, g.bbox.as<int>(), g.okeys.as<unsigned long long>(),
                         g.okeys_alt.as<unsigned long long>(), g.ovals_alt.as<int>(),
                         g.iperm.as<int>(), g.otemp.p, g.otemp.bytes, st),
            GPUNB_E_CUDA);
    is.perm = g.iperm.as<int>();
  }
  if (!g.irec.ensure((size_t)std::max(is.ni, 1) * 4 * sizeof(float4))) return GPUNB_E_ALLOC;
  CUDA_OR(launch_regf_prep(is, g.irec.as<float4>(), g.err.as<int>(), st), GPUNB_E_CUDA);
  is.rec = g.irec.as<float4>();
  return GPUNB_OK;
}

static JSet jset() {
  JSet js;
  const double *m = g.jraw.as<double>();
  js.tiles = g.jtiles.as<float>();
  js.m64 = m;
  js.x64 = m + g.nj;
  js.v64 = m + 4 * (size_t)g.nj;
  js.perm = g.jperm.as<int>();
  js.nj = g.nj;
  js.ntile = (g.nj + JT - 1) / JT;
  js.ntile64 = (g.nj + JT64 - 1) / JT64;
  return js;
}

// ---------------------------------------------------------------------------
// launch planning
static long long tune_key(int nj, int ni, int mflag, int prec) {
  auto bucket = [](int n) {
    if (n <= 1) return 0;
    int b = 0;
    while ((2ll << b) <= n) ++b;                      // floor(log2 n)
    const int half = (n >= (3ll << b) / 2) ? 1 : 0;  // half-octave
    return 2 * b + half;
  };
  return ((long long)bucket(nj) << 24) | ((long long)bucket(ni) << 8) | (mflag << 1) | prec;
}

// j-splits: about 32 work items per resident block (the dynamic queue then
// balances the blocks to within one short item), at least one tile per item.
// Measured on GB300 (Plummer N = 65536, blocks of 16384 and 65536): 32 items
// per block beat 64 by 1-1.3% (half the partial sums to write and merge) and
// 16 by about as much (coarser balance).
static int plan_splits(int variant, int ni, int ntile, bool mflag) {
  const VariantDesc d = regf_variant(variant);
  const int gx = (ni + d.itile() - 1) / d.itile();
  const int bps = regf_ds_blocks_per_sm(variant, mflag);
  const long long want = 32ll * g.n_sm * bps;
  long long s = (want + gx - 1) / gx;
  const int smax = std::max(1, ntile);
  if (s > smax) s = smax;
  if (s < 1) s = 1;
  return (int)s;
}

// Shapes measured on GB300 (Plummer N = 65536, pair-kernel time of each
// variant at its own split count): below 256 i-particles one warp of 32 i
// with the j tile split over 8 warps (variant 2); from 256 on 4 warps x 32 i
// reading 8 j per warp vote (variant 6, 4 blocks per SM), which beats the
// 4-j vote at 5 blocks per SM (variant 4) by 3-5 % at every size from 512 to
// 16384 (0.081 / 0.132 / 0.214 / 0.370 / 0.673 / 1.235 ms at ni = 512 ...
// 16384 against 0.085 / 0.136 / 0.224 / 0.388 / 0.722 / 1.286) and variant 2
// by 15 % at 256.
static void heuristic_plan(int ni, int ntile, bool mflag, int &variant, int &splits) {
  variant = ni < 256 ? 2 : 6;
  splits = plan_splits(variant, ni, ntile, mflag);
}

static void fp64_plan(int ni, int ntile64, int &gx, int &splits) {
  gx = (ni + FP64_THREADS - 1) / FP64_THREADS;
  const long long want = 8ll * g.n_sm;
  long long s = (want + gx - 1) / gx;
  if (s > std::max(1, ntile64)) s = std::max(1, ntile64);
  splits = (int)std::max(1ll, s);
}

// ---------------------------------------------------------------------------
// the pair pass + merge + list compaction, all queued on `st`.
// Inputs: device ISet; outputs: device acc/jrk/pot/nnb/dense list.
struct RegfDev {
  double *acc, *jrk, *pot;
  int *nnb, *rowlen, *off, *btot, *dense;
};

static bool ensure_work(int ni, int nnbmax, int S, int ni_pad) {
  return g.part.ensure((size_t)S * NQ * ni_pad * sizeof(double)) &&
         g.cnt.ensure((size_t)ni * sizeof(int)) &&
         g.rows.ensure((size_t)ni * std::max(nnbmax, 1) * sizeof(int));
}

// The pair kernel merges its partials itself (merge_itile) for the split
// kernel when S <= FUSE_MAX_SPLITS: one block sums an i-tile's S rows, which
// for many splits (small blocks against a large j-set, S up to thousands) is
// a long serial tail that the merge kernels spread over many blocks.
// Measured on GB300 at S = 38 (Plummer N = ni = 65536): pair kernel + merge
// 4.55 -> 4.52 ms and 135 -> 42 MB of DRAM traffic per launch.
constexpr int FUSE_MAX_SPLITS = 48;

// fuse: the outputs the pair kernel merges into (used when the rule above
// holds; g.last_fused tells finish_lists whether a merge kernel must run).
static int run_pair_pass(const ISet &is, int nnbmax, bool mflag, int variant, int S,
                         cudaStream_t st, bool timed, const RegfDev *fuse) {
  const JSet js = jset();
  const int ni = is.ni;
  RegfOut out;
  int gx;
  if (g.precision != 0) {
    gx = (ni + FP64_THREADS - 1) / FP64_THREADS;
    out.ni_pad = gx * FP64_THREADS;
  } else {
    const VariantDesc d = regf_variant(variant);
    gx = (ni + d.itile() - 1) / d.itile();
    out.ni_pad = gx * d.itile();
  }
  if (!ensure_work(ni, nnbmax, S, out.ni_pad)) return GPUNB_E_ALLOC;
  const bool fused = fuse && g.precision == 0 && S <= FUSE_MAX_SPLITS;
  g.last_fused = fused;
  if (!g.queue.ensure((size_t)(1 + (fused ? gx : 0)) * sizeof(int))) return GPUNB_E_ALLOC;
  if (fused) {
    out.done = g.queue.as<int>() + 1;
    out.perm = is.perm;
    out.acc = fuse->acc;
    out.jrk = fuse->jrk;
    out.pot = fuse->pot;
    out.nnb = fuse->nnb;
    out.rowlen = fuse->rowlen;
    out.nnbmax = nnbmax;
  }
  out.part = g.part.as<double>();
  out.cnt = g.cnt.as<int>();
  out.rows = g.rows.as<int>();
  out.cap = std::max(nnbmax, 0);
  out.err = g.err.as<int>();
  CUDA_OR(cudaMemsetAsync(out.cnt, 0, (size_t)ni * sizeof(int), st), GPUNB_E_CUDA);
  // events: the autotuner uses ek0/ek1; timing mode takes a fresh pair from
  // the pool so that every launch of a timed region can be read afterwards
  cudaEvent_t e0 = g.ek0, e1 = g.ek1;
  const bool pooled = !timed && g.timing;
  if (pooled) {
    if ((int)g.evpool.size() < 2 * (g.evused + 1)) {
      cudaEvent_t a, b;
      CUDA_OR(cudaEventCreate(&a), GPUNB_E_CUDA);
      CUDA_OR(cudaEventCreate(&b), GPUNB_E_CUDA);
      g.evpool.push_back(a);
      g.evpool.push_back(b);
    }
    e0 = g.evpool[2 * g.evused];
    e1 = g.evpool[2 * g.evused + 1];
    g.evused++;
  }
  if (timed || pooled) CUDA_OR(cudaEventRecord(e0, st), GPUNB_E_CUDA);
  if (g.precision == 1) {
    CUDA_OR(launch_regf_fp64(mflag, gx, S, js, is, out, st), GPUNB_E_CUDA);
  } else if (g.precision == 2) {
    CUDA_OR(launch_regf_df(mflag, gx, S, js, is, out, st), GPUNB_E_CUDA);
  } else {
    const long long items = (long long)gx * S;
    const long long resident = (long long)g.n_sm * regf_ds_blocks_per_sm(variant, mflag);
    const int grid = (int)std::max(1ll, std::min(items, resident));
    CUDA_OR(launch_regf_ds(variant, mflag, gx, S, grid, g.queue.as<int>(), js, is, out, st),
            GPUNB_E_CUDA);
  }
  if (timed || pooled) CUDA_OR(cudaEventRecord(e1, st), GPUNB_E_CUDA);
  g.last_variant = g.precision != 0 ? -1 : variant;
  g.last_splits = S;
  g.last_gx = gx;
  return GPUNB_OK;
}

// merged: the pair kernel merged its partials into o (run_pair_pass with o)
static int finish_lists(int ni, int nnbmax, int S, int ni_pad, const int *perm, const RegfDev &o,
                        size_t list_cap, cudaStream_t st, bool merged) {
  if (!merged)
    CUDA_OR(launch_regf_merge(g.part.as<double>(), g.precision == 0, S, ni, ni_pad, perm,
                              g.cnt.as<int>(), nnbmax, o.acc, o.jrk, o.pot, o.nnb, o.rowlen, st),
            GPUNB_E_CUDA);
  CUDA_OR(launch_list_scan(o.rowlen, ni, o.off, o.btot, st), GPUNB_E_CUDA);
  (void)list_cap;
  CUDA_OR(launch_list_gather(g.rows.as<int>(), std::max(nnbmax, 0), o.rowlen, o.off, o.btot, ni,
                             o.dense, st),
          GPUNB_E_CUDA);
  return GPUNB_OK;
}

static void choose_plan(int ni, bool mflag, int &variant, int &S) {
  const JSet js = jset();
  if (g.precision != 0) {
    int gx;
    fp64_plan(ni, js.ntile64, gx, S);
    variant = -1;
    return;
  }
  heuristic_plan(ni, js.ntile, mflag, variant, S);
  auto it = g.tune.find(tune_key(g.nj, ni, mflag, 0));
  if (it != g.tune.end()) {
    variant = it->second.variant;
    S = std::min(it->second.splits, std::max(1, js.ntile));
  }
  if (g.force_variant >= 0 && g.force_variant < regf_num_variants()) variant = g.force_variant;
  if (g.force_splits > 0) S = std::min(g.force_splits, std::max(1, js.ntile));
}

// Times every launch shape (kernel variant x j-split count around the
// heuristic's) on the given device i-set -- the caller's own active block --
// and keeps the fastest in the cache under the (N, ni) bucket.  The time
// covers the pair kernel with the merge of its split partials, which its
// last item per i-tile does (more splits balance the persistent queue better
// but leave more partials to merge); the merge writes into scratch.  Runs on `st`, synchronously.
static int autotune_with(const ISet &is, int nnbmax, bool mflag, int *splits_out,
                         float *ms_out, cudaStream_t st) {
  const JSet js = jset();
  const int ni = is.ni;
  int best_v = -1, best_s = 1;
  float best = 1e30f;
  // the fastest plan whose pair kernel merges itself (its partial rows stay
  // in L2): taken when within 1% of the fastest overall
  int fused_v = -1, fused_s = 1;
  float fused_best = 1e30f;
  if (!g.outblk.ensure((size_t)7 * ni * sizeof(double) + (size_t)(ni + 2) * sizeof(int)) ||
      !g.rowlen.ensure((size_t)ni * sizeof(int)))
    return -1;
  double *sacc = g.outblk.as<double>();
  RegfDev scratch;   // the merge writes here (the pair kernel merges itself)
  scratch.acc = sacc;
  scratch.jrk = sacc + 3 * (size_t)ni;
  scratch.pot = sacc + 6 * (size_t)ni;
  scratch.nnb = (int *)(sacc + 7 * (size_t)ni);
  scratch.rowlen = g.rowlen.as<int>();
  for (int v = 0; v < regf_num_variants(); ++v) {
    const long long base = plan_splits(v, ni, js.ntile, mflag);
    const long long cands[5] = {base / 4, base / 2, base, base * 2, base * 4};
    int last_s = -1;
    for (long long sc : cands) {
      int s = (int)std::max(1ll, std::min<long long>(sc, std::max(1, js.ntile)));
      if (s == last_s) continue;
      last_s = s;
      // one warm-up pass, then three timed ones -- or one when a pass takes
      // longer than 20 ms (large blocks: the timing is stable, the sweep long)
      float tot = 0.f;
      int reps = 3;
      bool ok = true;
      for (int r = 0; r < reps + 1 && ok; ++r) {
        if (run_pair_pass(is, nnbmax, mflag, v, s, st, true, &scratch) != GPUNB_OK) ok = false;
        if (ok && cudaEventRecord(g.ek1, st) != cudaSuccess) ok = false;
        if (cudaStreamSynchronize(st) != cudaSuccess) ok = false;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, g.ek0, g.ek1);
        if (r > 0) tot += ms;
        if (r == 0 && ms > 20.f) reps = 1;
      }
      if (!ok) cudaGetLastError();
      if (!ok) continue;
      const float ms = tot / reps;
      if (ms < best) {
        best = ms;
        best_v = v;
        best_s = s;
      }
      if (s <= FUSE_MAX_SPLITS && ms < fused_best) {
        fused_best = ms;
        fused_v = v;
        fused_s = s;
      }
    }
  }
  if (fused_v >= 0 && fused_best <= 1.01f * best) {
    best = fused_best;
    best_v = fused_v;
    best_s = fused_s;
  }
  if (best_v >= 0) g.tune[tune_key(g.nj, ni, mflag, 0)] = TuneEntry{best_v, best_s, best};
  if (splits_out) *splits_out = best_s;
  if (ms_out) *ms_out = best;
  return best_v;
}

// ---------------------------------------------------------------------------
// host-buffer regf where the device reads and writes the caller's arrays
// (coherent host memory): every step is device work, so the call is one
// launch sequence, replayed as a CUDA graph per call key when graphs are on.
static void regf_host_direct(int ni, const double *h2, const double *dtr, const double (*xi)[3],
                             const double (*vi)[3], double (*acc)[3], double (*jrk)[3],
                             double *pot, int lmax, int nnbmax, int *list, int m_flag,
                             double t_begin) {
  cudaStream_t st = g.stream;
  const bool mflag = m_flag != 0;
  int variant, S;
  choose_plan(ni, mflag, variant, S);
  if (!g.hout.ensure(sizeof(int))) return;
  int *h_err = g.hout.as<int>();
  auto issue = [&](cudaStream_t s) -> int {
    double *din = g.iraw.as<double>();
    CUDA_OR(cudaMemsetAsync(g.err.p, 0, sizeof(int), s), GPUNB_E_CUDA);
    HostCopyJobs jobs;
    jobs.count = 4;
    jobs.j[0] = HostCopyJob{h2, din, ni, 8};
    jobs.j[1] = HostCopyJob{dtr, din + ni, ni, 8};
    jobs.j[2] = HostCopyJob{xi, din + 2 * (size_t)ni, 3ll * ni, 8};
    jobs.j[3] = HostCopyJob{vi, din + 5 * (size_t)ni, 3ll * ni, 8};
    CUDA_OR(launch_host_copy(jobs, s), GPUNB_E_CUDA);
    ISet is;
    is.h2 = din;
    is.dtr = din + ni;
    is.x = din + 2 * (size_t)ni;
    is.v = din + 5 * (size_t)ni;
    is.ni = ni;
    is.perm = nullptr;
    is.rec = nullptr;
    if (g.precision == 0 && order_iset(is, s) != GPUNB_OK) return GPUNB_E_ALLOC;
    const int nb = list_scan_blocks(ni);
    if (!g.outblk.ensure((size_t)7 * ni * sizeof(double) + (size_t)(ni + 2) * sizeof(int)) ||
        !g.rowlen.ensure((size_t)ni * sizeof(int)) ||
        !g.off.ensure((size_t)(ni + 1) * sizeof(int)) ||
        !g.btot.ensure((size_t)(nb + 1) * sizeof(int)) ||
        !g.dense.ensure((size_t)ni * std::max(nnbmax, 1) * sizeof(int)))
      return GPUNB_E_ALLOC;
    double *ob = g.outblk.as<double>();
    RegfDev o;
    o.acc = ob;
    o.jrk = ob + 3 * (size_t)ni;
    o.pot = ob + 6 * (size_t)ni;
    o.nnb = (int *)(ob + 7 * (size_t)ni);
    o.rowlen = g.rowlen.as<int>();
    o.off = g.off.as<int>();
    o.btot = g.btot.as<int>();
    o.dense = g.dense.as<int>();
    int rc = run_pair_pass(is, nnbmax, mflag, variant, S, s, false, &o);
    if (rc != GPUNB_OK) return rc;
    const int itile = g.precision != 0 ? FP64_THREADS : regf_variant(variant).itile();
    const int ni_pad = ((ni + itile - 1) / itile) * itile;
    rc = finish_lists(ni, nnbmax, S, ni_pad, is.perm, o, 0, s, g.last_fused);
    if (rc != GPUNB_OK) return rc;
    // results straight into the caller's arrays; the device writes the rows
    CUDA_OR(launch_list_rows(o.dense, o.off, o.btot, o.nnb, ni, lmax, list, s), GPUNB_E_CUDA);
    HostCopyJobs oj;
    oj.count = 4;
    oj.j[0] = HostCopyJob{o.acc, acc, 3ll * ni, 8};
    oj.j[1] = HostCopyJob{o.jrk, jrk, 3ll * ni, 8};
    oj.j[2] = HostCopyJob{o.pot, pot, ni, 8};
    oj.j[3] = HostCopyJob{g.err.p, h_err, 1, 4};
    CUDA_OR(launch_host_copy(oj, s), GPUNB_E_CUDA);
    return GPUNB_OK;
  };
  int rc;
  if (g_use_graphs && !g.timing) {
    const std::vector<long long> key = {
        3, ni, g.nj, lmax, nnbmax, m_flag, g.precision, variant, S,
        (long long)(uintptr_t)h2, (long long)(uintptr_t)dtr, (long long)(uintptr_t)xi,
        (long long)(uintptr_t)vi, (long long)(uintptr_t)acc, (long long)(uintptr_t)jrk,
        (long long)(uintptr_t)pot, (long long)(uintptr_t)list, (long long)(uintptr_t)st};
    rc = run_graphed(dev_graph(key), true, st, issue);
  } else {
    rc = issue(st);
  }
  if (rc != GPUNB_OK) return;
  CUDA_OR(cudaStreamSynchronize(st), );
  g.time_grav += wtime() - t_begin;
  check_device_error(*h_err);
}

// ---------------------------------------------------------------------------
// host-buffer regf: the gpunb_regf_ contract
static void regf_host(int ni, const double *h2, const double *dtr, const double (*xi)[3],
                      const double (*vi)[3], double (*acc)[3], double (*jrk)[3], double *pot,
                      int lmax, int nnbmax, int *list, int m_flag) {
  if (!g.is_open) { fail(GPUNB_E_NOT_OPEN, "gpunb_regf_ called before gpunb_open_"); return; }
  if (ni <= 0 || ni > kMaxNi) {
    fail(GPUNB_E_ARG, "gpunb_regf_: ni = %d outside [1, %d]", ni, kMaxNi);
    return;
  }
  if (nnbmax < 0 || lmax < 1 || nnbmax > lmax - 1) {
    fail(GPUNB_E_ARG, "gpunb_regf_: need 0 <= nnbmax (%d) <= lmax-1 (%d)", nnbmax, lmax - 1);
    return;
  }
  const double t_begin = wtime();
  g.num_inter += (long long)ni * g.nj;
  g.ini += ni;
  g.icall++;
  cudaStream_t st = g.stream;
  const bool mflag = m_flag != 0;

  // inputs: h2 | dtr | x | v
  const size_t in_doubles = (size_t)8 * ni;
  if (!g.iraw.ensure(in_doubles * sizeof(double))) return;
  double *din = g.iraw.as<double>();
  if (g.host_direct && !(g.autotune_on && g.precision == 0 && g.force_variant < 0 &&
                         g.tune.find(tune_key(g.nj, ni, mflag, 0)) == g.tune.end())) {
    regf_host_direct(ni, h2, dtr, xi, vi, acc, jrk, pot, lmax, nnbmax, list, m_flag, t_begin);
    return;
  }
  CUDA_OR(cudaMemsetAsync(g.err.p, 0, sizeof(int), st), );
  if (g.host_direct) {
    HostCopyJobs jobs;
    jobs.count = 4;
    jobs.j[0] = HostCopyJob{h2, din, ni, 8};
    jobs.j[1] = HostCopyJob{dtr, din + ni, ni, 8};
    jobs.j[2] = HostCopyJob{xi, din + 2 * (size_t)ni, 3ll * ni, 8};
    jobs.j[3] = HostCopyJob{vi, din + 5 * (size_t)ni, 3ll * ni, 8};
    CUDA_OR(launch_host_copy(jobs, st), );
  } else {
    if (!g.hin.ensure(in_doubles * sizeof(double))) return;
    double *hin = g.hin.as<double>();
    hcopy(hin, h2, (size_t)ni * sizeof(double));
    hcopy(hin + ni, dtr, (size_t)ni * sizeof(double));
    hcopy(hin + 2 * (size_t)ni, xi, (size_t)ni * 3 * sizeof(double));
    hcopy(hin + 5 * (size_t)ni, vi, (size_t)ni * 3 * sizeof(double));
    CUDA_OR(cudaMemcpyAsync(din, hin, in_doubles * sizeof(double), cudaMemcpyHostToDevice, st), );
  }
  ISet is;
  is.h2 = din;
  is.dtr = din + ni;
  is.x = din + 2 * (size_t)ni;
  is.v = din + 5 * (size_t)ni;
  is.ni = ni;
  is.perm = nullptr;
  is.rec = nullptr;
  if (g.precision == 0 && order_iset(is, st) != GPUNB_OK) return;

  int variant, S;
  if (g.autotune_on && g.precision == 0 && g.force_variant < 0 &&
      g.tune.find(tune_key(g.nj, ni, mflag, 0)) == g.tune.end())
    autotune_with(is, nnbmax, mflag, nullptr, nullptr, st);
  choose_plan(ni, mflag, variant, S);

  // outputs: acc | jrk | pot (doubles), then nnb (ints)
  const int nb = list_scan_blocks(ni);
  if (!g.outblk.ensure((size_t)7 * ni * sizeof(double) + (size_t)(ni + 2) * sizeof(int)) ||
      !g.rowlen.ensure((size_t)ni * sizeof(int)) || !g.off.ensure((size_t)(ni + 1) * sizeof(int)) ||
      !g.btot.ensure((size_t)(nb + 1) * sizeof(int)) ||
      !g.dense.ensure((size_t)ni * std::max(nnbmax, 1) * sizeof(int)))
    return;
  double *ob = g.outblk.as<double>();
  RegfDev o;
  o.acc = ob;
  o.jrk = ob + 3 * (size_t)ni;
  o.pot = ob + 6 * (size_t)ni;
  o.nnb = (int *)(ob + 7 * (size_t)ni);
  o.rowlen = g.rowlen.as<int>();
  o.off = g.off.as<int>();
  o.btot = g.btot.as<int>();
  o.dense = g.dense.as<int>();
  if (run_pair_pass(is, nnbmax, mflag, variant, S, st, false, &o) != GPUNB_OK) return;
  const int ni_pad = g.precision != 0
                         ? ((ni + FP64_THREADS - 1) / FP64_THREADS) * FP64_THREADS
                         : ((ni + regf_variant(variant).itile() - 1) / regf_variant(variant).itile()) *
                               regf_variant(variant).itile();
  if (finish_lists(ni, nnbmax, S, ni_pad, is.perm, o, 0, st, g.last_fused) != GPUNB_OK)
    return;
  if (g.host_direct) {
    // results straight into the caller's arrays; the device writes the rows
    CUDA_OR(launch_list_rows(o.dense, o.off, o.btot, o.nnb, ni, lmax, list, st), );
    if (!g.hout.ensure(sizeof(int))) return;
    int *h_err = g.hout.as<int>();
    HostCopyJobs jobs;
    jobs.count = 4;
    jobs.j[0] = HostCopyJob{o.acc, acc, 3ll * ni, 8};
    jobs.j[1] = HostCopyJob{o.jrk, jrk, 3ll * ni, 8};
    jobs.j[2] = HostCopyJob{o.pot, pot, ni, 8};
    jobs.j[3] = HostCopyJob{g.err.p, h_err, 1, 4};
    CUDA_OR(launch_host_copy(jobs, st), );
    CUDA_OR(cudaStreamSynchronize(st), );
    const double t_grav = wtime();
    g.time_grav += t_grav - t_begin;
    check_device_error(*h_err);
    return;
  }
  const size_t out_bytes = (size_t)7 * ni * sizeof(double) + (size_t)ni * sizeof(int);
  if (!g.hout.ensure(out_bytes + 2 * sizeof(int))) return;
  char *hob = g.hout.as<char>();
  int *h_total = (int *)(hob + out_bytes);
  int *h_err = h_total + 1;
  CUDA_OR(cudaMemcpyAsync(hob, ob, out_bytes, cudaMemcpyDeviceToHost, st), );
  CUDA_OR(cudaMemcpyAsync(h_total, o.btot + nb, sizeof(int), cudaMemcpyDeviceToHost, st), );
  CUDA_OR(cudaMemcpyAsync(h_err, g.err.p, sizeof(int), cudaMemcpyDeviceToHost, st), );
  CUDA_OR(cudaStreamSynchronize(st), );
  const double t_grav = wtime();
  g.time_grav += t_grav - t_begin;
  if (!check_device_error(*h_err)) return;
  const int total = *h_total;
  if (total > 0) {
    if (!g.hlist.ensure((size_t)total * sizeof(int))) return;
    CUDA_OR(cudaMemcpyAsync(g.hlist.p, o.dense, (size_t)total * sizeof(int),
                            cudaMemcpyDeviceToHost, st), );
    CUDA_OR(cudaStreamSynchronize(st), );
  }
  const double *hd = (const double *)hob;
  hcopy(acc, hd, (size_t)ni * 3 * sizeof(double));
  hcopy(jrk, hd + 3 * (size_t)ni, (size_t)ni * 3 * sizeof(double));
  hcopy(pot, hd + 6 * (size_t)ni, (size_t)ni * sizeof(double));
  const int *hnnb = (const int *)(hd + 7 * (size_t)ni);
  const int *hl = g.hlist.as<int>();
  // host scatter of the compacted list into rows of lmax
  if (ni < 4096) {
    size_t o2 = 0;
    for (int i = 0; i < ni; ++i) {
      const int c = hnnb[i];
      if (c > 0) o2 += c;
    }
    if (o2 != (size_t)std::max(total, 0)) {
      fail(GPUNB_E_CUDA, "list length mismatch: device %d, host %zu", total, o2);
      return;
    }
    o2 = 0;
    for (int i = 0; i < ni; ++i) {
      int *row = list + (size_t)i * lmax;
      const int c = hnnb[i];
      row[0] = c;
      if (c > 0) {
        memcpy(row + 1, hl + o2, (size_t)c * sizeof(int));
        o2 += c;
      }
    }
  } else {
    // offsets first (sequential), then parallel copies; the offsets live in
    // an engine-owned buffer shared by all worker threads
    g.host_offs.resize(ni);
    size_t *offs = g.host_offs.data();
    size_t o2 = 0;
    for (int i = 0; i < ni; ++i) {
      offs[i] = o2;
      if (hnnb[i] > 0) o2 += hnnb[i];
    }
    if (o2 != (size_t)std::max(total, 0)) {
      fail(GPUNB_E_CUDA, "list length mismatch: device %d, host %zu", total, o2);
      return;
    }
#pragma omp parallel for schedule(static)
    for (int i = 0; i < ni; ++i) {
      int *row = list + (size_t)i * lmax;
      const int c = hnnb[i];
      row[0] = c;
      if (c > 0) memcpy(row + 1, hl + offs[i], (size_t)c * sizeof(int));
    }
  }
  g.time_reduce += wtime() - t_grav;
}

// batched-cluster state lives in batch_impl.inc (end of this file)
static void batch_release();

}  // namespace gpunb

// ===========================================================================
// C ABI
using namespace gpunb;

extern "C" {

void gpunb_devinit_(int *irank) {
  std::lock_guard<std::mutex> lk(g_mutex);
  devinit(irank ? *irank : 0);
}

void gpunb_open_(int *nbmax, int *irank) {
  std::lock_guard<std::mutex> lk(g_mutex);
  const int rank = irank ? *irank : 0;
  g.time_send = g.time_grav = g.time_reduce = g.time_out = 0.0;
  g.num_inter = 0;
  g.icall = g.ini = g.isend = 0;
  if (!devinit(rank)) return;
  if (g.is_open) {
    fprintf(stderr, "gpunb: it is already open\n");
    return;
  }
  if (!nbmax || *nbmax < 0) {
    fail(GPUNB_E_ARG, "gpunb_open_: nbmax must be >= 0");
    return;
  }
  g.nbodymax = *nbmax;
  const size_t nmax = (size_t)std::max(g.nbodymax, 1);
  if (!g.jraw.ensure(nmax * 7 * sizeof(double)) ||
      !g.jtiles.ensure(((nmax + JT - 1) / JT) * (size_t)TILE_BYTES) ||
      !g.hj.ensure(nmax * 7 * sizeof(double)))
    return;
  g.nj = 0;
  // a new run starts from the default configuration (GPUNB_PRECISION: the
  // pair kernel, as gpunb_set_precision)
  g.precision = 0;
  if (const char *p = getenv("GPUNB_PRECISION")) {
    const int v = atoi(p);
    g.precision = (v == 1 || v == 2) ? v : 0;
  }
  g.force_variant = -1;
  g.force_splits = 0;
  g.timing = 0;
  g.evused = 0;
  g.is_open = true;
  fprintf(stderr, "# Open GPU regular force - rank: %d; nbmax: %d\n", rank, g.nbodymax);
}

void gpunb_close_(void) {
  std::lock_guard<std::mutex> lk(g_mutex);
  if (!g.is_open) {
    fprintf(stderr, "gpunb: it is already close\n");
    return;
  }
  if (g.stream) cudaStreamSynchronize(g.stream);
  batch_release();
  dev_graphs_drop();
  g.jraw.release(); g.jtiles.release(); g.hj.release();
  g.iraw.release(); g.part.release(); g.cnt.release(); g.rows.release();
  g.rowlen.release(); g.off.release(); g.btot.release(); g.dense.release();
  g.outblk.release(); g.hin.release(); g.hout.release(); g.hlist.release();
  g.jperm.release(); g.iperm.release(); g.okeys.release(); g.okeys_alt.release();
  g.ovals_alt.release(); g.otemp.release(); g.irec.release();
  g.nbodymax = 0;
  g.nj = 0;
  g.sorted_nj = -1;
  g.sends_since_sort = 0;
  g.is_open = false;
}

void gpunb_send_(int *nj, double mj[], double xj[][3], double vj[][3]) {
  std::lock_guard<std::mutex> lk(g_mutex);
  if (!g.is_open) { fail(GPUNB_E_NOT_OPEN, "gpunb_send_ called before gpunb_open_"); return; }
  const int n = *nj;
  if (n < 0 || n > g.nbodymax) {
    fail(GPUNB_E_CAPACITY, "gpunb_send_: nj = %d outside [0, nbmax = %d]", n, g.nbodymax);
    return;
  }
  const double t0 = wtime();
  g.isend++;
  cudaStream_t st = g.stream;
  const bool resort = send_resorts(n);
  if (g.host_direct) {
    // the device reads the caller's arrays: the whole call is device work,
    // replayed as a CUDA graph per (n, arrays) when graphs are on
    if (!g.hout.ensure(sizeof(int))) return;
    int *herr = g.hout.as<int>();
    auto issue = [&](cudaStream_t s) -> int {
      CUDA_OR(cudaMemsetAsync(g.err.p, 0, sizeof(int), s), GPUNB_E_CUDA);
      if (n > 0) {
        double *d = g.jraw.as<double>();
        HostCopyJobs jobs;
        jobs.count = 3;
        jobs.j[0] = HostCopyJob{mj, d, n, 8};
        jobs.j[1] = HostCopyJob{xj, d + n, 3ll * n, 8};
        jobs.j[2] = HostCopyJob{vj, d + 4 * (size_t)n, 3ll * n, 8};
        CUDA_OR(launch_host_copy(jobs, s), GPUNB_E_CUDA);
      }
      const int rc = send_common(n, s, resort);
      if (rc != GPUNB_OK) return rc;
      HostCopyJobs ej;
      ej.count = 1;
      ej.j[0] = HostCopyJob{g.err.p, herr, 1, 4};
      CUDA_OR(launch_host_copy(ej, s), GPUNB_E_CUDA);
      return GPUNB_OK;
    };
    int rc;
    if (g_use_graphs && !g.timing)
      rc = run_graphed(dev_graph({2, n, (long long)(uintptr_t)mj, (long long)(uintptr_t)xj,
                                  (long long)(uintptr_t)vj, (long long)(uintptr_t)st,
                                  resort ? 1 : 0}),
                       true, st, issue);
    else
      rc = issue(st);
    if (rc != GPUNB_OK) return;
    send_account(n, resort);
    g.nj = n;
    CUDA_OR(cudaStreamSynchronize(st), );
    check_device_error(*herr);
    g.time_send += wtime() - t0;
    return;
  }
  CUDA_OR(cudaMemsetAsync(g.err.p, 0, sizeof(int), st), );
  if (n > 0) {
    double *h = g.hj.as<double>();
    hcopy(h, mj, (size_t)n * sizeof(double));
    hcopy(h + n, xj, (size_t)n * 3 * sizeof(double));
    hcopy(h + 4 * (size_t)n, vj, (size_t)n * 3 * sizeof(double));
    CUDA_OR(cudaMemcpyAsync(g.jraw.p, h, (size_t)n * 7 * sizeof(double), cudaMemcpyHostToDevice,
                            st), );
  }
  if (send_common(n, st, resort) != GPUNB_OK) return;
  send_account(n, resort);
  if (!g.hout.ensure(sizeof(int))) return;
  int *herr = g.hout.as<int>();
  CUDA_OR(cudaMemcpyAsync(herr, g.err.p, sizeof(int), cudaMemcpyDeviceToHost, st), );
  CUDA_OR(cudaStreamSynchronize(st), );
  check_device_error(*herr);
  g.time_send += wtime() - t0;
}

void gpunb_regf_(int *ni, double h2[], double dtr[], double xi[][3], double vi[][3],
                 double acc[][3], double jrk[][3], double pot[], int *lmax, int *nnbmax,
                 int *list, int *m_flag) {
  std::lock_guard<std::mutex> lk(g_mutex);
  regf_host(*ni, h2, dtr, xi, vi, acc, jrk, pot, *lmax, *nnbmax, list, m_flag ? *m_flag : 0);
}

void gpunb_profile_(int *irank) {
  std::lock_guard<std::mutex> lk(g_mutex);
  const int rank = irank ? *irank : 0;
  if (g.icall) {
    fprintf(stderr,
            "[R.%d GPU Reg.F ] Nsend %lld  Ngrav %lld  <Ni> %lld   send(s) %f grav(s) %f  nb(s) %f  "
            "out(s) %f  Perf.(Gflops) %f\n",
            rank, g.isend, g.icall, g.isend ? g.ini / g.isend : 0, g.time_send, g.time_grav,
            g.time_reduce, g.time_out,
            g.time_grav > 0 ? 60.e-9 * (double)g.num_inter / g.time_grav : 0.0);
  }
  g.time_send = g.time_grav = g.time_reduce = g.time_out = 0.0;
  g.num_inter = 0;
  g.icall = g.ini = g.isend = 0;
}

void gpupot_(int *irank, int *istart, int *ni, int *n, double m[], double x[][3], double pot[]) {
  std::lock_guard<std::mutex> lk(g_mutex);
  if (!devinit(irank ? *irank : 0)) return;
  const double t0 = wtime();
  const int nn = *n, k = *ni, is0 = *istart - 1;
  if (nn < 0 || k < 0 || is0 < 0 || is0 + k > nn) {
    fail(GPUNB_E_ARG, "gpupot_: need 1 <= istart, istart-1+ni <= n (istart %d ni %d n %d)",
         *istart, k, nn);
    return;
  }
  if (k == 0) return;
  cudaStream_t st = g.stream;
  // the set in Morton order, packed into the regular force's tile layout
  // (own permutation and box buffers: the sent j-set's stay as they are)
  const int ntile = (nn + JT - 1) / JT;
  const int itile = pot_itile();
  const int gx = (k + itile - 1) / itile;
  const long long want = 2ll * g.n_sm * pot_rel_blocks_per_sm();
  int S = (int)std::max(1ll, std::min<long long>((want + gx - 1) / gx, std::max(1, ntile / 2)));
  const int ni_pad = gx * itile;
  const bool whole = is0 == 0 && k == nn;   // i in the j-set's own Morton order
  if (!g.praw.ensure((size_t)nn * 4 * sizeof(double)) || !g.hp.ensure((size_t)nn * 4 * sizeof(double)) ||
      !g.ptiles.ensure((size_t)std::max(ntile, 1) * TILE_FLOATS * sizeof(float)) ||
      !g.pperm.ensure((size_t)std::max(ntile, 1) * JT * sizeof(int)) ||
      !g.piperm.ensure((size_t)k * sizeof(int)) || !g.pbbox.ensure_zero(BBOX_INTS * sizeof(int)) ||
      !ensure_order_scratch(nn) || !g.ppart.ensure((size_t)S * ni_pad * sizeof(double)) ||
      !g.pout.ensure((size_t)k * sizeof(double) + sizeof(int)))
    return;
  double *h = g.hp.as<double>();
  hcopy(h, m, (size_t)nn * sizeof(double));
  hcopy(h + nn, x, (size_t)nn * 3 * sizeof(double));
  double *d = g.praw.as<double>();
  CUDA_OR(cudaMemsetAsync(g.err.p, 0, sizeof(int), st), );
  CUDA_OR(cudaMemcpyAsync(d, h, (size_t)nn * 4 * sizeof(double), cudaMemcpyHostToDevice, st), );
  int *perm = g.pperm.as<int>();
  CUDA_OR(launch_bbox(d + nn, nn, g.pbbox.as<int>(), st), );
  CUDA_OR(launch_order(d + nn, nn, g.pbbox.as<int>(), g.okeys.as<unsigned long long>(),
                       g.okeys_alt.as<unsigned long long>(), g.ovals_alt.as<int>(), perm,
                       g.otemp.p, g.otemp.bytes, st), );
  if (ntile * JT > nn)
    CUDA_OR(cudaMemsetAsync(perm + nn, 0xff, (size_t)(ntile * JT - nn) * sizeof(int), st), );
  CUDA_OR(launch_pack_jtiles(d, d + nn, nullptr, nn, perm, g.ptiles.as<float>(), ntile,
                             g.err.as<int>(), st), );
  const int *iorder = perm;
  if (!whole) {
    CUDA_OR(launch_order(d + nn + 3 * (size_t)is0, k, g.pbbox.as<int>(),
                         g.okeys.as<unsigned long long>(), g.okeys_alt.as<unsigned long long>(),
                         g.ovals_alt.as<int>(), g.piperm.as<int>(), g.otemp.p, g.otemp.bytes,
                         st), );
    iorder = g.piperm.as<int>();
  }
  CUDA_OR(launch_pot_rel(g.ptiles.as<float>(), ntile, d + nn, iorder, is0, k, gx, S,
                         g.ppart.as<double>(), ni_pad, g.err.as<int>(), st), );
  CUDA_OR(launch_pot_merge(g.ppart.as<double>(), S, k, ni_pad, g.err.as<int>(),
                           g.pout.as<double>(), st, iorder), );
  // results land in the staging buffer (reused: m/x no longer needed)
  CUDA_OR(cudaMemcpyAsync(h, g.pout.p, (size_t)k * sizeof(double), cudaMemcpyDeviceToHost, st), );
  int herr = 0;
  CUDA_OR(cudaMemcpyAsync(h + k, g.err.p, sizeof(int), cudaMemcpyDeviceToHost, st), );
  CUDA_OR(cudaStreamSynchronize(st), );
  memcpy(&herr, h + k, sizeof(int));
  if (!check_device_error(herr)) return;
  hcopy(pot, h, (size_t)k * sizeof(double));
  fprintf(stderr, "[R.%d GPU Pot.A] Ni %d  NTOT %d  pot(s) %f\n", irank ? *irank : 0, k, nn,
          wtime() - t0);
}

// ---- additions ------------------------------------------------------------

int gpunb_last_error(void) { return g_err_code; }
const char *gpunb_last_error_message(void) { return g_err_msg.c_str(); }
void gpunb_clear_error(void) {
  g_err_code = 0;
  g_err_msg.clear();
}
void gpunb_set_abort_on_error(int flag) { g_abort_on_error = flag; }

void gpunb_set_precision(int mode) { g.precision = (mode == 1 || mode == 2) ? mode : 0; }

void gpunb_set_launch(int variant, int splits) {
  g.force_variant = variant;
  g.force_splits = splits;
}

int gpunb_num_variants(void) { return regf_num_variants(); }

int gpunb_variant_info(int variant, int *ipt, int *warps_i, int *warps_j) {
  if (variant < 0 || variant >= regf_num_variants()) return -1;
  const VariantDesc d = regf_variant(variant);
  if (ipt) *ipt = d.ipt;
  if (warps_i) *warps_i = d.wi;
  if (warps_j) *warps_j = d.wj;
  return 0;
}

int gpunb_set_host_path(int mode) {
  std::lock_guard<std::mutex> lk(g_mutex);
  if (!devinit(0)) return -1;
  g.host_direct = (mode != 0) && g.host_direct_supported;
  return g.host_direct;
}

void gpunb_set_timing(int flag) {
  g.timing = flag;
  g.evused = 0;
}

int gpunb_kernel_times(float *ms, int max) {
  std::lock_guard<std::mutex> lk(g_mutex);
  int n = 0;
  for (int k = 0; k < g.evused && n < max; ++k) {
    if (cudaEventSynchronize(g.evpool[2 * k + 1]) != cudaSuccess) break;
    float t = 0.f;
    cudaEventElapsedTime(&t, g.evpool[2 * k], g.evpool[2 * k + 1]);
    ms[n++] = t;
  }
  if (n > 0) g.last_kernel_ms = ms[n - 1];
  g.evused = 0;
  return n;
}

float gpunb_last_kernel_ms(void) { return g.last_kernel_ms; }
void gpunb_last_launch(int *variant, int *splits, int *grid_x) {
  if (variant) *variant = g.last_variant;
  if (splits) *splits = g.last_splits;
  if (grid_x) *grid_x = g.last_gx;
}

int gpunb_autotune(int ni, int m_flag, int *splits, float *ms) {
  std::lock_guard<std::mutex> lk(g_mutex);
  if (!g.is_open || g.nj <= 0) {
    fail(GPUNB_E_NOT_OPEN, "gpunb_autotune needs an open library with a j-set");
    return -1;
  }
  if (ni <= 0) { fail(GPUNB_E_ARG, "gpunb_autotune: ni must be positive"); return -1; }
  // synthetic i-set: the first ni j-bodies (wrapping), h2 from the mean
  // inter-particle spacing so that lists have realistic lengths
  const int nj = g.nj;
  if (!g.iraw.ensure((size_t)8 * ni * sizeof(double)) || !g.hin.ensure((size_t)8 * ni * sizeof(double)))
    return -1;
  std::vector<double> hj((size_t)7 * nj);
  CUDA_OR(cudaMemcpy(hj.data(), g.jraw.p, hj.size() * sizeof(double), cudaMemcpyDeviceToHost), -1);
  double r2s = 0.0;
  for (int j = 0; j < nj; ++j)
    for (int c = 0; c < 3; ++c) r2s += hj[nj + 3 * (size_t)j + c] * hj[nj + 3 * (size_t)j + c];
  const double rms = std::sqrt(r2s / std::max(nj, 1));
  const double h2v = std::pow(rms * std::cbrt(100.0 / std::max(nj, 1)), 2);
  double *hin = g.hin.as<double>();
  for (int i = 0; i < ni; ++i) {
    const int j = i % nj;
    hin[i] = h2v;
    hin[ni + i] = 0.01;
    for (int c = 0; c < 3; ++c) {
      hin[2 * (size_t)ni + 3 * (size_t)i + c] = hj[nj + 3 * (size_t)j + c];
      hin[5 * (size_t)ni + 3 * (size_t)i + c] = hj[4 * (size_t)nj + 3 * (size_t)j + c];
    }
  }
  double *din = g.iraw.as<double>();
  CUDA_OR(cudaMemcpy(din, hin, (size_t)8 * ni * sizeof(double), cudaMemcpyHostToDevice), -1);
  ISet is;
  is.h2 = din; is.dtr = din + ni; is.x = din + 2 * (size_t)ni; is.v = din + 5 * (size_t)ni;
  is.ni = ni;
  if (order_iset(is, g.stream) != GPUNB_OK) return -1;
  const int saved = g.precision;
  g.precision = 0;
  const int v = autotune_with(is, 1024, m_flag != 0, splits, ms, g.stream);
  g.precision = saved;
  return v;
}

int gpunb_set_resort_interval(int every) {
  std::lock_guard<std::mutex> lk(g_mutex);
  const int prev = g.resort_every;
  g.resort_every = std::max(1, every);
  g.sends_since_sort = 0;
  g.sorted_nj = -1;   // the next send re-orders
  return prev;
}

long long gpunb_sort_count(void) { return g.sorts; }

int gpunb_set_autotune(int flag) {
  std::lock_guard<std::mutex> lk(g_mutex);
  const int prev = g.autotune_on;
  g.autotune_on = flag ? 1 : 0;
  return prev;
}

int gpunb_tune_load(const char *path) {
  std::lock_guard<std::mutex> lk(g_mutex);
  return tune_load(path);
}

int gpunb_tune_save(const char *path) {
  std::lock_guard<std::mutex> lk(g_mutex);
  FILE *f = path ? fopen(path, "w") : nullptr;
  if (!f) return -1;
  int n = 0;
  for (const auto &kv : g.tune) {
    fprintf(f, "%lld %d %d %.6f\n", kv.first, kv.second.variant, kv.second.splits, kv.second.ms);
    ++n;
  }
  fclose(f);
  return n;
}

int gpunb_send_device(int nj, const double *m, const double *x, const double *v, void *stream) {
  std::lock_guard<std::mutex> lk(g_mutex);
  if (!g.is_open) { fail(GPUNB_E_NOT_OPEN, "gpunb_send_device before gpunb_open_"); return GPUNB_E_NOT_OPEN; }
  if (nj < 0 || nj > g.nbodymax) {
    fail(GPUNB_E_CAPACITY, "gpunb_send_device: nj = %d outside [0, nbmax = %d]", nj, g.nbodymax);
    return GPUNB_E_CAPACITY;
  }
  cudaStream_t st = stream ? (cudaStream_t)stream : g.stream;
  const bool resort = send_resorts(nj);
  auto issue = [&](cudaStream_t s) -> int {
    double *d = g.jraw.as<double>();
    HostCopyJobs jobs;   // one copy kernel for the three arrays
    jobs.count = 3;
    jobs.j[0] = HostCopyJob{m, d, nj, 8};
    jobs.j[1] = HostCopyJob{x, d + nj, 3ll * nj, 8};
    jobs.j[2] = HostCopyJob{v, d + 4 * (size_t)nj, 3ll * nj, 8};
    CUDA_OR(launch_host_copy(jobs, s), GPUNB_E_CUDA);
    return send_common(nj, s, resort);
  };
  int rc;
  if (g_use_graphs && !g.timing)
    rc = run_graphed(dev_graph({0, nj, (long long)(uintptr_t)m, (long long)(uintptr_t)x,
                                (long long)(uintptr_t)v, (long long)(uintptr_t)st,
                                resort ? 1 : 0}),
                     true, st, issue);
  else
    rc = issue(st);
  if (rc == GPUNB_OK) {
    send_account(nj, resort);
    g.nj = nj;
  }
  return rc;
}

// A wait that nothing completes: one thread polls an mbarrier that no copy or
// arrival will ever complete, at most `polls` times, then records a timeout
// the way the library's kernels do when a bounded wait gives up.
__global__ void bounded_wait_probe_kernel(unsigned int polls, int *err) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
    if (!mbar_wait_bounded(&bar, 0u, polls)) raise_error(err, GPUNB_E_TIMEOUT);
  }
}

int gpunb_test_bounded_wait(int polls, void *stream) {
  std::lock_guard<std::mutex> lk(g_mutex);
  if (!devinit(0)) return GPUNB_E_NO_DEVICE;
  if (polls < 1 || polls > (1 << 22)) {
    fail(GPUNB_E_ARG, "gpunb_test_bounded_wait: polls %d outside [1, 2^22]", polls);
    return GPUNB_E_ARG;
  }
  cudaStream_t st = stream ? (cudaStream_t)stream : g.stream;
  bounded_wait_probe_kernel<<<1, 32, 0, st>>>((unsigned int)polls, g.err.as<int>());
  CUDA_OR(cudaGetLastError(), GPUNB_E_CUDA);
  return GPUNB_OK;
}

void gpunb_test_fail_allocs(int n) {
  std::lock_guard<std::mutex> lk(g_mutex);
  g_fail_allocs = n > 0 ? n : 0;
}

int gpunb_device_status(void *stream) {
  std::lock_guard<std::mutex> lk(g_mutex);
  if (!g.devinit || !g.err.p) return GPUNB_E_NO_DEVICE;
  cudaStream_t st = stream ? (cudaStream_t)stream : g.stream;
  int herr = 0;
  CUDA_OR(cudaStreamSynchronize(st), GPUNB_E_CUDA);
  CUDA_OR(cudaMemcpy(&herr, g.err.p, sizeof(int), cudaMemcpyDeviceToHost), GPUNB_E_CUDA);
  CUDA_OR(cudaMemset(g.err.p, 0, sizeof(int)), GPUNB_E_CUDA);
  check_device_error(herr);
  return herr;
}

int gpunb_regf_device(int ni, const double *h2, const double *dtr, const double *xi,
                      const double *vi, double *acc, double *jrk, double *pot, int *nnb,
                      int *list_off, int *list, size_t list_cap, int nnbmax, int m_flag,
                      void *stream) {
  std::lock_guard<std::mutex> lk(g_mutex);
  if (!g.is_open) { fail(GPUNB_E_NOT_OPEN, "gpunb_regf_device before gpunb_open_"); return GPUNB_E_NOT_OPEN; }
  if (ni <= 0 || ni > kMaxNi || nnbmax < 0) {
    fail(GPUNB_E_ARG, "gpunb_regf_device: ni %d nnbmax %d", ni, nnbmax);
    return GPUNB_E_ARG;
  }
  if (list_cap < (size_t)ni * (size_t)nnbmax) {
    fail(GPUNB_E_ARG, "gpunb_regf_device: list_cap %zu < ni*nnbmax", list_cap);
    return GPUNB_E_ARG;
  }
  cudaStream_t st = stream ? (cudaStream_t)stream : g.stream;
  const bool mflag = m_flag != 0;
  if (g.autotune_on && g.precision == 0 && g.force_variant < 0 && g.nj > 0 &&
      g.tune.find(tune_key(g.nj, ni, mflag, 0)) == g.tune.end()) {
    // first sight of this (N, ni) bucket: tune on the caller's own block
    ISet is;
    is.h2 = h2; is.dtr = dtr; is.x = xi; is.v = vi; is.ni = ni;
    is.perm = nullptr;
    is.rec = nullptr;
    if (order_iset(is, st) != GPUNB_OK) return GPUNB_E_ALLOC;
    if (autotune_with(is, nnbmax, mflag, nullptr, nullptr, st) < 0) return GPUNB_E_CUDA;
  }
  int variant, S;
  choose_plan(ni, mflag, variant, S);
  g.num_inter += (long long)ni * g.nj;
  g.ini += ni;
  g.icall++;
  auto issue = [&](cudaStream_t s) -> int {
    ISet is;
    is.h2 = h2; is.dtr = dtr; is.x = xi; is.v = vi; is.ni = ni;
    is.perm = nullptr;
    is.rec = nullptr;
    if (g.precision == 0 && order_iset(is, s) != GPUNB_OK) return GPUNB_E_ALLOC;
    const int nb = list_scan_blocks(ni);
    if (!g.rowlen.ensure((size_t)ni * sizeof(int)) ||
        !g.btot.ensure((size_t)(nb + 1) * sizeof(int)))
      return GPUNB_E_ALLOC;
    RegfDev o;
    o.acc = acc; o.jrk = jrk; o.pot = pot; o.nnb = nnb;
    o.rowlen = g.rowlen.as<int>(); o.off = list_off; o.btot = g.btot.as<int>(); o.dense = list;
    int rc = run_pair_pass(is, nnbmax, mflag, variant, S, s, false, &o);
    if (rc != GPUNB_OK) return rc;
    const int itile = g.precision != 0 ? FP64_THREADS : regf_variant(variant).itile();
    const int ni_pad = ((ni + itile - 1) / itile) * itile;
    rc = finish_lists(ni, nnbmax, S, ni_pad, is.perm, o, list_cap, s, g.last_fused);
    if (rc != GPUNB_OK) return rc;
    CUDA_OR(launch_list_finalize_offsets(list_off, o.btot, ni, s), GPUNB_E_CUDA);
    return GPUNB_OK;
  };
  // timing mode records host-side event bookkeeping per launch: run eagerly
  if (g_use_graphs && !g.timing) {
    const std::vector<long long> key = {
        1, ni, g.nj, nnbmax, m_flag, (long long)list_cap, g.precision, variant, S,
        (long long)(uintptr_t)h2, (long long)(uintptr_t)dtr, (long long)(uintptr_t)xi,
        (long long)(uintptr_t)vi, (long long)(uintptr_t)acc, (long long)(uintptr_t)jrk,
        (long long)(uintptr_t)pot, (long long)(uintptr_t)nnb, (long long)(uintptr_t)list_off,
        (long long)(uintptr_t)list, (long long)(uintptr_t)st};
    return run_graphed(dev_graph(key), true, st, issue);
  }
  return issue(st);
}

}  // extern "C"

// batched clusters (shares the engine state above)
#include "batch_impl.inc"
