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
// then one warp per active particle predicts the particle and its listed
// neighbours to the block time and sums the force, all in FP64.  On systems
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

#include "gpunb.h"
#include "internal.h"
#include "irr.h"

namespace gpunb {
namespace irr {

// particle record: 16 doubles {x0[3], m, v0[3], t0, a2[3], 0, j6[3], 0}
constexpr int REC = 16;
constexpr int IRR_WARPS = 8;   // warps per block; one active particle per warp

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

template <bool PRE>
__global__ void __launch_bounds__(32 * IRR_WARPS)
    irr_firr_kernel(int n, const double *__restrict__ rec, const double *__restrict__ pred,
                    int lmax, const int *__restrict__ lists, double ti, int ni,
                    const int *__restrict__ addr, int base, double *__restrict__ acc,
                    double *__restrict__ jrk, int *__restrict__ nnbid, int *__restrict__ err) {
  const int lane = threadIdx.x & 31;
  const int nwarps = (int)((gridDim.x * blockDim.x) >> 5);
  for (int k = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5); k < ni; k += nwarps) {
    const int i = addr[k] - base;
    double ax = 0, ay = 0, az = 0, jx = 0, jy = 0, jz = 0;
    double best = INFINITY;
    int bj = INT_MAX;
    if (i < 0 || i >= n) {
      if (lane == 0) flag(err, GPUNB_E_ARG);
    } else {
      double xi[3], vi[3], mi;
      state<PRE>(rec, pred, i, ti, xi, vi, mi);
      const int *row = lists + (size_t)i * lmax;
      int nnb = row[0];
      if (nnb < 0 || nnb > lmax - 1) {
        if (lane == 0) flag(err, GPUNB_E_ARG);
        nnb = 0;
      }
      for (int q = lane; q < nnb; q += 32) {
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
    // fixed butterfly: the same order on every call (deterministic)
    for (int o = 16; o > 0; o >>= 1) {
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
    if (lane == 0) {
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
  cudaStream_t st = nullptr;
  std::vector<double> rec_h;     // host mirror of the records
  std::vector<int> list_h;       // host mirror of the rows (0-based ids)
  std::vector<int> dirty_rec, dirty_row;
  std::atomic<long long> n_rec{0}, n_row{0};
  std::vector<unsigned> seen;    // epoch stamps for de-duplication
  unsigned epoch = 0;
  std::vector<int> uniq;
  DevBuf rec_d, list_d, addr_d, out_d, nid_d, idx_d, stage_d, off_d, err_d, pm_d, px_d, pv_d;
  DevBuf pred_d;   // predicted states of all particles (large blocks)
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
                    &S.off_d, &S.err_d, &S.pm_d, &S.px_d, &S.pv_d, &S.pred_d})
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

// pred: scratch of n * PRED doubles.  Blocks of at least n/32 particles
// predict every particle once first (with ~100 neighbours each, the lists
// then name every particle several times); smaller ones predict per listing.
static int launch_firr(int n, const double *rec, double *pred, int lmax, const int *lists,
                       double ti, int ni, const int *addr, int base, double *acc, double *jrk,
                       int *nnbid, int *err, cudaStream_t st) {
  if (ni <= 0) return GPUNB_OK;
  const long long blocks = std::min<long long>((ni + IRR_WARPS - 1) / IRR_WARPS, 1ll << 20);
  if (pred && 32ll * ni >= n) {
    irr_pred_kernel<<<(n + 255) / 256, 256, 0, st>>>(n, rec, ti, pred);
    irr_firr_kernel<true><<<(unsigned)blocks, 32 * IRR_WARPS, 0, st>>>(
        n, rec, pred, lmax, lists, ti, ni, addr, base, acc, jrk, nnbid, err);
  } else {
    irr_firr_kernel<false><<<(unsigned)blocks, 32 * IRR_WARPS, 0, st>>>(
        n, rec, nullptr, lmax, lists, ti, ni, addr, base, acc, jrk, nnbid, err);
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
      !S.list_d.ensure(n * (size_t)lmax * sizeof(int)) || !S.err_d.ensure(sizeof(int)) ||
      !S.err_h.ensure(sizeof(int))) {
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
  IRR_CUDA(cudaMemsetAsync(S.err_d.p, 0, sizeof(int), st), );
  double *pred = nullptr;
  if (32ll * ni >= S.nmax) {
    if (!S.pred_d.ensure((size_t)S.nmax * PRED * sizeof(double))) {
      failf(GPUNB_E_ALLOC, "irr: prediction buffer allocation failed");
      return;
    }
    pred = S.pred_d.as<double>();
  }
  if (S.direct) {
    // address list read, results written in the caller's arrays
    if (launch_firr(S.nmax, S.rec_d.as<double>(), pred, S.lmax, S.list_d.as<int>(), ti, ni,
                    addr, 1, &acc[0][0], &jrk[0][0], nnbid, S.err_d.as<int>(), st) != GPUNB_OK) {
      failf(GPUNB_E_CUDA, "irr: force kernel launch failed");
      return;
    }
  } else {
    if (!S.addr_d.ensure((size_t)ni * sizeof(int)) ||
        !S.out_d.ensure((size_t)ni * 6 * sizeof(double)) ||
        !S.nid_d.ensure((size_t)ni * sizeof(int))) {
      failf(GPUNB_E_ALLOC, "irr: output allocation failed");
      return;
    }
    IRR_CUDA(cudaMemcpyAsync(S.addr_d.p, addr, (size_t)ni * sizeof(int), cudaMemcpyHostToDevice,
                             st), );
    double *o = S.out_d.as<double>();
    if (launch_firr(S.nmax, S.rec_d.as<double>(), pred, S.lmax, S.list_d.as<int>(), ti, ni,
                    S.addr_d.as<int>(), 1, o, o + 3 * (size_t)ni, S.nid_d.as<int>(),
                    S.err_d.as<int>(), st) != GPUNB_OK) {
      failf(GPUNB_E_CUDA, "irr: force kernel launch failed");
      return;
    }
    IRR_CUDA(cudaMemcpyAsync(&acc[0][0], o, (size_t)ni * 3 * sizeof(double),
                             cudaMemcpyDeviceToHost, st), );
    IRR_CUDA(cudaMemcpyAsync(&jrk[0][0], o + 3 * (size_t)ni, (size_t)ni * 3 * sizeof(double),
                             cudaMemcpyDeviceToHost, st), );
    IRR_CUDA(cudaMemcpyAsync(nnbid, S.nid_d.p, (size_t)ni * sizeof(int), cudaMemcpyDeviceToHost,
                             st), );
  }
  int *herr = S.err_h.as<int>();
  IRR_CUDA(cudaMemcpyAsync(herr, S.err_d.p, sizeof(int), cudaMemcpyDeviceToHost, st), );
  IRR_CUDA(cudaStreamSynchronize(st), );
  if (*herr) failf(*herr, "irr_simd_firr_vec_: an address or a listed id is out of range");
  unsigned long long inter = 0;
  for (int k = 0; k < ni; ++k) {
    const int a = addr[k] - 1;
    if (a >= 0 && a < S.nmax) inter += (unsigned long long)S.list_h[(size_t)a * S.lmax];
  }
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
  cudaStream_t st = stream ? (cudaStream_t)stream : S.st;
  return launch_firr(n, rec, nullptr, lmax, lists, ti, ni, addr, 0, acc, jrk, nnbid, nullptr, st);
}

}  // extern "C"
