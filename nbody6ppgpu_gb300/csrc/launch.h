// Host-side launchers of the device kernels (one translation unit per kernel
// family; the engine calls only these).
#pragma once
#include <cstddef>
#include <cuda_runtime.h>

#include "regf_kernels.cuh"

namespace gpunb {

struct VariantDesc {
  int ipt, wi, wj;                       // i per thread, warps along i, warps along j
  int jv;                                // j read per shared-memory load (2 or 4)
  int minb;                              // minimum resident blocks (register cap)
  int threads() const { return 32 * wi * wj; }
  int itile() const { return 32 * ipt * wi; }
};

int regf_num_variants();
VariantDesc regf_variant(int v);
size_t regf_ds_smem(int v);
int regf_ds_blocks_per_sm(int v, bool mflag);
cudaError_t launch_pack_jtiles(const double *m, const double *x, const double *v, int nj, const int *perm,
                               float *tiles, int ntile, int *err, cudaStream_t st);
// persistent launch: `grid` blocks drain n_itiles * S work items from `queue`
// (single j-set), or the n_items entries of `items` in `order` (batches).
// out.done (single j-set only) must be queue + 1, with room for n_itiles
// counters: the kernel then merges each i-tile itself into out.acc etc.
cudaError_t launch_regf_ds(int v, bool mflag, int n_itiles, int S, int grid, int *queue,
                           const JSet &js, const ISet &is, const RegfOut &out, cudaStream_t st,
                           const ItemDesc *items = nullptr, const int *order = nullptr,
                           int n_items = 0);
cudaError_t launch_regf_fp64(bool mflag, int gx, int S, const JSet &js, const ISet &is,
                             const RegfOut &out, cudaStream_t st);
// the same call shape in double-float arithmetic (gpunb_set_precision(2))
cudaError_t launch_regf_df(bool mflag, int gx, int S, const JSet &js, const ISet &is,
                             const RegfOut &out, cudaStream_t st);
constexpr int FP64_THREADS = 128;
// ff: the partials are float-float pairs (split kernel), else doubles (FP64 kernel)
cudaError_t launch_regf_merge(const double *part, bool ff, int S, int ni, int ni_pad,
                              const int *perm, const int *cnt, int nnbmax, double *acc,
                              double *jrk, double *pot, int *nnb, int *rowlen, cudaStream_t st);
// batched clusters: tiles[k] = {slot0, nslots, first partial row, number of rows}
cudaError_t launch_regf_merge_batch(const double *part, const int4 *tiles, int ntiles, int itile,
                                    const int *perm, const int *cnt, int nnbmax, double *acc,
                                    double *jrk, double *pot, int *nnb, int *rowlen,
                                    cudaStream_t st);
// FP32 i-records in processing order (NaN check of the i inputs included)
cudaError_t launch_regf_prep(const ISet &is, float4 *rec, int *err, cudaStream_t st);
// scan of rowlen -> off (+ block offsets in btot, grand total at btot[nblocks])
int list_scan_blocks(int ni);
cudaError_t launch_list_scan(const int *rowlen, int ni, int *off, int *btot, cudaStream_t st);
cudaError_t launch_list_gather(int *rows, int cap, const int *rowlen, const int *off,
                               const int *btot, int ni, int *dense, cudaStream_t st);
// rows[i * lmax] = nnb[i], rows[i * lmax + 1 ..] = the i-th compacted sublist
// (offsets as left by launch_list_scan: in-block off + block base boff);
// rows may be host memory the device reaches coherently
cudaError_t launch_list_rows(const int *dense, const int *off, const int *boff, const int *nnb,
                             int ni, int lmax, int *rows, cudaStream_t st);
// up to HOSTCOPY_MAX element copies in one launch, one side of each in host
// memory the device reaches coherently
constexpr int HOSTCOPY_MAX = 4;
struct HostCopyJob {
  const void *src;
  void *dst;
  long long n;   // elements
  int esize;     // 8 or 4 bytes
};
struct HostCopyJobs {
  HostCopyJob j[HOSTCOPY_MAX];
  int count;
};
cudaError_t launch_host_copy(const HostCopyJobs &jobs, cudaStream_t st);
cudaError_t launch_list_finalize_offsets(int *off, const int *btot, int ni, cudaStream_t st);

// spatial (Morton) ordering
size_t order_temp_bytes(int n);
// bounding-box buffer: [0..6) the box, [BBOX_TICKET] the last-block ticket
// (zero between launches), [BBOX_PART..) the per-block partial boxes
constexpr int BBOX_THREADS = 256;
constexpr int BBOX_MAX_BLOCKS = 256;
constexpr int BBOX_TICKET = 7;
constexpr int BBOX_PART = 8;
constexpr int BBOX_INTS = BBOX_PART + 6 * BBOX_MAX_BLOCKS;
cudaError_t launch_bbox(const double *x, int n, int *bb, cudaStream_t st);
cudaError_t launch_order(const double *x, int n, const int *bb, unsigned long long *keys,
                         unsigned long long *keys_alt, int *vals_alt, int *perm, void *temp,
                         size_t temp_bytes, cudaStream_t st);

// batched sets: order each set (off[nset+1] boundaries) along the Morton
// curve and place set c at slots slot_off[c].. of perm (other slots -1)
size_t order_batch_temp_bytes(int n, int nset);
cudaError_t launch_order_batch(const double *x, int n, const int *bb, const int *off, int nset,
                               const int *slot_off, int nslots, unsigned long long *keys,
                               unsigned long long *keys_alt, int *vals_alt, int *sorted,
                               int *perm, void *temp, size_t temp_bytes, cudaStream_t st);

// potential
constexpr int POT_JT = 128;
constexpr int POT_TILE_FLOATS = 7 * POT_JT;
cudaError_t launch_pack_pot(const double *m, const double *x, int n, float *tiles, int ntile,
                            int *err, cudaStream_t st);
int pot_itile();
cudaError_t launch_pot(const float *tiles, int ntile, const double *x, int istart0, int ni,
                       int gx, int S, double *part, int ni_pad, int *err, cudaStream_t st);
int pot_blocks_per_sm();
// err (may be null): the call's device error word; nonzero -> every pot[i] = NaN
cudaError_t launch_pot_merge(const double *part, int S, int ni, int ni_pad, const int *err,
                             double *pot, cudaStream_t st, const int *iorder = nullptr);
// potential on the regular force's Morton-ordered tiles (pack_jtiles with
// v = null); slot s of the i-range is the i-particle istart0 + iorder[s]
int pot_rel_blocks_per_sm();
cudaError_t launch_pot_rel(const float *tiles, int ntile, const double *x, const int *iorder,
                           int istart0, int ni, int gx, int S, double *part, int ni_pad, int *err,
                           cudaStream_t st);

}  // namespace gpunb
