/*
 * gpunb.h -- C ABI of libgpunb.so, the GB300 (sm_103a) regular-force library.
 *
 * Drop-in replacement for the reference's regular-force back-ends.  The first
 * block of entry points keeps the exact Fortran-mangled names, argument
 * meaning and in-band conventions that NBODY6++'s Fortran host code calls
 * (src/Main/fpoly0.F:31,76,125; intgrt.F:168,918,1497; util_gpu.F:60;
 * adjust.F:315,424; energy.F:38), so the Fortran side links against this
 * library unchanged.  All array arguments are caller-owned HOST memory:
 *   xj/vj/xi/vi/acc/jrk are C double[n][3] (Fortran X(3,N) column-major),
 *   list is Fortran LISTGP(LMAX,NI): row i at list + i*lmax,
 *   list[i*lmax] = count, list[i*lmax+1 .. count] = 0-based j indices into the
 *   array given to gpunb_send_, ascending, the i-particle itself included;
 *   count > nnbmax is reported as -count (entries undefined).
 * Errors: the reference aborts through assert(); this library prints the
 * reason and calls abort() by default too, or, after
 * gpunb_set_abort_on_error(0), records the code for gpunb_last_error().
 */
#ifndef GPUNB_GB300_H
#define GPUNB_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- reference ABI ----------------------------------------------------- */

/* Select and initialise the device (reference: GPUNB_devinit,
 * src/Main/gpunb.velocity.cu:574-626, export :905-907).  GPU_LIST picks the
 * device (its first entry; one GPU per process). */
void gpunb_devinit_(int *irank);

/* Open the library for up to *nbmax j-particles (reference: GPUNB_open,
 * gpunb.velocity.cu:628-666, export :908-910). */
void gpunb_open_(int *nbmax, int *irank);

/* Release device buffers (reference: GPUNB_close, gpunb.velocity.cu:668-701,
 * export :911-913). */
void gpunb_close_(void);

/* Upload the j-set: nj bodies, masses mj[nj], positions xj[nj][3], velocities
 * vj[nj][3] (FP64, already predicted to the current time) (reference:
 * GPUNB_send, gpunb.velocity.cu:703-729, export :914-920). */
void gpunb_send_(int *nj, double mj[], double xj[][3], double vj[][3]);

/* Regular force, jerk, potential and neighbour lists of *ni i-particles
 * against the whole j-set (reference: GPUNB_regf, gpunb.velocity.cu:731-880,
 * export :921-935; CPU variant src/Main/reg.avx.cpp:185-331).
 *   h2[i]  neighbour radius squared (RS**2, or RS**2/BODYM when *m_flag)
 *   dtr[i] regular step for the predicted-distance criterion
 *   neighbour iff min(r2, |dx + dtr dv|^2) < h2 (< m_j h2 when *m_flag);
 *   neighbours are excluded from acc, jrk and pot; pot is +sum m/r.
 * Differences from the reference, all in the direction of fewer limits:
 * no NIMAX cap on ni, no 2^21 cap on the total list length, no per-j-block
 * 256 cap; overflow is count > nnbmax only. */
void gpunb_regf_(int *ni, double h2[], double dtr[], double xi[][3], double vi[][3],
                 double acc[][3], double jrk[][3], double pot[], int *lmax, int *nnbmax,
                 int *list, int *m_flag);

/* Print and reset the call counters in the reference's format
 * (reference: GPUNB_profile, gpunb.velocity.cu:882-902, export :936-938). */
void gpunb_profile_(int *irank);

/* Potential for the energy check: pot[k] = sum_{j: r2 > 0} m_j / r_ij for
 * i = istart-1+k, k < ni, over n bodies (reference: gpupot_,
 * src/Main/gpupot.gpu.cu:61-127; CPU src/Main/pot.avx.cpp:72-159).  Bodies
 * closer than 1e-19 (r2 below 2^-126) count as coincident. */
void gpupot_(int *irank, int *istart, int *ni, int *n, double m[], double x[][3],
             double pot[]);

/* ---- additions of this library (no reference counterpart) -------------- */

/* Error codes (0 = none). */
enum {
  GPUNB_OK = 0, GPUNB_E_NOT_OPEN = 1, GPUNB_E_ARG = 2, GPUNB_E_NAN = 3,
  GPUNB_E_CUDA = 4, GPUNB_E_CAPACITY = 5, GPUNB_E_TIMEOUT = 6,
  GPUNB_E_NO_DEVICE = 7, GPUNB_E_ALLOC = 8
};
int gpunb_last_error(void);                 /* code of the first error since clear */
const char *gpunb_last_error_message(void); /* text of that error */
void gpunb_clear_error(void);
void gpunb_set_abort_on_error(int flag);    /* 1 (default): print + abort() */

/* Pair kernel selection: 0 = split precision (FP32 arithmetic on double-single
 * positions, float-float merges and FP64 neighbour re-tests; default),
 * 1 = plain FP64, 2 = double-float (every pair in hi + lo pairs of floats on
 * the FP32 pipe: FP64-class results, within ~1e-11 of FP64, several times
 * faster than FP64 on GB300; lists identical to FP64).  The batched entry
 * points always use the split kernel.  gpunb_open_ resets the mode to the
 * environment variable GPUNB_PRECISION (0 when unset). */
void gpunb_set_precision(int mode);

/* Force a launch shape (variant index, j-splits; for the batched entry
 * points, work items per resident block instead of j-splits); -1/0 restores
 * the autotuned or heuristic choice.  gpunb_num_variants() lists the shapes. */
void gpunb_set_launch(int variant, int splits);
int gpunb_num_variants(void);
int gpunb_variant_info(int variant, int *ipt, int *warps_i, int *warps_j);

/* How gpunb_send_/gpunb_regf_ move the caller's host arrays (no reference
 * counterpart).  mode 1 (the default where supported): copy straight from and
 * to the caller's pageable arrays and let the device write the LISTGP rows,
 * which needs a device that reads pageable memory coherently through the
 * host's page tables (Grace + Blackwell over NVLink-C2C); the environment
 * variable GPUNB_HOST_DIRECT=0 turns it off at start-up.  mode 0: stage
 * through pinned buffers and scatter the rows on the host.  Returns the mode
 * in effect, or -1 without a device.  Results are identical in both modes. */
int gpunb_set_host_path(int mode);

/* Ordering of the j-set (no reference counterpart).  Every send packs the
 * bodies into tiles that follow a Morton order; the order itself (bounding
 * box, keys, radix sort) is recomputed when nj changes and on every
 * `every`-th send (default 8, or the environment variable
 * GPUNB_RESORT_EVERY), and the sends between reuse it with the tiles re-packed
 * from the current positions.  Results do not depend on the order; only the
 * tiles' spatial coherence, and with it the speed, would decay if bodies
 * travelled far between re-orderings.  1 re-orders on every send.  The next
 * send after this call re-orders.  Returns the previous interval;
 * gpunb_sort_count returns the number of re-orderings so far. */
int gpunb_set_resort_interval(int every);
long long gpunb_sort_count(void);

/* Autotuner.  With gpunb_set_autotune(1) (or the environment variable
 * GPUNB_AUTOTUNE=1 at start-up) the first regf call of an (N, ni)
 * half-octave bucket -- gpunb_regf_, gpunb_regf_device, or a batched call's
 * (total bodies, total active) bucket -- times every launch shape (kernel
 * variant: i-particles per thread, warps along i and j, j per warp vote; and
 * the j-split count, or for batches the work items per resident block) on
 * that call's own active block, caches the fastest and uses it from then on;
 * later calls of the bucket read the cache.  Returns the previous setting.
 * gpunb_autotune tunes the bucket of ni ahead of any call, on synthetic
 * i-particles drawn from the current j-set; returns the chosen variant and
 * *splits, *ms. */
int gpunb_set_autotune(int flag);
int gpunb_autotune(int ni, int m_flag, int *splits, float *ms);
/* Save the tuning cache to a text file / replace the cache with a saved
 * one; return the number of entries, or -1 when the file cannot be opened
 * (the cache is then unchanged). */
int gpunb_tune_load(const char *path);
int gpunb_tune_save(const char *path);

/* Time the pair kernel of each subsequent regf call with a pair of CUDA events
 * recorded on the stream it is launched on.  gpunb_kernel_times() waits for
 * the recorded launches, writes up to max durations (ms) in launch order,
 * returns their number and starts a new record; gpunb_last_kernel_ms()
 * returns the last duration read. */
void gpunb_set_timing(int flag);
int gpunb_kernel_times(float *ms, int max);
float gpunb_last_kernel_ms(void);
/* Launch shape used by the last regf call. */
void gpunb_last_launch(int *variant, int *splits, int *grid_x);

/* Device-resident variants: all pointers are device memory, work is queued
 * on `stream` (a cudaStream_t; NULL = the library's stream) and nothing is
 * copied to the host.  regf writes acc[ni][3], jrk[ni][3], pot[ni], nnb[ni]
 * (count or -count), list_off[ni+1] (offsets of accepted rows in list) and
 * list[...] (capacity list_cap ints; ni*nnbmax always suffices). */
int gpunb_send_device(int nj, const double *m, const double *x, const double *v, void *stream);
/* Device-side errors of the device entry points (a NaN input, an exhausted
 * wait) are raised by the kernels into the library's error word, which
 * these calls do not read back.  gpunb_device_status synchronises `stream`
 * (NULL: the library's stream), returns that word (0 or a GPUNB_E_* code),
 * records a nonzero code as the calls on host arrays do, and clears the
 * word.  The host-array calls clear it when they start. */
int gpunb_device_status(void *stream);

/* Test support for the failure paths (no reference counterpart; neither
 * faults nor hangs the device).  gpunb_test_bounded_wait queues one thread
 * that waits, at most `polls` polls, on an mbarrier that nothing completes,
 * then records GPUNB_E_TIMEOUT in the device error word as the library's
 * kernels do when a bounded wait gives up (read it with
 * gpunb_device_status); the context stays usable.  gpunb_test_fail_allocs
 * makes the next n device-buffer allocations of the regular-force library
 * state report GPUNB_E_ALLOC. */
int gpunb_test_bounded_wait(int polls, void *stream);
void gpunb_test_fail_allocs(int n);
int gpunb_regf_device(int ni, const double *h2, const double *dtr, const double *xi,
                      const double *vi, double *acc, double *jrk, double *pot, int *nnb,
                      int *list_off, int *list, size_t list_cap, int nnbmax, int m_flag,
                      void *stream);

/* Batched clusters (no reference counterpart): ncl independent j-sets, each
 * with its own active block, served by one persistent launch.  nj[] and ni[]
 * are host arrays of ncl counts; all other pointers are device memory with
 * the sets concatenated in order (m, x, v of all j-sets; h2, dtr, xi, vi and
 * the outputs of all active blocks).  Each active block interacts with its
 * own set only; neighbour ids are 0-based within the particle's own set;
 * nnb/list_off/list are per concatenated i as in gpunb_regf_device.  The
 * j-data are copied, so the inputs may change after the send. */
int gpunb_batch_send_device(int ncl, const int *nj, const double *m, const double *x,
                            const double *v, void *stream);
int gpunb_batch_regf_device(int ncl, const int *ni, const double *h2, const double *dtr,
                            const double *xi, const double *vi, double *acc, double *jrk,
                            double *pot, int *nnb, int *list_off, int *list, size_t list_cap,
                            int nnbmax, int m_flag, void *stream);
/* Launch plan of the last batched call: kernel variant and work items. */
int gpunb_batch_last_plan(int *variant, int *items);

/* CUDA graphs: with flag = 1, the first call of a shape (sizes, active
 * counts, caller pointers, stream, launch plan) runs normally and is then
 * captured; later calls of that shape replay the graph while no library
 * buffer has moved.  Covers gpunb_send_device, gpunb_regf_device, the batched
 * pair, and gpunb_send_ / gpunb_regf_ where the device reads host memory
 * directly (gpunb_set_host_path).  Calls made with per-launch timing on
 * (gpunb_set_timing) run without graphs.  Default 0, or the value of the
 * environment variable GPUNB_GRAPHS. */
void gpunb_set_graphs(int flag);

/* Potential of gpupot_ for callers that cannot allocate device memory (no
 * counterpart in the reference).  Meant for host programs that must not call
 * cudaMalloc: one whose own caching allocator already holds the free device
 * memory (cudaMalloc would fail), or a step loop that cannot afford the
 * device-wide synchronisation of cudaFree.  All pointers are device memory
 * (m[n], x[n][3], pot[ni]); work is queued on `stream` (a cudaStream_t).  The
 * scratch is a fixed 4 MiB array in the library image, present on every GPU
 * that loads the library; the call allocates nothing.  Limits: 1 <= n <=
 * 65536, 1 <= istart, istart-1+ni <= n; anything else returns GPUNB_E_ARG
 * without launching.  The first call on a device looks up the array's device
 * address.  The call waits for its own work on `stream` and returns 0 or an
 * error code, including the codes its kernels raise (GPUNB_E_NAN for a NaN
 * input, GPUNB_E_TIMEOUT for a bounded wait that gave up); with such a code
 * every pot[k] is NaN.  Calls share the scratch: calls that overlap on the
 * GPU race, so serialise them on one stream. */
int gpupot_device_noalloc(int istart, int ni, int n, const double *m, const double *x,
                          double *pot, void *stream);

/* Measured FP32 throughput of this device (no reference counterpart): a
 * kernel of independent packed f32x2 FMA chains, the instruction of the pair
 * loop; *tflops = achieved FP32 TFLOP/s, *ms = its duration.  The roofline
 * denominator of the regular-force kernel. */
int gpunb_fp32_peak(float *tflops, float *ms);

/* Predict-and-send (no reference counterpart; replaces the host prediction
 * of src/Main/xbpredall.f:16-27 followed by GPUNB_SEND at intgrt.F:916-918).
 * Predicts bodies *ifirst .. *ntot (1-based) to *time from the state stored
 * with irr_simd_set_jp_ (include/irr.h: X0, X0DOT, F, FDOT, T0), returns
 * X and XDOT of those bodies in x[ntot-ifirst+1][3], xdot[...] (the values
 * xbpredall would compute, for the caller's other uses) and uploads them with
 * the masses body[ntot-ifirst+1] as the regular-force j-set, as
 * gpunb_send_(NN, BODY(IFIRST), X(1,IFIRST), XDOT(1,IFIRST)) would: the j-set
 * never crosses to the host and back.  Needs irr_simd_open_ with nmax >= ntot
 * and gpunb_open_.  KS components (KSRES2 in xbpredall) stay with the caller. */
void gpunb_send_predicted_(int *ifirst, int *ntot, double *time, double body[], double x[][3],
                           double xdot[][3]);

/* ---- Learned neighbour-radius predictor (no reference counterpart) --------
 * An 8 -> 64 -> 64 -> 1 GELU MLP that proposes each active particle's next
 * RS in place of the plain rule of src/Main/regcor_gpu.F:146-253; the caller
 * falls back to that rule (and to the overflow rule of
 * src/Main/util_gpu.F:81-97) whenever the proposal is rejected.  It never
 * touches forces.  Parameters: P floats (gpunb_rsmlp_num_params) in the order
 * W1[64][8] | b1[64] | W2[64][64] | b2[64] | W3[64] | b3, held as an FP32
 * master copy `wf` and a BF16 copy `wq` (P x 2 bytes) of the same order; the
 * kernels read matrices from `wq`, biases from `wf`, and accumulate in FP32.
 * All pointers are device pointers; calls are asynchronous on `stream`. */
int gpunb_rsmlp_num_params(void);
/* wq <- bf16(wf) */
int gpunb_rsmlp_to_bf16(const float *wf, void *wq, void *stream);
/* y[B] <- MLP(X[B][8]) */
int gpunb_rsmlp_forward(int B, const float *X, const void *wq, const float *wf, float *y,
                        void *stream);
/* grad[P] <- d/dparams of loss = (1/B) sum_b W[b] (y_b - T[b])^2 (W may be NULL
 * for unit weights); loss[1] <- that loss.  `part` is scratch of
 * ceil(B/128) * (P + 1) floats.  The reduction order is fixed: repeated calls
 * give bit-identical gradients. */
int gpunb_rsmlp_backward(int B, const float *X, const float *T, const float *W, const void *wq,
                         const float *wf, float *grad, float *loss, float *part, void *stream);
/* One Adam step on the FP32 master (bias-corrected, step >= 1), then
 * wq <- bf16(wf). */
int gpunb_rsmlp_adam(float *wf, float *m1, float *m2, const float *grad, float lr, float beta1,
                     float beta2, float eps, int step, void *wq, void *stream);

/* Training labels of the predictor on the device.  For particle i < ni
 * (position xi, velocity vi, regular step dtr[i], target membership k[i] >=
 * 1): logr[i] = log R_i with R_i^2 the geometric mean of the k-th and
 * (k+1)-th smallest keys min(|dx|^2, |dx + dtr dv|^2) over the j-set xj, vj
 * (the body itself first, key 0) -- the radius at which the regular force's
 * own membership test admits exactly k[i] bodies besides i.  The keys are
 * read from rows of the library's neighbour list taken at an enlarged radius
 * (list_off, list, nnb as written by gpunb_regf_device, ids into xj/vj):
 * ok[i] = 1 when the row held at least k[i] + 2 members (the label is then
 * exact), 0 when it held fewer and -1 when it overflowed or held more than
 * 1024 (retry those rows with a larger / smaller radius).  Device pointers,
 * asynchronous on `stream`. */
int gpunb_rsmlp_label_device(int ni, const int *list_off, const int *list, const int *nnb,
                             const double *xj, const double *vj, const double *xi,
                             const double *vi, const double *dtr, const int *k, double *logr,
                             int *ok, void *stream);

/* RS update of an active block on the device (no reference counterpart: the
 * reference runs src/Main/regcor_gpu.F:120-253 on the host, one particle at a
 * time).  Plain rule as regcor_gpu.F (with the few-member rule of
 * fpoly0.F:153-158 for counts below 2 when few_nb_rule), and, when wq is not
 * NULL, the MLP proposal from the 8 features of each particle normalised by
 * norm[0..7] (mean) and norm[8..15] (spread), taken where its count stays
 * within [band_lo, band_hi] x the rule's target (0.5-1.5 when the fields are
 * 0).  The count of a proposed radius R' is the count at the current
 * density, (nnb + 1)(R'/RS)^3 - 1, or, when the block's neighbour rows are
 * given (list_off != NULL), the larger of that and an estimate at the next
 * regular step: the members j of row i (list[list_off[i] .. list_off[i+1]),
 * indices into xj/vj, the j-set the rows were computed on, e.g. the CSR output
 * of gpunb_regf_device) with min(|d|^2, |d + dtr dv|^2) < R'^2,
 * d = dx + dtr dv (the kernel's membership test one step later, separations
 * moved on the current relative velocity), plus, when R' > RS, the members x
 * ((R'/RS)^3 - 1); a member with the particle's own position and velocity is
 * the particle itself and is skipped.  Inputs per
 * active particle i < ni: x, v ([ni][3]), m_scaled (mass x N), rs, nnb (count,
 * self excluded), nnb0 (previous count), acc, jrk ([ni][3], regular force and
 * derivative; only read with wq), dtr.  Outputs rs_new[ni], and when not NULL
 * target[ni] (the rule's membership target) and used[ni] (1: MLP value).
 * All pointers are device memory (p is a host struct). */
typedef struct {
  int nnbopt, nnbmax;       /* NNBOPT, NNBMAX */
  int nb_flag;              /* 1: KZ(39) = 0 or 2 (distances from the density centre) */
  int few_nb_rule;          /* 1: counts below 2 take 1.5 RS (fpoly0.F:153-158) */
  double rscale, rc, rsfac; /* RSCALE, RC, RSFAC */
  double bodym;             /* mean mass */
  double rdens[3];          /* density centre RDENS */
  double band_lo, band_hi;  /* acceptance band of the MLP proposal (0: 0.5, 1.5) */
  const int *list_off;      /* neighbour rows for the band check (device), or NULL */
  const int *list;
  const double *xj, *vj;    /* positions, velocities of the j-set the rows index */
} gpunb_rs_params;
int gpunb_rs_update_device(int ni, const gpunb_rs_params *p, const double *x, const double *v,
                           const double *m_scaled, const double *rs, const int *nnb,
                           const int *nnb0, const double *acc, const double *jrk,
                           const double *dtr, const void *wq, const float *wf,
                           const float *norm, double *rs_new, double *target, int *used,
                           void *stream);

/* Regular corrector of an active block on the device (no reference
 * counterpart as an entry point: it does, for every body of the block at
 * once, the work of src/Main/regcor_gpu.F REGCOR_GPU, which the reference
 * runs on the host body by body).  For body I = iact[k] (1-based), with its
 * new regular force freg[k][3], derivative fdr[k][3] and new neighbour row
 * nlist[k*lmax ..] (count, then ascending 1-based body indices, self
 * removed): the RS rule with the c.m.-body and <= 3-neighbour branches
 * (:120-252), the small-central-mass change for an empty list (:120-143), the
 * force changes of lost and gained neighbours with the retention of old
 * neighbours whose step is below SMIN (:262-460; a retained body is inserted
 * into nlist and the row count updated; into an empty list as into any
 * other, where the reference's insertion loop displaces the first kept body
 * by the saved last old member), the Hermite corrector (:462-552:
 * XN, XNDOT, FI, FR, FIDOT, FRDOT, D0, D0R..D3R, T0R; tidal FIDOT term for
 * KZ(14) <= 2), the list copy LIST(.,I) = NLIST on a change (:608-616), the
 * new regular step STEPR and the irregular step reduction (:618-800).  Not
 * done here: XTRNLF, FCLOUD, CHECKL, FPCORR and the tidal energy ETIDE.
 * All state arrays are device memory in the Fortran COMMON layout of all
 * NTOT bodies (index I-1; vectors as [NTOT][3]); list is LIST(LMAX,NTOT)
 * as [NTOT][lmax] with 1-based members.  The active bodies must be distinct;
 * the small-step tests read the neighbours' STEP as it was when the call
 * started (the reference's OpenMP loop leaves open whether a neighbour in
 * the same block has already changed its own).  Asynchronous on `stream`;
 * returns 0, GPUNB_E_ARG or GPUNB_E_ALLOC (a grow-only scratch of ni doubles
 * for the new steps). */
typedef struct {
  double time;              /* TIME */
  double dtmin, smin, smax; /* DTMIN, SMIN, SMAX */
  double etar;              /* ETAR */
  double tidal4;            /* TIDAL(4) */
  int kz14;                 /* KZ(14) */
  int m_flag;               /* 1: mass-weighted neighbour criterion (KZ(39) = 2, 3) */
  int nnbmax;               /* NNBMAX */
  int n;                    /* N: single bodies 1..N, c.m. bodies N+1..NTOT */
  int ntot;                 /* NTOT */
  int ifirst;               /* IFIRST */
  int lmax;                 /* row stride of list and nlist */
  gpunb_rs_params rs;       /* NNBOPT, NNBMAX, RSCALE, RC, RSFAC, BODYM, RDENS, NB_FLAG */
} gpunb_regcor_params;
typedef struct {
  const double *x, *xdot;         /* X, XDOT predicted to TIME */
  const double *body;             /* BODY */
  const double *h;                /* H(IPAIR) of the KS pairs (c.m. branch); may be NULL */
  const double *x0, *x0dot;       /* X0, X0DOT */
  double *t0r, *stepr, *step, *t0, *timenw;
  double *fi, *fidot, *fr, *frdot;
  double *d0, *d0r, *d1r, *d2r, *d3r;
  double *xn, *xndot;             /* XN, XNDOT */
  double *rs;                     /* RS */
  int *list;                      /* LIST */
  int *counters;                  /* NBVOID, NBSMIN, NBFLUX, NICONV increments; may be NULL */
} gpunb_regcor_state;
int gpunb_regcor_device(int ni, const int *iact, const double *freg, const double *fdr,
                        int *nlist, const gpunb_regcor_params *p, const gpunb_regcor_state *s,
                        void *stream);

#ifdef __cplusplus
}
#endif
#endif /* GPUNB_GB300_H */
