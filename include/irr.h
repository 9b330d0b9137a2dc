/*
 * irr.h -- C ABI of the irregular (neighbour) force in libgpunb.so.
 *
 * Drop-in replacement for the reference's SIMD irregular-force library
 * src/Main/irr.avx.cpp (and irr.sse.cpp): the same Fortran-mangled entry
 * points (irr.avx.cpp:565-603) with the same arguments, called by
 * src/Main/intgrt.F:175,202-204,545,680,971,1194,1270, fcorr.F:163,
 * ksinit.F:64-66, ksterm.F:466-469, remove_ks.F:87-89, update.F:286,
 * adjust.F:320.  Addresses and neighbour ids are Fortran (1-based) indices;
 * all arrays are caller-owned host memory.
 *
 * Semantics (irr.avx.cpp:162-176, 275-309, 496-560): a particle's state is
 * set with irr_simd_set_jp_ (position X0, velocity X0DOT, F = force/2,
 * FDOT = force derivative/6, mass, time T0) and its neighbour list with
 * irr_simd_set_list_ (LIST(1,I): count, then ids).  irr_simd_firr_vec_
 * predicts each listed particle and the particle itself to time *ti,
 *     x = X0 + dt (X0DOT + dt (F + dt FDOT)),  v = X0DOT + 2 dt (F + 1.5 dt FDOT),
 * and returns the force and its derivative from the neighbours,
 *     acc += m dx / r^3,  jrk += m / r^3 (dv - 3 (dx.dv) / r^2 dx),
 * and nnbid = the Fortran index of the nearest listed neighbour (0 for an
 * empty list).  Precision (irr_set_precision), the prediction in FP64 in
 * every mode: by default double-float arithmetic (hi + lo pairs of floats,
 * error-free transforms) on the FP32 pipe, within ~1e-11 of FP64; FP64
 * throughout; or the reference's own scheme -- double-single positions, FP32
 * velocities, masses and force arithmetic (irr.avx.cpp:58-176), the nearest
 * neighbour taken on the FP32 r^2: the accuracy class of the reference's
 * library (force and derivative within 2e-6 of FP64 at the 99th percentile,
 * within 5e-6 of max(|Q|, S/8) per particle, S the sum of the terms'
 * magnitudes).
 * Deliberate differences: no 600-entry list cap (lmax up to 2^16 per row);
 * a listed body at zero distance (the particle itself) adds nothing instead
 * of a NaN (in the double-float and split modes: any body closer than
 * 1e-19); invalid addresses or ids are reported as GPUNB_E_ARG.  The
 * double-float and split modes hold each term m/r^3 (dv - ...) in the FP32
 * exponent range, below ~3e38: enough for every unregularised pair of an
 * N-body run in its own units (with m ~ 1/N and r >= 1e-10, m/r^3 < 1e30),
 * while pairs closer still, which the integrator regularises, need the FP64
 * mode.
 *
 * set_jp / set_list are safe to call concurrently for different particles
 * (the Fortran callers run them inside OpenMP loops); they only update host
 * mirrors, and the changed entries are uploaded by the next force call.
 */
#ifndef GPUNB_IRR_H
#define GPUNB_IRR_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- reference ABI (irr.avx.cpp:565-603) --------------------------------- */
void irr_simd_open_(int *nmax, int *lmax, int *rank);
void irr_simd_close_(int *rank);
void irr_simd_profile_(int *rank);
void irr_simd_set_jp_(int *addr, double pos[3], double vel[3], double acc2[3], double jrk6[3],
                      double *mass, double *time);
void irr_simd_set_list_(int *addr, int *nblist);
void irr_simd_firr_vec_(double *ti, int *ni, int addr[], double acc[][3], double jrk[][3],
                        int nnbid[]);

/* ---- additions (no reference counterpart) -------------------------------- */
/* Host-array path of the calls above, as gpunb_set_host_path: 1 (default
 * where supported) = the device reads the mirrors and the address list and
 * writes the results in host memory directly, 0 = pinned staging.  Returns
 * the mode in effect, -1 without a device. */
int irr_set_host_path(int mode);

/* Arithmetic of the force: 2 (default) = double-float, 1 = FP64, 0 = split
 * FP32, as above.  Also set at irr_simd_open_ from the environment variable
 * GPUNB_IRR_PRECISION.  Applies to the next force call, host or
 * device-resident form.  Returns the mode in effect. */
int irr_set_precision(int mode);

/* Device-resident form: state and lists already in device memory, 0-based
 * indices, work queued on `stream` (NULL: the library's stream).
 *   rec: n records of 16 doubles {x0[3], m, v0[3], t0, a2[3], 0, j6[3], 0}
 *   lists: n rows of lmax ints, [0] = count, then 0-based ids
 *   addr[ni]: 0-based particles; outputs acc[ni][3], jrk[ni][3], nnbid[ni]
 *   (nnbid is 1-based like the host form, 0 for an empty list).
 * Blocks of at least n/32 particles predict the whole set first into a
 * buffer the library keeps for this form (allocated on first use): calls of
 * this form that overlap on the GPU must be serialised on one stream. */
int irr_firr_device(int n, const double *rec, int lmax, const int *lists, double ti, int ni,
                    const int *addr, double *acc, double *jrk, int *nnbid, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* GPUNB_IRR_H */
