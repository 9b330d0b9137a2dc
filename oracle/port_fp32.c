/*
 * Portable FP32 restatement of the reference's CPU regular-force and potential
 * path (src/Main/reg.avx.cpp:137-331, src/Main/pot.avx.cpp:46-146).
 * TEST INFRASTRUCTURE ONLY: it is the CPU baseline (bench.py's cpu_baseline
 * and --impl reference legs) on hosts where the x86-only AVX source cannot be
 * compiled, and a second FP32 check in the CPU tests.  The product never links
 * or calls it.  Compiled with FP contraction allowed (the AVX build contracts
 * too), unlike the FP64 oracle in oracle_fp64.c.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------ */
/* Portable FP32 restatement of reg.avx.cpp (CPU baseline "port").           */
/* The pair loop has the reference's shape (reg.avx.cpp:204-329): a vector of
 * i-particles (4 per 128-bit NEON vector on aarch64, 8 per 256-bit AVX vector
 * on x86 hosts built with -mavx -mfma; the reference packs 4 i x 2 j into one
 * 8-lane AVX vector) meets one j at a time, broadcast to every lane; the
 * reciprocal square root is a hardware estimate refined by Newton steps, the
 * neighbours are masked out of the sums with an and-not of the comparison,
 * and the lanes' neighbour bits are inspected once per 4 j.  GCC vector
 * extensions keep the source portable; the only target-specific parts are
 * the estimate and the any-lane test. */

#if defined(__aarch64__)
#include <arm_neon.h>
#define PORT_VW 4
#elif defined(__AVX__)
#define PORT_VW 8
#else
#define PORT_VW 4
#endif
typedef float vf __attribute__((vector_size(4 * PORT_VW)));
typedef int32_t vi __attribute__((vector_size(4 * PORT_VW)));

/* 1/sqrt(x) per lane, to FP32 rounding level (the role of v8sf_rsqrt,
 * reg.avx.cpp:74-77: hardware estimate + one Newton step).  aarch64: the
 * FRSQRTE estimate (about 8 bits) and two Newton steps with FRSQRTS, which
 * computes (3 - a b) / 2 in one instruction.  Elsewhere: the bit-level
 * estimate with the modified first iteration of Moroz, Walczyk, Hrynchyshyn,
 * Holimath and Cieslinski ("Fast calculation of inverse square root with the
 * use of magic constant - analytical approach", Appl. Math. Comput. 316,
 * 2018: magic 0x5f1ffff9, y1 = 0.703952253 y0 (2.38924456 - x y0^2), relative
 * error < 6.5e-4), then one ordinary Newton step (< 1e-6). */
static inline vf v_rsqrt(vf x)
{
#if defined(__aarch64__)
    const float32x4_t xx = (float32x4_t)x;
    float32x4_t y = vrsqrteq_f32(xx);
    y = vmulq_f32(y, vrsqrtsq_f32(vmulq_f32(xx, y), y));
    y = vmulq_f32(y, vrsqrtsq_f32(vmulq_f32(xx, y), y));
    return (vf)y;
#else
    const vi i = 0x5f1ffff9 - (((vi)x) >> 1);
    vf y = (vf)i;
    y = (0.703952253f * y) * (2.38924456f - x * y * y);
    return (-0.5f * y) * (x * y * y - 3.0f);
#endif
}

static inline int v_any(vi m)
{
#if defined(__aarch64__)
    return vmaxvq_u32((uint32x4_t)m) != 0;
#else
    int r = 0;
    for (int k = 0; k < PORT_VW; k++) r |= m[k];
    return r != 0;
#endif
}

static inline vf v_zero(void)
{
    const vf z = {0};
    return z;
}

static float *port_j = NULL;      /* 7 arrays of port_cap: x y z m vx vy vz */
static int port_nbody = 0, port_cap = 0;

/* scalar reciprocal square root for the potential port: the published
 * bit-level estimate (C. Lomont, "Fast inverse square root", 2003) refined
 * by three Newton steps to FP32 rounding level; finite for x = 0. */
static inline float port_rsqrt(float x)
{
    uint32_t i;
    memcpy(&i, &x, sizeof(i));
    i = 0x5f375a86u - (i >> 1);
    float y;
    memcpy(&y, &i, sizeof(y));
    y = (-0.5f * y) * (x * y * y - 3.0f);
    y = (-0.5f * y) * (x * y * y - 3.0f);
    return (-0.5f * y) * (x * y * y - 3.0f);
}

/* GPUNB_send of reg.avx.cpp:137-160: FP64 -> FP32, padded to a multiple of
 * 4 bodies with massless bodies far away (the reference pads to an even
 * count: it reads two j per vector). */
void port_send_fp32(int nj, const double *mj, const double (*xj)[3],
                    const double (*vj)[3])
{
    if (nj + 4 > port_cap) {
        free(port_j);
        port_cap = nj + 4;
        port_j = (float *)malloc(sizeof(float) * 7 * (size_t)port_cap);
    }
    float *X = port_j, *Y = X + port_cap, *Z = Y + port_cap, *M = Z + port_cap;
    float *VX = M + port_cap, *VY = VX + port_cap, *VZ = VY + port_cap;
#pragma omp parallel for
    for (int j = 0; j < nj; j++) {
        X[j] = (float)xj[j][0]; Y[j] = (float)xj[j][1]; Z[j] = (float)xj[j][2];
        M[j] = (float)mj[j];
        VX[j] = (float)vj[j][0]; VY[j] = (float)vj[j][1]; VZ[j] = (float)vj[j][2];
    }
    port_nbody = nj;
    while (port_nbody % 4) {
        const int j = port_nbody++;
        X[j] = Y[j] = Z[j] = 255.0f;
        M[j] = VX[j] = VY[j] = VZ[j] = 0.0f;
    }
}

void port_free_fp32(void)
{
    free(port_j);
    port_j = NULL;
    port_cap = port_nbody = 0;
}

/* GPUNB_regf of reg.avx.cpp:185-331: PORT_VW i-particles per vector against
 * every j, FP32 pair arithmetic, per-lane FP32 sums, FP64 results; neighbour
 * lists ascending per i, -count on overflow (reg.avx.cpp:316-328). */
void port_regf_fp32(int ni, const double *h2d, const double *dtrd,
                    const double (*xid)[3], const double (*vid)[3],
                    double (*acc)[3], double (*jrk)[3], double *pot, int lmax,
                    int nbmax, int *list, int m_flag)
{
    const int nj = port_nbody, cap = port_cap;
    const float *X = port_j, *Y = X + cap, *Z = Y + cap, *M = Z + cap;
    const float *VX = M + cap, *VY = VX + cap, *VZ = VY + cap;
#pragma omp parallel
    {
        int *nbl = (int *)malloc(sizeof(int) * (size_t)PORT_VW * (size_t)(nj + 4));
#pragma omp for schedule(dynamic, 1)
        for (int i0 = 0; i0 < ni; i0 += PORT_VW) {
            const int nii = (ni - i0 < PORT_VW) ? ni - i0 : PORT_VW;
            vf xi, yi, zi, vxi, vyi, vzi, h2i, dtri;
            for (int k = 0; k < PORT_VW; k++) {
                /* missing lanes repeat the last i with h2 = 0 (no neighbours) */
                const int i = i0 + (k < nii ? k : nii - 1);
                xi[k] = (float)xid[i][0]; yi[k] = (float)xid[i][1]; zi[k] = (float)xid[i][2];
                vxi[k] = (float)vid[i][0]; vyi[k] = (float)vid[i][1]; vzi[k] = (float)vid[i][2];
                h2i[k] = k < nii ? (float)h2d[i] : 0.0f;
                dtri[k] = (float)dtrd[i];
            }
            vf ax = v_zero(), ay = ax, az = ax, jx = ax, jy = ax, jz = ax, po = ax;
            int nnb[PORT_VW] = {0};
            for (int j0 = 0; j0 < nj; j0 += 4) {
                vi many = (vi)v_zero();
#pragma GCC unroll 4
                for (int u = 0; u < 4; u++) {
                    const int j = j0 + u;
                    /* a scalar operand is broadcast to every lane */
                    const float mj = M[j];
                    const vf dx = X[j] - xi, dy = Y[j] - yi, dz = Z[j] - zi;
                    const vf dvx = VX[j] - vxi, dvy = VY[j] - vyi, dvz = VZ[j] - vzi;
                    const vf dxp = dx + dtri * dvx, dyp = dy + dtri * dvy, dzp = dz + dtri * dvz;
                    const vf r2 = dx * dx + dy * dy + dz * dz;
                    vf rv = dx * dvx + dy * dvy + dz * dvz;
                    const vf r2p = dxp * dxp + dyp * dyp + dzp * dzp;
                    const vi lt = r2 < r2p;
                    const vf r2min = (vf)((lt & (vi)r2) | (~lt & (vi)r2p));
                    const vf crit = m_flag ? mj * h2i : h2i;
                    const vi in = r2min < crit;
                    many |= in;
                    vf rinv1 = (vf)(~in & (vi)v_rsqrt(r2));
                    const vf rinv2 = rinv1 * rinv1;
                    rinv1 *= mj;
                    po += rinv1;
                    const vf rinv3 = rinv1 * rinv2;
                    rv *= -3.0f * rinv2;
                    ax += rinv3 * dx; ay += rinv3 * dy; az += rinv3 * dz;
                    jx += rinv3 * (dvx + rv * dx);
                    jy += rinv3 * (dvy + rv * dy);
                    jz += rinv3 * (dvz + rv * dz);
                }
                if (v_any(many)) {
                    /* rare: redo the test of these 4 j (the same arithmetic,
                     * so the same decisions) and record the neighbours */
                    for (int u = 0; u < 4; u++) {
                        const int j = j0 + u;
                        const float mj = M[j];
                        const vf dx = X[j] - xi, dy = Y[j] - yi, dz = Z[j] - zi;
                        const vf dvx = VX[j] - vxi, dvy = VY[j] - vyi, dvz = VZ[j] - vzi;
                        const vf dxp = dx + dtri * dvx, dyp = dy + dtri * dvy,
                                 dzp = dz + dtri * dvz;
                        const vf r2 = dx * dx + dy * dy + dz * dz;
                        const vf r2p = dxp * dxp + dyp * dyp + dzp * dzp;
                        const vi lt = r2 < r2p;
                        const vf r2min = (vf)((lt & (vi)r2) | (~lt & (vi)r2p));
                        const vf crit = m_flag ? mj * h2i : h2i;
                        const vi in = r2min < crit;
                        for (int k = 0; k < PORT_VW; k++)
                            if (in[k]) nbl[(size_t)k * (nj + 4) + nnb[k]++] = j;
                    }
                }
            }
            for (int k = 0; k < nii; k++) {
                const int i = i0 + k;
                acc[i][0] = ax[k]; acc[i][1] = ay[k]; acc[i][2] = az[k];
                jrk[i][0] = jx[k]; jrk[i][1] = jy[k]; jrk[i][2] = jz[k];
                pot[i] = po[k];
                int *row = list + (size_t)i * lmax;
                if (nnb[k] > nbmax) {
                    row[0] = -nnb[k];
                } else {
                    row[0] = nnb[k];
                    memcpy(row + 1, nbl + (size_t)k * (nj + 4), sizeof(int) * (size_t)nnb[k]);
                }
            }
        }
        free(nbl);
    }
}

/* float2_split of pot.avx.cpp:46-54 (shift 16, truncation toward zero). */
static inline void port_split16(double x, float *hi, float *lo)
{
    x *= (double)(1 << 16);
    const double xi = (double)(int)x;
    const double xf = x - xi;
    *hi = (float)(xi * (1.0 / (1 << 16)));
    *lo = (float)(xf * (1.0 / (1 << 16)));
}

/* gpupot of pot.avx.cpp:72-146: double-single positions, FP32 rsqrt with a
 * Newton step, compensated (hi, lo) sum, result hi + lo in FP64. */
void port_pot_fp32(int istart, int ni, int n, const double *m,
                   const double (*x)[3], double *pot)
{
    float *ph = (float *)malloc(sizeof(float) * 3 * (size_t)(n + 1));
    float *pl = (float *)malloc(sizeof(float) * 3 * (size_t)(n + 1));
    float *pm = (float *)malloc(sizeof(float) * (size_t)(n + 1));
    for (int j = 0; j < n; j++) {
        for (int k = 0; k < 3; k++) port_split16(x[j][k], &ph[3 * j + k], &pl[3 * j + k]);
        pm[j] = (float)m[j];
    }
#pragma omp parallel for schedule(dynamic, 16)
    for (int k = 0; k < ni; k++) {
        const int i = istart - 1 + k;
        float sh = 0.0f, sl = 0.0f;
        for (int j = 0; j < n; j++) {
            const float dx = (ph[3 * j + 0] - ph[3 * i + 0]) + (pl[3 * j + 0] - pl[3 * i + 0]);
            const float dy = (ph[3 * j + 1] - ph[3 * i + 1]) + (pl[3 * j + 1] - pl[3 * i + 1]);
            const float dz = (ph[3 * j + 2] - ph[3 * i + 2]) + (pl[3 * j + 2] - pl[3 * i + 2]);
            const float r2 = dx * dx + dy * dy + dz * dz;
            float rinv = ((r2 > 0.0f) ? pm[j] : 0.0f) * port_rsqrt(r2);
            const float t = sh;
            sh += rinv;
            sl -= (sh - t) - rinv;
        }
        pot[k] = (double)sh + (double)sl;
    }
    free(ph); free(pl); free(pm);
}

