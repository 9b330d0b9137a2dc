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
/* j-particles in SoA FP32 arrays so that the pair loop vectorises (NEON on
 * aarch64, SSE/AVX on x86) under "#pragma omp simd" with partial sums per
 * lane, the portable analogue of the 8-lane AVX loop of reg.avx.cpp:239-306. */

static float *port_j = NULL;      /* 7 arrays of port_cap: x y z m vx vy vz */
static int port_nbody = 0, port_cap = 0;

/* reciprocal square root: an initial estimate refined by Newton steps, as
 * v8sf_rsqrt does (reg.avx.cpp:74-77: hardware estimate, then
 * y1 = -0.5*y0*(x*y0*y0 - 3)).  The x86 estimate instruction has no portable
 * equivalent; the estimate here is the published bit-level one (C. Lomont,
 * "Fast inverse square root", 2003: i = 0x5f375a86 - (bits(x) >> 1), relative
 * error of the raw estimate < 3.5e-2, < 1.8e-3 after one Newton step), and
 * three Newton steps bring it to FP32 rounding level (max relative error
 * 4.7e-6 after two).  Finite for x = 0.  It vectorises on every target (NEON
 * on aarch64, SSE/AVX on x86). */
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

/* GPUNB_send of reg.avx.cpp:137-160: FP64 -> FP32, pad to an even count
 * with a massless body far away. */
void port_send_fp32(int nj, const double *mj, const double (*xj)[3],
                    const double (*vj)[3])
{
    if (nj + 2 > port_cap) {
        free(port_j);
        port_cap = nj + 2;
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
    if (nj % 2) {
        X[nj] = Y[nj] = Z[nj] = 255.0f;
        M[nj] = VX[nj] = VY[nj] = VZ[nj] = 0.0f;
        port_nbody++;
    }
}

void port_free_fp32(void)
{
    free(port_j);
    port_j = NULL;
    port_cap = port_nbody = 0;
}

#define PORT_JB 512

/* GPUNB_regf of reg.avx.cpp:185-331, one i at a time: FP32 pair arithmetic
 * with lane partial sums, FP64 result.  Neighbour flags are written per
 * j-block inside the vector loop and turned into the ascending list after it. */
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
        int *nbl = (int *)malloc(sizeof(int) * (size_t)(nj + 1));
        unsigned char flag[PORT_JB] __attribute__((aligned(64)));
#pragma omp for schedule(dynamic, 4)
        for (int i = 0; i < ni; i++) {
            const float xi = (float)xid[i][0], yi = (float)xid[i][1], zi = (float)xid[i][2];
            const float vxi = (float)vid[i][0], vyi = (float)vid[i][1], vzi = (float)vid[i][2];
            const float h2i = (float)h2d[i], dtri = (float)dtrd[i];
            const float mf = m_flag ? 1.0f : 0.0f;
            float ax = 0, ay = 0, az = 0, jx = 0, jy = 0, jz = 0, po = 0;
            int nnb = 0;
            for (int jb = 0; jb < nj; jb += PORT_JB) {
                const int jn = (nj - jb < PORT_JB) ? nj - jb : PORT_JB;
                const float *x = X + jb, *y = Y + jb, *z = Z + jb, *m = M + jb;
                const float *vx = VX + jb, *vy = VY + jb, *vz = VZ + jb;
                int any = 0;
#pragma omp simd reduction(+:ax, ay, az, jx, jy, jz, po) reduction(|:any)
                for (int jj = 0; jj < jn; jj++) {
                    const float dx = x[jj] - xi, dy = y[jj] - yi, dz = z[jj] - zi;
                    const float dvx = vx[jj] - vxi, dvy = vy[jj] - vyi, dvz = vz[jj] - vzi;
                    const float dxp = dx + dtri * dvx, dyp = dy + dtri * dvy, dzp = dz + dtri * dvz;
                    const float r2 = dx * dx + dy * dy + dz * dz;
                    float rv = dx * dvx + dy * dvy + dz * dvz;
                    const float r2p = dxp * dxp + dyp * dyp + dzp * dzp;
                    const float r2min = r2 < r2p ? r2 : r2p;
                    /* arithmetic instead of a select on m_flag, so that both
                     * criteria share one vectorised loop */
                    const float crit = h2i * (mf * m[jj] + (1.0f - mf));
                    const int in = r2min < crit;
                    flag[jj] = (unsigned char)in;
                    any |= in;
                    /* masked by multiplication, as the and-not mask of
                     * reg.avx.cpp:292 (a select after the call would keep
                     * the loop from vectorising) */
                    float rinv1 = (in ? 0.0f : 1.0f) * port_rsqrt(r2);
                    const float rinv2 = rinv1 * rinv1;
                    rinv1 *= m[jj];
                    const float rinv3 = rinv1 * rinv2;
                    rv *= -3.0f * rinv2;
                    po += rinv1;
                    ax += rinv3 * dx; ay += rinv3 * dy; az += rinv3 * dz;
                    jx += rinv3 * (dvx + rv * dx);
                    jy += rinv3 * (dvy + rv * dy);
                    jz += rinv3 * (dvz + rv * dz);
                }
                if (any) {
                    for (int jj = 0; jj < jn; jj++)
                        if (flag[jj]) nbl[nnb++] = jb + jj;
                }
            }
            acc[i][0] = ax; acc[i][1] = ay; acc[i][2] = az;
            jrk[i][0] = jx; jrk[i][1] = jy; jrk[i][2] = jz;
            pot[i] = po;
            int *row = list + (size_t)i * lmax;
            if (nnb > nbmax) {
                row[0] = -nnb;
            } else {
                row[0] = nnb;
                memcpy(row + 1, nbl, sizeof(int) * (size_t)nnb);
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

