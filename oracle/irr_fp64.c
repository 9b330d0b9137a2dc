/*
 * FP64 restatement of the irregular (neighbour) force of NBODY6++'s SIMD
 * library, src/Main/irr.avx.cpp (TEST INFRASTRUCTURE ONLY: the checker of the
 * GPU irregular-force kernels, never part of the product).
 *
 * For each active particle i (0-based index addr[k]) at time ti:
 *   - predict i and each listed neighbour j from its stored state
 *     (x0, v0, a2 = F/2 as set, j6 = FDOT/6 as set, t0) to ti
 *     (irr.avx.cpp:162-176, Pred2):
 *         dt = ti - t0
 *         x  = x0 + dt (v0 + dt (a2 + dt j6))
 *         v  = v0 + 2 dt (a2 + 1.5 dt j6)
 *   - sum over the list (irr.avx.cpp:275-299, calc_and_accum):
 *         acc += m_j dx / r^3
 *         jrk += m_j / r^3 (dv - 3 (dx.dv) / r^2 dx)
 *   - nnbid = 1 + index of the listed j with the smallest r^2 (smaller index
 *     on ties), 0 for an empty list (irr.avx.cpp:257-273,283-285,308-309).
 * Lists: row i of lists[n][lmax] holds the count in [0] and 0-based ids after
 * it (the library stores the Fortran ids minus one, irr.avx.cpp:449-481).
 */
#include <math.h>
#include <stddef.h>

void oracle_irr_fp64(int n, const double *x0, const double *v0, const double *a2,
                     const double *j6, const double *m, const double *t0, int lmax,
                     const int *lists, double ti, int ni, const int *addr, double *acc,
                     double *jrk, int *nnbid)
{
    (void)n;
#pragma omp parallel for schedule(dynamic, 8)
    for (int k = 0; k < ni; k++) {
        const int i = addr[k];
        double xi[3], vi[3];
        const double dti = ti - t0[i];
        for (int c = 0; c < 3; c++) {
            const size_t o = 3 * (size_t)i + c;
            xi[c] = x0[o] + dti * (v0[o] + dti * (a2[o] + dti * j6[o]));
            vi[c] = v0[o] + 2.0 * dti * (a2[o] + 1.5 * dti * j6[o]);
        }
        const int *row = lists + (size_t)i * lmax;
        const int nnb = row[0];
        double ax = 0, ay = 0, az = 0, jx = 0, jy = 0, jz = 0;
        double best = INFINITY;
        int best_j = -1;
        for (int q = 0; q < nnb; q++) {
            const int j = row[1 + q];
            const double dt = ti - t0[j];
            double dx[3], dv[3];
            for (int c = 0; c < 3; c++) {
                const size_t o = 3 * (size_t)j + c;
                const double xj = x0[o] + dt * (v0[o] + dt * (a2[o] + dt * j6[o]));
                const double vj = v0[o] + 2.0 * dt * (a2[o] + 1.5 * dt * j6[o]);
                dx[c] = xj - xi[c];
                dv[c] = vj - vi[c];
            }
            const double r2 = dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2];
            const double rv = dx[0] * dv[0] + dx[1] * dv[1] + dx[2] * dv[2];
            const double rinv2 = 1.0 / r2;
            const double mr3 = m[j] * rinv2 * sqrt(rinv2);
            const double al = -3.0 * rv * rinv2;
            ax += mr3 * dx[0];
            ay += mr3 * dx[1];
            az += mr3 * dx[2];
            jx += mr3 * (dv[0] + al * dx[0]);
            jy += mr3 * (dv[1] + al * dx[1]);
            jz += mr3 * (dv[2] + al * dx[2]);
            if (r2 < best || (r2 == best && j < best_j)) {
                best = r2;
                best_j = j;
            }
        }
        acc[3 * (size_t)k] = ax;
        acc[3 * (size_t)k + 1] = ay;
        acc[3 * (size_t)k + 2] = az;
        jrk[3 * (size_t)k] = jx;
        jrk[3 * (size_t)k + 1] = jy;
        jrk[3 * (size_t)k + 2] = jz;
        nnbid[k] = best_j + 1;
    }
}
