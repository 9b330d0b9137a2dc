/*
 * CPU oracle for the NBODY6++GPU regular-force path.  TEST INFRASTRUCTURE ONLY:
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load this
 * library, and only to check or time against it.  The product (libgpunb.so)
 * never links or calls anything here.
 *
 * oracle_regf_fp64 / oracle_pot_fp64  -- FP64 truth.
 *   Arithmetic follows the FP64 Fortran loop src/Main/regint.f:39-79
 *   (A = X(J)-X(I), DV, RIJ2, DP = A + DV*DTR, RIJP, DR2I = 1/RIJ2,
 *    DR3I = BODY(J)*DR2I*SQRT(DR2I), DRDP = 3*DRDV*DR2I,
 *    FREG += A*DR3I, FDR += (DV - A*DRDP)*DR3I, POT += DR3I*RIJ2),
 *   but with the contract of the GPU/AVX back-ends that the Fortran caller
 *   sees through gpunb_regf_ (src/Main/gpunb.velocity.cu:162-208,822-878,
 *   src/Main/reg.avx.cpp:239-328):
 *     - the j-set is exactly what gpunb_send_ uploaded; i-particles are given
 *       by coordinates, so "self" (r2 == 0) is listed as a neighbour;
 *     - neighbour iff min(r2, r2p) < h2  (strict), or < m_j*h2 when m_flag
 *       (gpunb.velocity.cu:187,235; reg.avx.cpp:265-273);
 *     - neighbours contribute nothing to acc, jrk and pot;
 *     - list row i at list + i*lmax: [0] = count, [1..count] = 0-based j in
 *       ascending order; count > nnbmax -> [0] = -count, entries undefined
 *       (reg.avx.cpp:316-328; gpunb.velocity.cu:872-877).
 *   regint.f itself differs (non-strict test, self skipped, neighbours kept in
 *   POT); the GPU contract is what gpunb_regf_ callers rely on.
 *   The neighbour decision is evaluated with exactly the expression order of
 *   nb_test_fp64 and no FMA contraction (built with -ffp-contract=off), so that
 *   a device kernel re-testing a pair in FP64 in the same order reaches the
 *   same decision bit for bit.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------ */
/* FP64 neighbour decision: shared expression order with the device re-test. */
static inline int nb_test_fp64(const double xi[3], const double vi[3], double h2,
                               double dtr, const double xj[3], const double vj[3],
                               double mj, int m_flag, double *r2_out)
{
    const double dx = xj[0] - xi[0];
    const double dy = xj[1] - xi[1];
    const double dz = xj[2] - xi[2];
    const double dvx = vj[0] - vi[0];
    const double dvy = vj[1] - vi[1];
    const double dvz = vj[2] - vi[2];
    const double r2 = (dx * dx + dy * dy) + dz * dz;
    const double px = dx + dvx * dtr;
    const double py = dy + dvy * dtr;
    const double pz = dz + dvz * dtr;
    const double r2p = (px * px + py * py) + pz * pz;
    const double r2min = r2 < r2p ? r2 : r2p;
    const double crit = m_flag ? mj * h2 : h2;
    *r2_out = r2;
    return r2min < crit;
}

/*
 * FP64 regular force, jerk, potential and neighbour lists.
 * Optional outputs (may be NULL): accabs[i] = sum_j |m_j dx/r^3| and
 * jrkabs[i] = sum_j |jerk term|, potabs = pot (all terms positive); they give
 * the "sum of |terms|" normalisation for the error metric where |F| ~ 0.
 */
void oracle_regf_fp64(int nj, const double *mj, const double (*xj)[3],
                      const double (*vj)[3], int ni, const double *h2,
                      const double *dtr, const double (*xi)[3],
                      const double (*vi)[3], double (*acc)[3], double (*jrk)[3],
                      double *pot, int lmax, int nnbmax, int *list, int m_flag,
                      double *accabs, double *jrkabs)
{
#pragma omp parallel for schedule(dynamic, 4)
    for (int i = 0; i < ni; i++) {
        double ax = 0, ay = 0, az = 0, jx = 0, jy = 0, jz = 0, po = 0;
        double sa = 0, sj = 0;
        int nnb = 0;
        int *row = list + (size_t)i * lmax;
        for (int j = 0; j < nj; j++) {
            double r2;
            if (nb_test_fp64(xi[i], vi[i], h2[i], dtr[i], xj[j], vj[j], mj[j],
                             m_flag, &r2)) {
                if (nnb < nnbmax) row[1 + nnb] = j;
                nnb++;
                continue;
            }
            /* regint.f:41-78 arithmetic */
            const double a1 = xj[j][0] - xi[i][0];
            const double a2 = xj[j][1] - xi[i][1];
            const double a3 = xj[j][2] - xi[i][2];
            const double dv1 = vj[j][0] - vi[i][0];
            const double dv2 = vj[j][1] - vi[i][1];
            const double dv3 = vj[j][2] - vi[i][2];
            const double dr2i = 1.0 / r2;
            const double dr3i = mj[j] * dr2i * sqrt(dr2i);
            const double drdv = a1 * dv1 + a2 * dv2 + a3 * dv3;
            const double drdp = 3.0 * drdv * dr2i;
            const double fx = a1 * dr3i, fy = a2 * dr3i, fz = a3 * dr3i;
            const double gx = (dv1 - a1 * drdp) * dr3i;
            const double gy = (dv2 - a2 * drdp) * dr3i;
            const double gz = (dv3 - a3 * drdp) * dr3i;
            ax += fx; ay += fy; az += fz;
            jx += gx; jy += gy; jz += gz;
            po += dr3i * r2;
            sa += sqrt(fx * fx + fy * fy + fz * fz);
            sj += sqrt(gx * gx + gy * gy + gz * gz);
        }
        acc[i][0] = ax; acc[i][1] = ay; acc[i][2] = az;
        jrk[i][0] = jx; jrk[i][1] = jy; jrk[i][2] = jz;
        pot[i] = po;
        row[0] = (nnb > nnbmax) ? -nnb : nnb;
        if (accabs) accabs[i] = sa;
        if (jrkabs) jrkabs[i] = sj;
    }
}

/*
 * FP64 potential for the energy check, semantics of gpupot_
 * (src/Main/gpupot.gpu.cu:32-57,61-114; pot.avx.cpp:72-146):
 * pot[k] = sum_{j: r2 > 0} m_j / r_ij for i = istart-1+k (istart is 1-based),
 * positive sign, all j including near ones, coincident bodies skipped.
 */
void oracle_pot_fp64(int istart, int ni, int n, const double *m,
                     const double (*x)[3], double *pot)
{
#pragma omp parallel for schedule(dynamic, 16)
    for (int k = 0; k < ni; k++) {
        const int i = istart - 1 + k;
        double s = 0.0;
        for (int j = 0; j < n; j++) {
            const double dx = x[j][0] - x[i][0];
            const double dy = x[j][1] - x[i][1];
            const double dz = x[j][2] - x[i][2];
            const double r2 = (dx * dx + dy * dy) + dz * dz;
            if (r2 > 0.0) s += m[j] / sqrt(r2);
        }
        pot[k] = s;
    }
}

int oracle_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
