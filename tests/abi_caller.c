/*
 * abi_caller.c -- a plain C caller of libgpunb.so, as the Fortran integrator
 * links it: no Python, no torch, only the C ABI of include/gpunb.h with host
 * arrays.  Built and run by tests/test_abi_caller_gpu.py.
 *
 * A seeded cube of N bodies (FP64 host arrays); one gpunb_send_ and one
 * gpunb_regf_ of every body (the i-set = the j-set, as fpoly0.F:125 calls
 * it), and gpupot_ of all bodies.  Sampled rows are checked against a direct
 * FP64 sum written here: neighbour lists identical (count, ascending ids,
 * self included); potentials within 1e-6 relative; force and jerk within
 * 1e-6 of max(|Q|, S/8), S the sum of the pair terms' magnitudes (the bound
 * the library states: in a uniform cube the sums cancel in the interior).
 * Exit status 0 when every check passes.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "gpunb.h"

static unsigned long long lcg = 0x9E3779B97F4A7C15ull;
static double urand(void) {
  lcg = lcg * 6364136223846793005ull + 1442695040888963407ull;
  return (double)(lcg >> 11) * (1.0 / 9007199254740992.0);
}

int main(int argc, char **argv) {
  const int n = argc > 1 ? atoi(argv[1]) : 8192;
  const int lmax = 257, nnbmax = 256, mflag = 0;
  double *m = malloc(sizeof(double) * n), *h2 = malloc(sizeof(double) * n);
  double *dtr = malloc(sizeof(double) * n), *pot = malloc(sizeof(double) * n);
  double *pot2 = malloc(sizeof(double) * n);
  double(*x)[3] = malloc(sizeof(double[3]) * n), (*v)[3] = malloc(sizeof(double[3]) * n);
  double(*acc)[3] = malloc(sizeof(double[3]) * n), (*jrk)[3] = malloc(sizeof(double[3]) * n);
  int *list = malloc(sizeof(int) * (size_t)n * lmax);
  if (!m || !h2 || !dtr || !pot || !pot2 || !x || !v || !acc || !jrk || !list) return 2;
  /* ~40 neighbours each: h such that (4/3) pi h^3 n = 40 in the unit cube */
  const double h = cbrt(40.0 / (n * 4.18879));
  for (int i = 0; i < n; ++i) {
    m[i] = (0.5 + urand()) / n;
    for (int c = 0; c < 3; ++c) {
      x[i][c] = urand() - 0.5;
      v[i][c] = 0.1 * (urand() - 0.5);
    }
    h2[i] = h * h;
    dtr[i] = 1e-3;
  }
  int nb = n + 10, rank = 0, ni = n, nj = n;
  gpunb_open_(&nb, &rank);
  gpunb_send_(&nj, m, x, v);
  gpunb_regf_(&ni, h2, dtr, x, v, acc, jrk, pot, (int *)&lmax, (int *)&nnbmax, list,
              (int *)&mflag);
  int one = 1;
  gpupot_(&rank, &one, &ni, &nj, m, x, pot2);
  gpunb_close_();

  int bad = 0, rows = 0;
  double emax = 0.0;
  int *ids = malloc(sizeof(int) * lmax);
  for (int i = 0; i < n && bad < 10; i += 61) {
    double a[3] = {0, 0, 0}, j[3] = {0, 0, 0}, p = 0.0, pall = 0.0, sa = 0.0, sj = 0.0;
    int cnt = 0;
    for (int k = 0; k < n; ++k) {
      double dx[3], dv[3], dp[3], r2 = 0, rp2 = 0, rv = 0;
      for (int c = 0; c < 3; ++c) {
        dx[c] = x[k][c] - x[i][c];
        dv[c] = v[k][c] - v[i][c];
        dp[c] = dx[c] + dtr[i] * dv[c];
        r2 += dx[c] * dx[c];
        rp2 += dp[c] * dp[c];
        rv += dx[c] * dv[c];
      }
      if (r2 > 0) pall += m[k] / sqrt(r2);
      if ((r2 < rp2 ? r2 : rp2) < h2[i]) {
        if (cnt < lmax - 1) ids[cnt] = k;
        ++cnt;
        continue;
      }
      const double rinv = 1.0 / sqrt(r2), mr3 = m[k] * rinv * rinv * rinv;
      const double al = -3.0 * rv * rinv * rinv;
      p += m[k] * rinv;
      double t2 = 0.0;
      for (int c = 0; c < 3; ++c) {
        const double t = mr3 * (dv[c] + al * dx[c]);
        a[c] += mr3 * dx[c];
        j[c] += t;
        t2 += t * t;
      }
      sa += m[k] * rinv * rinv;
      sj += sqrt(t2);
    }
    ++rows;
    const int *row = list + (size_t)i * lmax;
    if (row[0] != cnt) {
      printf("row %d: count %d, expected %d\n", i, row[0], cnt);
      ++bad;
      continue;
    }
    for (int e = 0; e < cnt; ++e)
      if (row[1 + e] != ids[e]) {
        printf("row %d: entry %d is %d, expected %d\n", i, e, row[1 + e], ids[e]);
        ++bad;
        break;
      }
    double da = 0, na = 0, dj = 0, nj2 = 0;
    for (int c = 0; c < 3; ++c) {
      da += (acc[i][c] - a[c]) * (acc[i][c] - a[c]);
      na += a[c] * a[c];
      dj += (jrk[i][c] - j[c]) * (jrk[i][c] - j[c]);
      nj2 += j[c] * j[c];
    }
    const double ea = sqrt(da / fmax(na, sa * sa / 64.0)), ej = sqrt(dj / fmax(nj2, sj * sj / 64.0));
    const double ep = fabs(pot[i] - p) / p, eq = fabs(pot2[i] - pall) / pall;
    const double e = fmax(fmax(ea, ej), fmax(ep, eq));
    if (e > emax) emax = e;
    if (e > 1e-6) {
      printf("row %d: relative errors acc %.2e jrk %.2e pot %.2e gpupot %.2e\n", i, ea, ej, ep,
             eq);
      ++bad;
    }
  }
  printf("%s: %d rows checked, largest relative error %.2e\n", bad ? "FAILED" : "OK", rows, emax);
  return bad ? 1 : 0;
}
