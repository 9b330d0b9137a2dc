// The plain neighbour-radius rule of src/Main/regcor_gpu.F:120-234 on the
// device, shared by the learned RS update (rsmlp.cu) and the regular
// corrector (regcor.cu): NNBOPT stabilisation, NBAVE cap, taper outside the
// half-mass radius, inertial and radial-velocity factors, the c.m.-body
// branch, RSFAC limit, second-order cube root, shell square root and the
// inward reduction; the zero-neighbour branch :120-143.  The rule of at most
// three neighbours (:237-252) needs their positions and lives in regcor.cu.
#pragma once
#include "gpunb.h"

namespace gpunb {

// rs: RS(I); nnb, nnb0: new and previous counts (self excluded); x, v: the
// particle's predicted position and velocity; dtr: TIME - T0R(I); cm_a2:
// 100 BODY(I) / |H(I-N)| for a c.m. body (I > N), else any value <= 0.
// out: the new RS; target: the membership the rule aims at (A3).
__device__ __forceinline__ void rs_plain(const gpunb_rs_params &p, double rs, int nnb,
                                         int nnb0, const double *x, const double *v, double dtr,
                                         double cm_a2, double &out, double &target) {
  const double znbmin = fmax(0.01 * p.nnbmax, 1.0);
  const double d0 = x[0] - p.rdens[0], d1 = x[1] - p.rdens[1], d2 = x[2] - p.rdens[2];
  double ri2, rh2;
  if (p.nb_flag) {
    ri2 = d0 * d0 + d1 * d1 + d2 * d2;
    rh2 = p.rscale * p.rscale;
  } else {
    ri2 = x[0] * x[0] + x[1] * x[1] + x[2] * x[2];
    rh2 = 9.0 * p.rscale * p.rscale;
  }
  const double rc2 = p.rc * p.rc;
  if (nnb == 0) {
    const double rdot = x[0] * v[0] + x[1] * v[1] + x[2] * v[2];
    out = rdot > 0.0 ? fmax(0.75 * rs, 0.1 * p.rscale) : 1.1 * rs;
    target = (double)p.nnbopt;
    return;
  }
  const double n = (double)nnb;
  const double fac = 1.0 + 0.1 * ((double)p.nnbopt - n) / n;
  double a3 = n * fac;
  const double nbave =
      (double)min(p.nnbopt + 150, max(p.nnbmax - 50, (int)znbmin));
  a3 = fmin(a3, 0.9 * nbave);
  const long long nbp = (long long)a3;
  if (p.nb_flag)
    a3 = ri2 > rh2 ? a3 * fmax(p.rscale / sqrt(ri2), 0.1) : fmax(a3, znbmin);
  else
    a3 = fmax(a3, znbmin);
  target = a3;
  double a4 = a3 / n;
  if ((a3 - (double)nnb0) * (a3 - n) < 0.0) a4 = sqrt(a4);
  const double ridot = d0 * v[0] + d1 * v[1] + d2 * v[2];
  if (p.nb_flag && ri2 > rc2 && ri2 < 100.0 * rh2) a4 = a4 * (1.0 + ridot * dtr / ri2);
  // c.m. body of a KS pair inside the half-mass radius (regcor_gpu.F:182-193):
  // with the perturber range A2 = 100 BODY / |H| beyond RS, stabilise the
  // count on NBAVE by a square-root volume factor
  if (cm_a2 > 0.0 && ri2 <= rh2 && cm_a2 > rs) a4 = 1.0 + 0.5 * fmax(1.0 - n / nbave, 0.0);
  const double a5 = fmin(p.rsfac * dtr, 0.25);
  a4 = a4 - 1.0;
  a4 = a4 > a5 ? a5 : fmax(a4, -a5);
  const double a3v = a4 / 3.0;
  double a1 = 1.0 + a3v - a3v * a3v;
  if (n < znbmin && (double)nbp > znbmin && a1 < 1.0) a1 = 1.05;
  const bool change = fabs(a1 - 1.0) > 0.003;
  const bool shell = rs * rs > ri2 && rs * rs < 2.0 * ri2 && n > 5.0;
  if (change && shell) a1 = sqrt(fmax(a1, 0.0));
  double nw = change ? a1 * rs : rs;
  if (n > nbave && ridot < 0.0) nw = nw * (1.0 - (n - nbave) / (3.0 * n));
  out = nw;
}


}  // namespace gpunb
