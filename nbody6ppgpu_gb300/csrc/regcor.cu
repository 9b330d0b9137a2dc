// Regular corrector of an active block on the device: the work of
// src/Main/regcor_gpu.F:1-805 (REGCOR_GPU) for every body of the block, one
// thread per body, after the regular force of the block has been computed
// (gpunb_regf_ / gpunb_regf_device).  The reference runs it on the host, body
// by body, inside an OpenMP loop (intgrt.F), so the neighbour lists and
// forces of every regular block cross to the host and back.
//
// Per body I (Fortran numbering, 1-based), with XI, XIDOT its predicted
// position and velocity, FREG, FDR the new regular force and derivative and
// NLIST the new neighbour list (self removed):
//   * neighbour radius RS(I): the plain rule (rsrule.cuh, regcor_gpu.F:120-234)
//     with the c.m.-body branch (:182-193), and the rule for at most three
//     neighbours (:237-252) from their predicted positions;
//   * zero new neighbours: the small-central-mass force change (:120-143);
//   * neighbour changes (:262-460): the old list LIST(.,I) and NLIST are
//     merged in index order; an old neighbour with a step below SMIN inside
//     2 RS is kept (its force moves from the regular to the irregular side,
//     :360-410); the force and derivative of every lost and gained neighbour
//     form DFIRR, DFD.  One deviation: when the new list is empty, the
//     reference's insertion loop compares against NLIST(1), which then holds
//     the saved last old member, so the first kept body is displaced by that
//     member and the list no longer matches the forces moved (:386-392);
//     here a kept body enters an empty list like any other;
//   * the Hermite corrector of the regular polynomial (:462-552): XN, XNDOT,
//     FI, FR, FIDOT, FRDOT, D0, D0R..D3R, T0R, with the tidal FIDOT term for
//     KZ(14) <= 2 and the corrector suppression for large step ratios;
//   * LIST(.,I) = NLIST when the membership changed (:608-616);
//   * the new regular step STEPR (:618-768: composite criterion, discrete
//     doubling/halving with the DMOD commensurability tests, Makino's
//     convergence test, SMAX cap) and the irregular step reductions
//     (:770-800).
// Not done here (caller's side, as in the reference's separate routines):
// external and cloud forces (XTRNLF, FCLOUD), CHECKL, FPCORR, the tidal
// energy ETIDE and the diagnostic prints.
#include <cmath>

#include "common.cuh"
#include "rsrule.cuh"

namespace gpunb {

constexpr int REGCOR_THREADS = 128;

__device__ __forceinline__ void pair_force(const double *xi, const double *vi,
                                           const double *xj, const double *vj, double mj,
                                           double *f, double *fd) {
  // regcor_gpu.F:346-357 (and :428-437, :450-459)
  const double a0 = xj[0] - xi[0], a1 = xj[1] - xi[1], a2 = xj[2] - xi[2];
  const double dv0 = vj[0] - vi[0], dv1 = vj[1] - vi[1], dv2 = vj[2] - vi[2];
  const double rij2 = a0 * a0 + a1 * a1 + a2 * a2;
  const double dr2i = 1.0 / rij2;
  const double dr3i = mj * dr2i * sqrt(dr2i);
  const double drdv = a0 * dv0 + a1 * dv1 + a2 * dv2;
  const double drdp = 3.0 * drdv * dr2i;
  f[0] = a0 * dr3i; f[1] = a1 * dr3i; f[2] = a2 * dr3i;
  fd[0] = (dv0 - a0 * drdp) * dr3i;
  fd[1] = (dv1 - a1 * drdp) * dr3i;
  fd[2] = (dv2 - a2 * drdp) * dr3i;
}

// Walks the old row a[0..n0) and the new row b[0..n1) (both ascending body
// indices) in merge order and calls lost(J) / gained(J) for the members of
// only one of them -- the comparison of regcor_gpu.F:300-330.
template <class L, class G>
__device__ __forceinline__ void merge_rows(const int *a, int n0, const int *b, int n1, L lost,
                                           G gained) {
  int p = 0, q = 0;
  while (p < n0 || q < n1) {
    if (q >= n1 || (p < n0 && a[p] < b[q])) {
      lost(a[p++]);
    } else if (p >= n0 || b[q] < a[p]) {
      gained(b[q++]);
    } else {
      ++p;
      ++q;
    }
  }
}

// One thread per active body.  STEP of other bodies is read (the small-step
// retention), so this kernel leaves STEP and TIMENW of the block untouched
// and writes the new irregular step to step_new[k]; regcor_apply_kernel
// stores them afterwards.  Every read of STEP therefore sees the values at
// entry, whatever the order in which the bodies run.
__global__ void __launch_bounds__(REGCOR_THREADS)
    regcor_kernel(int ni, const int *__restrict__ iact, const double *__restrict__ freg_in,
                  const double *__restrict__ fdr_in, int *__restrict__ nlist,
                  const gpunb_regcor_params p, const gpunb_regcor_state s,
                  double *__restrict__ step_new) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= ni) return;
  const int lmax = p.lmax;
  const int I = iact[k];           // 1-based
  const int ii = I - 1;
  const double *xi = s.x + 3 * (size_t)ii, *vi = s.xdot + 3 * (size_t)ii;
  int *nl = nlist + (size_t)k * lmax;        // nl[0] = NNB, nl[1..NNB] members
  int *ol = s.list + (size_t)ii * lmax;      // ol[0] = NNB0, ol[1..NNB0]
  int nnb = nl[0];
  const int nnb0 = ol[0];
  const double dtr = p.time - s.t0r[ii];
  double freg[3], fdr[3], dfirr[3] = {0.0, 0.0, 0.0}, dfd[3] = {0.0, 0.0, 0.0};
  for (int c = 0; c < 3; ++c) {
    freg[c] = freg_in[3 * (size_t)k + c];
    fdr[c] = fdr_in[3 * (size_t)k + c];
  }
  const gpunb_rs_params &rp = p.rs;
  const double rs_old = s.rs[ii];
  const double rs2 = rs_old * rs_old;
  double ri2, rh2;
  if (rp.nb_flag) {
    const double d0 = xi[0] - rp.rdens[0], d1 = xi[1] - rp.rdens[1], d2 = xi[2] - rp.rdens[2];
    ri2 = d0 * d0 + d1 * d1 + d2 * d2;
    rh2 = rp.rscale * rp.rscale;
  } else {
    ri2 = xi[0] * xi[0] + xi[1] * xi[1] + xi[2] * xi[2];
    rh2 = 9.0 * rp.rscale * rp.rscale;
  }

  // ---- neighbour radius -------------------------------------------------
  double rs_new, target;
  if (nnb == 0) {
    // small mass at the centre for a body without neighbours (:120-143)
    const double r2 = xi[0] * xi[0] + xi[1] * xi[1] + xi[2] * xi[2];
    const double fij = 0.01 * rp.bodym / (r2 * sqrt(r2));
    const double rdot = 3.0 * (xi[0] * vi[0] + xi[1] * vi[1] + xi[2] * vi[2]) / r2;
    for (int c = 0; c < 3; ++c) {
      dfirr[c] = -fij * xi[c];
      dfd[c] = -(vi[c] - rdot * xi[c]) * fij;
    }
    rs_new = rdot > 0.0 ? fmax(0.75 * rs_old, 0.1 * rp.rscale) : 1.1 * rs_old;
    if (s.counters) atomicAdd(s.counters + 0, 1);   // NBVOID
  } else {
    double cm_a2 = -1.0;
    if (I > p.n && s.h) {
      const double h = fabs(s.h[I - p.n - 1]);
      cm_a2 = h > 0.0 ? 100.0 * s.body[ii] / h : INFINITY;
    }
    rs_plain(rp, rs_old, nnb, nnb0, xi, vi, dtr, cm_a2, rs_new, target);
    // at most three neighbours: smallest separation a constant regular step
    // ahead (:237-252)
    if (!p.m_flag && nnb <= 3 && ri2 < 100.0 * rh2) {
      double a1 = 2.0 * rs_new;
      for (int l = 1; l <= nnb; ++l) {
        const int j = nl[l] - 1;
        const double *xj = s.x + 3 * (size_t)j, *vj = s.xdot + 3 * (size_t)j;
        const double e0 = xi[0] - xj[0], e1 = xi[1] - xj[1], e2 = xi[2] - xj[2];
        const double rij = sqrt(e0 * e0 + e1 * e1 + e2 * e2);
        const double rsdot =
            (e0 * (vi[0] - vj[0]) + e1 * (vi[1] - vj[1]) + e2 * (vi[2] - vj[2])) / rij;
        a1 = fmin(a1, rij + rsdot * dtr);
      }
      rs_new = fmax(a1, 1.1 * rs_new);
    }
  }
  s.rs[ii] = rs_new;

  // ---- neighbour changes --------------------------------------------------
  int nbloss = 0, nbgain = 0;
  if (nnb0 > 0) {
    bool jmin = false;
    merge_rows(ol + 1, nnb0, nl + 1, nnb,
               [&](int j) { if (s.step[j - 1] < p.smin) jmin = true; }, [&](int) {});
    if (jmin && I <= p.n) {
      // keep old neighbours with a step below SMIN inside 2 RS (:360-410):
      // each moves into NLIST (ascending) and its force out of FREG, FDR
      int pa = 0, qb = 0;
      while (pa < nnb0) {
        const int j = ol[1 + pa];
        while (qb < nnb && nl[1 + qb] < j) ++qb;
        ++pa;
        if (qb < nnb && nl[1 + qb] == j) continue;   // still a neighbour
        if (nnb > p.nnbmax) break;
        if (s.step[j - 1] > p.smin || j < p.ifirst || j > p.n) continue;
        const double *xj = s.x + 3 * (size_t)(j - 1);
        const double e0 = xi[0] - xj[0], e1 = xi[1] - xj[1], e2 = xi[2] - xj[2];
        if (e0 * e0 + e1 * e1 + e2 * e2 > 4.0 * rs2) continue;
        if (nnb + 1 > lmax - 1) break;   // no room in the row
        for (int l = nnb; l > qb; --l) nl[1 + l] = nl[l];
        nl[1 + qb] = j;
        ++nnb;
        double f[3], fd[3];
        pair_force(xi, vi, xj, s.xdot + 3 * (size_t)(j - 1), s.body[j - 1], f, fd);
        for (int c = 0; c < 3; ++c) {
          freg[c] -= f[c];
          fdr[c] -= fd[c];
        }
        if (s.counters) atomicAdd(s.counters + 1, 1);   // NBSMIN
      }
      nl[0] = nnb;
    }
    // losses first, then gains, each in index order (:414-460)
    merge_rows(ol + 1, nnb0, nl + 1, nnb,
               [&](int j) {
                 double f[3], fd[3];
                 pair_force(xi, vi, s.x + 3 * (size_t)(j - 1), s.xdot + 3 * (size_t)(j - 1),
                            s.body[j - 1], f, fd);
                 for (int c = 0; c < 3; ++c) {
                   dfirr[c] -= f[c];
                   dfd[c] -= fd[c];
                 }
                 ++nbloss;
               },
               [&](int) {});
    merge_rows(ol + 1, nnb0, nl + 1, nnb, [&](int) {},
               [&](int j) {
                 double f[3], fd[3];
                 pair_force(xi, vi, s.x + 3 * (size_t)(j - 1), s.xdot + 3 * (size_t)(j - 1),
                            s.body[j - 1], f, fd);
                 for (int c = 0; c < 3; ++c) {
                   dfirr[c] += f[c];
                   dfd[c] += fd[c];
                 }
                 ++nbgain;
               });
  } else {
    for (int l = 1; l <= nnb; ++l) {
      const int j = nl[l];
      double f[3], fd[3];
      pair_force(xi, vi, s.x + 3 * (size_t)(j - 1), s.xdot + 3 * (size_t)(j - 1), s.body[j - 1],
                 f, fd);
      for (int c = 0; c < 3; ++c) {
        dfirr[c] += f[c];
        dfd[c] += fd[c];
      }
    }
    nbgain = nnb;
  }

  // ---- corrector (:462-552) ------------------------------------------------
  const double dtsq = dtr * dtr;
  const double dt6 = 6.0 / (dtr * dtsq);
  const double dt2 = 2.0 / dtsq;
  double dtsq12 = dtsq / 12.0;
  double dtr13 = dtr / 3.0;
  s.t0r[ii] = p.time;
  const double step_i = s.step[ii];
  if (step_i < 5.0 * p.dtmin && dtr > 50.0 * step_i) {
    dtr13 = 0.0;
    dtsq12 = 0.0;
  }
  double *fi = s.fi + 3 * (size_t)ii, *fid = s.fidot + 3 * (size_t)ii;
  double *fr = s.fr + 3 * (size_t)ii, *frd = s.frdot + 3 * (size_t)ii;
  double d2r[3], d3r[3];
  for (int c = 0; c < 3; ++c) {
    const double dfr = fr[c] - freg[c] - dfirr[c];
    const double fdr0 = fdr[c] + dfd[c];
    const double frdc = frd[c];
    const double sum = frdc + fdr0;
    const double at3 = 2.0 * dfr + dtr * sum;
    const double bt2 = -3.0 * dfr - dtr * (sum + frdc);
    s.xn[3 * (size_t)ii + c] = s.x0[3 * (size_t)ii + c] + (0.6 * at3 + bt2) * dtsq12;
    s.xndot[3 * (size_t)ii + c] = s.x0dot[3 * (size_t)ii + c] + (0.75 * at3 + bt2) * dtr13;
    fi[c] += dfirr[c];
    fr[c] = freg[c];
    fid[c] += dfd[c];
    frd[c] = fdr[c];
    if (p.kz14 <= 2) {
      if (c == 1) fid[0] -= p.tidal4 * dfr;
      if (c == 0) fid[1] += p.tidal4 * dfr;
    }
    s.d0[3 * (size_t)ii + c] = fi[c];
    s.d0r[3 * (size_t)ii + c] = freg[c];
    s.d1r[3 * (size_t)ii + c] = fdr[c];
    d3r[c] = at3 * dt6;
    d2r[c] = (3.0 * at3 + bt2) * dt2;
    s.d3r[3 * (size_t)ii + c] = d3r[c];
    s.d2r[3 * (size_t)ii + c] = d2r[c];
  }

  // ---- new neighbour list (:608-616) ------------------------------------------
  if (nbloss + nbgain > 0) {
    ol[0] = nnb;
    for (int l = 1; l <= nnb; ++l) ol[l] = nl[l];
    if (s.counters) atomicAdd(s.counters + 2, nbloss + nbgain);   // NBFLUX
  }

  // ---- new regular step (:618-768) -------------------------------------------
  const double fr2 = freg[0] * freg[0] + freg[1] * freg[1] + freg[2] * freg[2];
  const double w1 = fdr[0] * fdr[0] + fdr[1] * fdr[1] + fdr[2] * fdr[2];
  const double w2 = d2r[0] * d2r[0] + d2r[1] * d2r[1] + d2r[2] * d2r[2];
  const double w3 = d3r[0] * d3r[0] + d3r[1] * d3r[1] + d3r[2] * d3r[2];
  double w0 = (sqrt(fr2 * w2) + w1) / (sqrt(w1 * w3) + w2);
  w0 = p.etar * w0;
  double ttmp = sqrt(w0);
  const double dt0 = ttmp;
  const double stepr = s.stepr[ii];
  if (ttmp > 2.0 * stepr) {
    if (fmod(p.time, 2.0 * dtr) == 0.0) {
      ttmp = fmin(2.0 * dtr, p.smax);
      while (dt0 > 2.0 * ttmp && 2.0 * ttmp < p.smax && fmod(p.time, 2.0 * ttmp) == 0.0)
        ttmp = 2.0 * ttmp;
    } else {
      ttmp = stepr;
    }
  } else if (ttmp < dtr) {
    ttmp = 0.5 * dtr;
    if (ttmp > dt0) ttmp = 0.5 * ttmp;
  } else {
    ttmp = stepr;
  }
  if (ttmp > 0.1 && ttmp > dtr) {
    double dv2 = 0.0;
    for (int c = 0; c < 3; ++c) {
      const double d = vi[c] - s.xndot[3 * (size_t)ii + c];
      dv2 += d * d;
    }
    const double dtj = dtr * pow(1.0e-4 * dtr * dtr * fr2 / dv2, 0.1);
    if (dtj < ttmp) ttmp = dtr;
  }
  ttmp = fmin(ttmp, p.smax);
  s.stepr[ii] = ttmp;
  double st = step_i;
  if (nnb0 == 0 && nnb >= 0) st = 0.125 * st;
  while (ttmp < st) {
    st = 0.5 * st;
    if (s.counters) atomicAdd(s.counters + 3, 1);   // NICONV
  }
  step_new[k] = st;
}

// STEP(I) and, where it changed, TIMENW(I) = T0(I) + STEP(I) (:770-800).
__global__ void regcor_apply_kernel(int ni, const int *__restrict__ iact,
                                    const double *__restrict__ step_new, double *__restrict__ step,
                                    const double *__restrict__ t0, double *__restrict__ timenw) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= ni) return;
  const int ii = iact[k] - 1;
  const double st = step_new[k];
  if (st != step[ii]) timenw[ii] = t0[ii] + st;
  step[ii] = st;
}

// scratch for the new steps of the last block (grow-only; the call is
// otherwise free of library state)
static double *g_step_new = nullptr;
static size_t g_step_cap = 0;

}  // namespace gpunb

using namespace gpunb;

extern "C" int gpunb_regcor_device(int ni, const int *iact, const double *freg, const double *fdr,
                                   int *nlist, const gpunb_regcor_params *p,
                                   const gpunb_regcor_state *s, void *stream) {
  if (ni < 0 || !p || !s || (ni > 0 && (!iact || !freg || !fdr || !nlist))) return GPUNB_E_ARG;
  if (p->lmax < 2 || p->n < 0 || p->ntot < p->n) return GPUNB_E_ARG;
  if (!s->x || !s->xdot || !s->body || !s->x0 || !s->x0dot || !s->t0r || !s->stepr ||
      !s->step || !s->t0 || !s->timenw || !s->fi || !s->fidot || !s->fr || !s->frdot ||
      !s->d0 || !s->d0r || !s->d1r || !s->d2r || !s->d3r || !s->xn || !s->xndot || !s->rs ||
      !s->list)
    return GPUNB_E_ARG;
  if (ni == 0) return GPUNB_OK;
  if ((size_t)ni > g_step_cap) {
    if (g_step_new) cudaFree(g_step_new);
    g_step_new = nullptr;
    g_step_cap = 0;
    if (cudaMalloc(&g_step_new, (size_t)ni * sizeof(double)) != cudaSuccess) {
      cudaGetLastError();
      return GPUNB_E_ALLOC;
    }
    g_step_cap = (size_t)ni;
  }
  const cudaStream_t st = (cudaStream_t)stream;
  const int grid = (ni + REGCOR_THREADS - 1) / REGCOR_THREADS;
  regcor_kernel<<<grid, REGCOR_THREADS, 0, st>>>(ni, iact, freg, fdr, nlist, *p, *s, g_step_new);
  regcor_apply_kernel<<<grid, REGCOR_THREADS, 0, st>>>(ni, iact, g_step_new, s->step, s->t0,
                                                        s->timenw);
  return cudaGetLastError() == cudaSuccess ? GPUNB_OK : GPUNB_E_CUDA;
}
