"""The plain neighbour-radius rules of NBODY6++, vectorised over the particles
of an active block.  They are the fallback of the learned predictor and the
baseline it is compared against.

* `overflow_rs`   -- src/Main/util_gpu.F:81-97 (and fpoly0.F:142-150): after
  a list overflow (count reported as -n), RS <- (NNBOPT/n)^0.333 RS when
  n > NNBOPT, else (NNBOPT/NNBMAX)^0.4 RS (NB_FLAG = 1), or 0.9 RS.
* `few_nb_rs`     -- src/Main/fpoly0.F:133-158: fewer than 2 members -> 1.5 RS.
* `regcor_rs`     -- src/Main/regcor_gpu.F:120-253: the volume-ratio update
  after a regular step (NNBOPT stabilisation, inertial factor, radial
  velocity factor, the RSFAC limit on the change per step, second-order cube
  root, the extra reduction for inward motion, the zero-neighbour branch).
  The c.m.-body branch (`I > N`, :183-198) needs KS-pair data and the
  few-member radial-velocity branch (`M_FLAG = 0`, NNB <= 3, :236-253) needs
  the neighbours' positions; both are left out.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class RSParams:
    nnbopt: int               # optimal neighbour number (input NNBOPT)
    nnbmax: int               # list capacity (NNBMAX)
    rscale: float = 0.8       # half-mass radius (RSCALE)
    rc: float = 0.3           # core radius (RC)
    rsfac: float = 50.0       # MAX(25/TCR, 3 VC/(2 RSMIN)) (adjust.F:220), Henon units
    nb_flag: int = 1          # KZ(39) = 0 or 2
    bodym: float = 1.0        # mean mass (for the zero-neighbour branch)

    @property
    def znbmin(self) -> float:      # input.F:122
        return max(0.01 * self.nnbmax, 1.0)

    @property
    def znbmax(self) -> float:      # input.F:123
        return 0.9 * self.nnbmax


def overflow_rs(rs: np.ndarray, nnb_neg: np.ndarray, p: RSParams) -> np.ndarray:
    """util_gpu.F:81-97: nnb_neg is the in-band overflow count (< 0)."""
    n = -nnb_neg.astype(np.float64)
    if p.nb_flag:
        fac = np.where(n > p.nnbopt, (p.nnbopt / np.maximum(n, 1.0)) ** 0.333,
                       (p.nnbopt / p.nnbmax) ** 0.4)
    else:
        fac = np.full_like(n, 0.9)
    return rs * fac


def few_nb_rs(rs: np.ndarray) -> np.ndarray:
    """fpoly0.F:153-158: fewer than two neighbours -> enlarge by 1.5."""
    return 1.5 * rs


def regcor_rs(rs: np.ndarray, nnb: np.ndarray, nnb0: np.ndarray, xi: np.ndarray,
              vi: np.ndarray, dtr: np.ndarray, p: RSParams, rdens=(0.0, 0.0, 0.0),
              return_target: bool = False):
    """New RS after a regular step (regcor_gpu.F:120-253).  With
    return_target, also returns the membership the rule aims at (A3 after
    the NBAVE cap, the taper outside the half-mass radius and the ZNBMIN
    floor, :152-163), which the rule then approaches by at most 25% in
    volume per step.

    rs, nnb (current count, self excluded), nnb0 (previous count), xi, vi
    (state of the particle), dtr (regular step just taken)."""
    rs = rs.astype(np.float64).copy()
    nnb = nnb.astype(np.float64)
    nnb0 = nnb0.astype(np.float64)
    d = xi - np.asarray(rdens)
    if p.nb_flag:
        ri2 = np.einsum("ij,ij->i", d, d)
        rh2 = p.rscale ** 2
    else:
        ri2 = np.einsum("ij,ij->i", xi, xi)
        rh2 = 9.0 * p.rscale ** 2
    rc2 = p.rc ** 2
    out = rs.copy()
    # zero neighbours (:120-143): shrink for outward, grow for inward motion
    zero = nnb == 0
    if np.any(zero):
        rdot = np.einsum("ij,ij->i", xi, vi)
        out[zero] = np.where(rdot[zero] > 0.0, np.maximum(0.75 * rs[zero], 0.1 * p.rscale),
                             1.1 * rs[zero])
    m = ~zero
    if not np.any(m):
        return (out, np.full(rs.shape, float(p.nnbopt))) if return_target else out
    n = nnb[m]
    fac = 1.0 + 0.1 * (p.nnbopt - n) / n                       # :152
    a3 = n * fac                                                # :155
    nbave = min(p.nnbopt + 150, max(p.nnbmax - 50, int(p.znbmin)))
    a3 = np.minimum(a3, 0.9 * nbave)
    nbp = a3.astype(np.int64)
    r2 = ri2[m]
    if p.nb_flag:
        a3 = np.where(r2 > rh2, a3 * np.maximum(p.rscale / np.sqrt(r2), 0.1), np.maximum(a3, p.znbmin))
    else:
        a3 = np.maximum(a3, p.znbmin)
    target = np.full(rs.shape, float(p.nnbopt))
    target[m] = a3
    a4 = a3 / n
    inertial = (a3 - nnb0[m]) * (a3 - n) < 0.0                  # :169
    a4 = np.where(inertial, np.sqrt(a4), a4)
    ridot = np.einsum("ij,ij->i", d[m], vi[m])
    if p.nb_flag:
        outer = (r2 > rc2) & (r2 < 100.0 * rh2)                 # :175
        a4 = np.where(outer, a4 * (1.0 + ridot * dtr[m] / r2), a4)
    a5 = np.minimum(p.rsfac * dtr[m], 0.25)                     # :201
    a4 = a4 - 1.0
    a4 = np.where(a4 > a5, a5, np.maximum(a4, -a5))
    a3v = a4 / 3.0
    a1 = 1.0 + a3v - a3v * a3v                                  # :213
    a1 = np.where((n < p.znbmin) & (nbp > p.znbmin) & (a1 < 1.0), 1.05, a1)
    change = np.abs(a1 - 1.0) > 0.003
    rsm = rs[m]
    shell = (rsm ** 2 > r2) & (rsm ** 2 < 2.0 * r2) & (n > 5)
    a1 = np.where(change & shell, np.sqrt(np.maximum(a1, 0.0)), a1)
    new = np.where(change, a1 * rsm, rsm)
    inward = (n > nbave) & (ridot < 0.0)                        # :232
    drs = (n - nbave) / (3.0 * n)
    new = np.where(inward, new * (1.0 - drs), new)
    out[m] = new
    return (out, target) if return_target else out
