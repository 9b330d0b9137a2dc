"""Seeded synthetic star-cluster inputs for the regular-force path.

The reference takes its initial conditions from the Fortran set-up chain; this
module restates the recipes that matter for the regular force so that every
test and benchmark input is reproducible from a seed:

* Plummer sphere: src/Main/setup.F:62-106 (radius from the cumulative mass
  ``(A**(-2/3) - 1)**(-1/2)`` with rejection beyond 10, isotropic direction,
  speed from the von Neumann rejection ``0.1*A5 > A4**2 (1-A4**2)**3.5``,
  centre-of-mass correction, scaling by ``SX = 3*pi/16``, ``SV = sqrt(M/SX)``).
* Kroupa IMF: the two segments of src/Main/imfbd.f:46-51 that lie inside
  0.08-100 Msun (slope 1.3 below 0.5 Msun, 2.3 above), sampled by inverse CDF.
* King (1966) model W0: written from the King distribution function (the
  reference reads King models from external files, src/Main/data.F:31-64).
* Henon units (G = M = 1, E = -1/4) as src/Main/scale.F does it: virial
  velocity scaling then a length scaling to E0 = -0.25.
* Initial neighbour radius and regular step: src/Main/fpoly0.F:46-56
  (``STEPR = min(SMAX/8*sqrt(1+r^2), SMAX)``); per-particle RS from the local
  density (k-th nearest neighbour distance), with one global factor bisected
  so that the mean neighbour count (self excluded) hits the target.

Random numbers come from numpy's PCG64 (the reference uses RAN2), so the
inputs have the reference's distributions, not its exact draws.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

SMAX = 0.125  # maximum regular step used for STEPR (fpoly0.F:55-56)


@dataclass
class Cluster:
    """FP64 particle set in the layout the gpunb_* ABI takes (C order)."""

    m: np.ndarray            # [N]
    x: np.ndarray            # [N, 3]
    v: np.ndarray            # [N, 3]
    rs: np.ndarray           # [N] neighbour radius RS
    dtr: np.ndarray          # [N] regular step STEPR
    meta: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return int(self.m.shape[0])

    def h2(self, m_flag: int = 0, bodym: float | None = None) -> np.ndarray:
        """GPU_RS of util_gpu.F:46-51: RS**2, or RS**2/BODYM when m_flag."""
        h2 = self.rs * self.rs
        if m_flag:
            h2 = h2 / (bodym if bodym is not None else float(self.m.mean()))
        return h2


# --------------------------------------------------------------------------
# masses

def kroupa_masses(n: int, rng: np.random.Generator, mlo: float = 0.08,
                  mbreak: float = 0.5, mhi: float = 100.0,
                  a1: float = 1.3, a2: float = 2.3) -> np.ndarray:
    """Two-segment Kroupa IMF dN/dm ~ m^-a1 (mlo..mbreak), m^-a2 (mbreak..mhi),
    continuous at the break; masses in Msun."""
    def seg_int(a, lo, hi):
        return (hi ** (1 - a) - lo ** (1 - a)) / (1 - a)
    c2 = mbreak ** (a2 - a1)          # continuity factor for segment 2
    w1 = seg_int(a1, mlo, mbreak)
    w2 = c2 * seg_int(a2, mbreak, mhi)
    u = rng.random(n)
    pick1 = rng.random(n) < w1 / (w1 + w2)
    out = np.empty(n)
    # inverse CDF of m^-a on [lo, hi]
    for sel, a, lo, hi in ((pick1, a1, mlo, mbreak), (~pick1, a2, mbreak, mhi)):
        k = int(sel.sum())
        if k:
            p = 1 - a
            out[sel] = (lo ** p + u[sel] * (hi ** p - lo ** p)) ** (1.0 / p)
    return out


# --------------------------------------------------------------------------
# Plummer (setup.F:62-106)

def _plummer_raw(n: int, rng: np.random.Generator):
    x = np.empty((n, 3))
    v = np.empty((n, 3))
    filled = 0
    while filled < n:
        k = (n - filled) * 2 + 16
        a1 = rng.random(k)
        a1 = a1[a1 >= 1e-10]
        ri = (a1 ** (-2.0 / 3.0) - 1.0) ** (-0.5)
        ri = ri[ri <= 10.0][: n - filled]
        kk = ri.shape[0]
        a2 = rng.random(kk)
        a3 = rng.random(kk)
        z = (1.0 - 2.0 * a2) * ri
        rho = np.sqrt(np.maximum(ri ** 2 - z ** 2, 0.0))
        x[filled:filled + kk, 0] = rho * np.cos(2 * math.pi * a3)
        x[filled:filled + kk, 1] = rho * np.sin(2 * math.pi * a3)
        x[filled:filled + kk, 2] = z
        # speed by rejection: q^2 (1-q^2)^3.5 against 0.1*u
        q = np.empty(kk)
        need = np.arange(kk)
        while need.size:
            a4 = rng.random(need.size)
            a5 = rng.random(need.size)
            ok = 0.1 * a5 <= a4 ** 2 * (1.0 - a4 ** 2) ** 3.5
            q[need[ok]] = a4[ok]
            need = need[~ok]
        a8 = q * math.sqrt(2.0) / (1.0 + ri ** 2) ** 0.25
        a6 = rng.random(kk)
        a7 = rng.random(kk)
        vz = (1.0 - 2.0 * a6) * a8
        vr = np.sqrt(np.maximum(a8 ** 2 - vz ** 2, 0.0))
        v[filled:filled + kk, 0] = vr * np.cos(2 * math.pi * a7)
        v[filled:filled + kk, 1] = vr * np.sin(2 * math.pi * a7)
        v[filled:filled + kk, 2] = vz
        filled += kk
    return x, v


# --------------------------------------------------------------------------
# King W0 model (King 1966 distribution function)

def _king_profile(w0: float, nr: int = 4000):
    """Integrate the King model in King units (r0 = 1, rho(W0) scaled).

    Returns r, W(r), rho(r) (normalised to rho(0) = 1) and M(<r), up to the
    tidal radius where W = 0."""
    from math import erf

    def rho_of_w(w):
        if w <= 0:
            return 0.0
        sw = math.sqrt(w)
        return math.exp(w) * erf(sw) - math.sqrt(4.0 * w / math.pi) * (1.0 + 2.0 * w / 3.0)

    rho0 = rho_of_w(w0)
    # d2W/dr2 + 2/r dW/dr = -9 rho/rho0 (King units: r0^2 = 9 sigma^2/(4 pi G rho0))
    h = 1e-3
    r, w, dw = 1e-6, w0, 0.0
    rs, ws, rhos, ms = [0.0], [w0], [1.0], [0.0]
    mass = 0.0

    def deriv(r_, w_, dw_):
        return dw_, -9.0 * rho_of_w(w_) / rho0 - 2.0 * dw_ / r_

    while w > 0 and r < 1e4:
        # RK4 step
        k1 = deriv(r, w, dw)
        k2 = deriv(r + h / 2, w + h / 2 * k1[0], dw + h / 2 * k1[1])
        k3 = deriv(r + h / 2, w + h / 2 * k2[0], dw + h / 2 * k2[1])
        k4 = deriv(r + h, w + h * k3[0], dw + h * k3[1])
        w_new = w + h / 6 * (k1[0] + 2 * k2[0] + 2 * k3[0] + k4[0])
        dw = dw + h / 6 * (k1[1] + 2 * k2[1] + 2 * k3[1] + k4[1])
        rho_mid = rho_of_w(max(0.5 * (w + w_new), 0.0)) / rho0
        mass += 4.0 * math.pi * (r + h / 2) ** 2 * rho_mid * h
        r += h
        w = w_new
        rs.append(r)
        ws.append(max(w, 0.0))
        rhos.append(rho_of_w(max(w, 0.0)) / rho0)
        ms.append(mass)
        h = min(0.02 * max(r, 0.05), 0.05)
    return np.array(rs), np.array(ws), np.array(rhos), np.array(ms)


def _king_raw(n: int, w0: float, rng: np.random.Generator):
    r_tab, w_tab, rho_tab, m_tab = _king_profile(w0)
    mfrac = m_tab / m_tab[-1]
    u = rng.random(n)
    r = np.interp(u, mfrac, r_tab)
    w = np.interp(r, r_tab, w_tab)
    # speed from f(E) ~ exp(W - v^2/(2 s^2)) - 1 with s = 1 in units of sigma,
    # v in [0, sqrt(2W)]: rejection on v^2 * (exp(W - v^2/2) - 1)
    vmax = np.sqrt(2.0 * w)
    speed = np.zeros(n)
    need = np.arange(n)
    fmax = np.maximum(vmax ** 2 * (np.exp(w) - 1.0), 1e-300) * 1.0001
    while need.size:
        vv = rng.random(need.size) * vmax[need]
        f = vv ** 2 * (np.exp(w[need] - 0.5 * vv ** 2) - 1.0)
        ok = rng.random(need.size) * fmax[need] <= f
        speed[need[ok]] = vv[ok]
        need = need[~ok]
    x = _iso(r, rng)
    v = _iso(speed, rng)
    return x, v, (r_tab, rho_tab, m_tab)


def _iso(mag: np.ndarray, rng: np.random.Generator) -> np.ndarray:
    n = mag.shape[0]
    cz = 1.0 - 2.0 * rng.random(n)
    ph = 2 * math.pi * rng.random(n)
    sz = np.sqrt(np.maximum(1.0 - cz ** 2, 0.0))
    return np.stack([mag * sz * np.cos(ph), mag * sz * np.sin(ph), mag * cz], axis=1)


# --------------------------------------------------------------------------
# energies and Henon scaling (scale.F)

def potential_energy(m: np.ndarray, x: np.ndarray, chunk: int = 2048) -> float:
    """Exact W = -sum_{i<j} m_i m_j / r_ij, O(N^2) in numpy chunks."""
    n = m.shape[0]
    w = 0.0
    for s in range(0, n, chunk):
        xs = x[s:s + chunk]
        d = xs[:, None, :] - x[None, :, :]
        r2 = np.einsum("ijk,ijk->ij", d, d)
        idx = np.arange(s, min(s + chunk, n))
        r2[np.arange(idx.size), idx] = np.inf
        w -= float(np.sum(m[s:s + chunk, None] * m[None, :] / np.sqrt(r2)))
    return 0.5 * w


def henon_scale(m, x, v, w_pot: float | None = None):
    """Centre-of-mass frame, virial velocities (Q = 1/2), then E = -1/4
    (src/Main/scale.F:178-255)."""
    mt = m.sum()
    x = x - (m[:, None] * x).sum(0) / mt
    v = v - (m[:, None] * v).sum(0) / mt
    if w_pot is None:
        w_pot = potential_energy(m, x)
    kin = 0.5 * float(np.sum(m * np.einsum("ij,ij->i", v, v)))
    qv = math.sqrt(0.5 * (-w_pot) / kin)
    v = v * qv
    e = 0.5 * w_pot                       # virial: K = -W/2
    s = -4.0 * e                          # positions *= s gives E = -1/4
    return x * s, v / math.sqrt(s), s


# --------------------------------------------------------------------------
# neighbour radius calibration

def neighbour_counts(x: np.ndarray, rs: np.ndarray, sample: np.ndarray, tree=None) -> np.ndarray:
    """Number of other bodies within RS_i of each sampled body (self excluded).
    KD-tree when scipy is present (pass a prebuilt `tree` of x to reuse it),
    chunked brute force otherwise."""
    try:
        from scipy.spatial import cKDTree
        if tree is None:
            tree = cKDTree(x)
        cnt = tree.query_ball_point(x[sample], rs[sample], return_length=True, workers=-1)
        return np.asarray(cnt) - 1
    except ImportError:  # pragma: no cover - scipy is present on both hosts
        out = np.empty(sample.size, dtype=np.int64)
        for s in range(0, sample.size, 256):
            idx = sample[s:s + 256]
            d = x[idx][:, None, :] - x[None, :, :]
            r2 = np.einsum("ijk,ijk->ij", d, d)
            out[s:s + 256] = (r2 < rs[idx, None] ** 2).sum(1) - 1
        return out


def calibrate_rs(x: np.ndarray, target: float, rng: np.random.Generator,
                 sample_size: int = 4096, k: int = 32) -> np.ndarray:
    """Per-particle RS from the local density: RS_i = c * d_k(i) *
    (target/k)^(1/3), d_k the distance to the k-th nearest other body; the
    single factor c is bisected so that the mean count (self excluded) over a
    sample equals ``target``."""
    n = x.shape[0]
    k = int(min(k, max(n - 1, 1)))
    tree = None
    try:
        from scipy.spatial import cKDTree
        tree = cKDTree(x)
        dk = tree.query(x, k=k + 1, workers=-1)[0][:, -1]
    except ImportError:  # pragma: no cover
        dk = np.empty(n)
        for s in range(0, n, 256):
            d = x[s:s + 256][:, None, :] - x[None, :, :]
            r2 = np.sort(np.einsum("ijk,ijk->ij", d, d), axis=1)
            dk[s:s + 256] = np.sqrt(r2[:, k])
    base = dk * (target / k) ** (1.0 / 3.0)
    sample = np.arange(n) if n <= sample_size else rng.choice(n, sample_size, replace=False)
    lo, hi = 0.3, 3.0
    for it in range(40):
        c = 0.5 * (lo + hi)
        mean = neighbour_counts(x, c * base, sample, tree).mean()
        if mean < target:
            lo = c
        else:
            hi = c
        if it > 8 and abs(mean - target) < 0.005 * target:
            break
    return 0.5 * (lo + hi) * base


def regular_step(x: np.ndarray, smax: float = SMAX) -> np.ndarray:
    r2 = np.einsum("ij,ij->i", x, x)
    return np.minimum(smax / 8.0 * np.sqrt(1.0 + r2), smax)


# --------------------------------------------------------------------------
# public constructors

def plummer(n: int, seed: int, masses: str = "equal", nb_target: float = 50.0,
            exact_energy_max: int = 16384) -> Cluster:
    """Plummer sphere in Henon units (setup.F:62-106 + scale.F)."""
    rng = np.random.default_rng(seed)
    x, v = _plummer_raw(n, rng)
    if masses == "equal":
        m = np.full(n, 1.0 / n)
    elif masses == "kroupa":
        m = kroupa_masses(n, rng)
        m = m / m.sum()
    else:
        raise ValueError(masses)
    # setup.F analytic scaling first (expected Henon units)
    sx = 1.5 * 2 * math.pi / 16.0
    x = x * sx
    v = v * math.sqrt(1.0 / sx)
    w = potential_energy(m, x) if n <= exact_energy_max else None
    if w is None:
        # mean-field value for a Plummer sphere of scale a = 3*pi/16 (G = M = 1):
        # W = -3*pi/32 / a = -1/2
        w = -0.5
    x, v, s = henon_scale(m, x, v, w_pot=w)
    rs = calibrate_rs(x, nb_target, rng)
    dtr = regular_step(x)
    return Cluster(m=m, x=np.ascontiguousarray(x), v=np.ascontiguousarray(v), rs=rs,
                   dtr=dtr, meta={"model": "plummer", "n": n, "seed": seed,
                                  "masses": masses, "nb_target": nb_target})


def king(n: int, seed: int, w0: float = 6.0, binary_fraction: float = 0.1,
         nb_target: float = 100.0) -> Cluster:
    """King W0 model, Kroupa masses, a fraction of bodies being binary centres
    of mass (summed mass of two IMF draws; log-uniform a in 0.1-100 AU and
    thermal e are recorded but do not enter the regular force)."""
    rng = np.random.default_rng(seed)
    x, v, prof = _king_raw(n, w0, rng)
    m = kroupa_masses(n, rng)
    nbin = int(round(binary_fraction * n))
    is_bin = np.zeros(n, dtype=bool)
    if nbin:
        bidx = rng.choice(n, nbin, replace=False)
        is_bin[bidx] = True
        m[bidx] += kroupa_masses(nbin, rng)
        semi_au = np.exp(rng.uniform(math.log(0.1), math.log(100.0), nbin))
        ecc = np.sqrt(rng.random(nbin))          # thermal: f(e) = 2e
    else:
        semi_au = ecc = np.zeros(0)
    m = m / m.sum()
    # mean-field potential energy from the model profile: W = -int G M(r) dm / r
    r_tab, rho_tab, m_tab = prof
    mf = m_tab / m_tab[-1]
    dm = np.diff(mf)
    rmid = 0.5 * (r_tab[1:] + r_tab[:-1])
    rmid[rmid == 0] = 1e-12
    w_model = -float(np.sum(0.5 * (mf[1:] + mf[:-1]) * dm / rmid))
    if n <= 16384:
        w_model = potential_energy(m, x)
    x, v, s = henon_scale(m, x, v, w_pot=w_model)
    rs = calibrate_rs(x, nb_target, rng)
    dtr = regular_step(x)
    return Cluster(m=m, x=np.ascontiguousarray(x), v=np.ascontiguousarray(v), rs=rs,
                   dtr=dtr, meta={"model": "king", "w0": w0, "n": n, "seed": seed,
                                  "binaries": nbin, "is_binary_cm": is_bin,
                                  "semi_au": semi_au, "ecc": ecc,
                                  "nb_target": nb_target})


def active_set(n: int, ni: int, seed: int) -> np.ndarray:
    """First ni of a seeded permutation (the active block of a block step)."""
    rng = np.random.default_rng(seed + 7919)
    return np.sort(rng.permutation(n)[:ni])
