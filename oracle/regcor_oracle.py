"""Host restatement of the reference's regular corrector REGCOR_GPU
(src/Main/regcor_gpu.F), TEST INFRASTRUCTURE ONLY: the checker of the
device corrector gpunb_regcor_device.  Plain Python, one body at a time, FP64,
following the Fortran control flow line by line (one deviation, marked where
it occurs: the insertion of a kept neighbour into an empty new list): the
neighbour-radius rule
(:120-252), the list comparison with its sentinels and JJLIST bookkeeping
(:262-330), the retention of small-step neighbours (:332-410), the force
changes of lost and gained neighbours (:414-460), the corrector (:462-552),
the list copy (:608-616) and the step selection (:618-800).  The parts the
device corrector leaves to the caller (XTRNLF, FCLOUD, CHECKL, FPCORR, ETIDE)
are left out here too.

State: a dict of numpy arrays over all NTOT bodies in the Fortran COMMON
layout (index I-1, vectors [NTOT, 3]): x, xdot, body, h (KS pairs, or None),
x0, x0dot, t0r, stepr, step, t0, timenw, fi, fidot, fr, frdot, d0, d0r, d1r,
d2r, d3r, xn, xndot, rs, and list [NTOT, LMAX] (count, then 1-based members).
Parameters: a dict with time, dtmin, smin, smax, etar, tidal4, kz14, m_flag,
nnbmax, n, ntot, ifirst, lmax and the RS-rule fields nnbopt, nb_flag, rscale,
rc, rsfac, bodym, rdens.
"""
from __future__ import annotations

import math

import numpy as np


def _pair(xi, vi, xj, vj, mj):
    a = [xj[k] - xi[k] for k in range(3)]
    dv = [vj[k] - vi[k] for k in range(3)]
    rij2 = a[0] * a[0] + a[1] * a[1] + a[2] * a[2]
    dr2i = 1.0 / rij2
    dr3i = mj * dr2i * math.sqrt(dr2i)
    drdv = a[0] * dv[0] + a[1] * dv[1] + a[2] * dv[2]
    drdp = 3.0 * drdv * dr2i
    return [a[k] * dr3i for k in range(3)], [(dv[k] - a[k] * drdp) * dr3i for k in range(3)]


def regcor_body(i1, freg, fdr, nlist, s, p, counters, step_entry=None):
    """One body I = i1 (1-based).  freg, fdr: 3-lists (modified as the
    reference modifies FREG, FDR); nlist: Python list in the LISTGP row form
    [NNB, members...] (modified as NLIST is).  step_entry: STEP of all bodies
    as it was when the block started (default: s["step"]); the small-step
    tests read the neighbours' STEP from it."""
    i = i1 - 1
    step_nb = s["step"] if step_entry is None else step_entry
    lmax = p["lmax"]
    ntot = p["ntot"]
    xi = [float(s["x"][i, k]) for k in range(3)]
    vi = [float(s["xdot"][i, k]) for k in range(3)]
    nnb = nlist[0]
    lst = s["list"][i]                       # LIST(.,I), 0-based positions
    nnb0 = int(lst[0])
    dtr = p["time"] - s["t0r"][i]
    irskip = 0
    rdens = p["rdens"]
    if p["nb_flag"]:
        ri2 = sum((xi[k] - rdens[k]) ** 2 for k in range(3))
        rh2 = p["rscale"] ** 2
    else:
        ri2 = xi[0] ** 2 + xi[1] ** 2 + xi[2] ** 2
        rh2 = 9.0 * p["rscale"] ** 2
    rs2 = s["rs"][i] ** 2
    znbmin = max(0.01 * p["nnbmax"], 1.0)
    dfirr = [0.0, 0.0, 0.0]
    dfd = [0.0, 0.0, 0.0]
    if nnb == 0:                             # :120-143
        r2 = xi[0] ** 2 + xi[1] ** 2 + xi[2] ** 2
        fij = 0.01 * p["bodym"] / (r2 * math.sqrt(r2))
        rdot = 3.0 * (xi[0] * vi[0] + xi[1] * vi[1] + xi[2] * vi[2]) / r2
        for k in range(3):
            dfirr[k] = -fij * xi[k]
            dfd[k] = -(vi[k] - rdot * xi[k]) * fij
        if rdot > 0.0:
            s["rs"][i] = max(0.75 * s["rs"][i], 0.1 * p["rscale"])
        else:
            s["rs"][i] = 1.1 * s["rs"][i]
        counters[0] += 1
        irskip = 1
    else:
        fac = 1.0 + 0.1 * (float(p["nnbopt"]) - float(nnb)) / float(nnb)   # :152
        a3 = float(nnb) * fac
        nbave = min(p["nnbopt"] + 150, max(p["nnbmax"] - 50, int(znbmin)))
        a3 = min(a3, 0.9 * nbave)
        nbp = int(a3)
        if ri2 > rh2 and p["nb_flag"]:
            a3 = a3 * max(p["rscale"] / math.sqrt(ri2), 0.1)
        else:
            a3 = max(a3, znbmin)
        a4 = a3 / float(nnb)
        if (a3 - float(nnb0)) * (a3 - float(nnb)) < 0.0:
            a4 = math.sqrt(a4)
        ridot = sum((xi[k] - rdens[k]) * vi[k] for k in range(3))
        if ri2 > p["rc"] ** 2 and p["nb_flag"] and ri2 < 100.0 * rh2:
            a4 = a4 * (1.0 + ridot * dtr / ri2)
        if i1 > p["n"] and ri2 <= rh2 and s.get("h") is not None:     # :182-193
            hh = abs(s["h"][i1 - p["n"] - 1])
            a2 = 100.0 * s["body"][i] / hh if hh > 0.0 else math.inf
            if a2 > s["rs"][i]:
                a3 = max(1.0 - float(nnb) / nbave, 0.0)
                a4 = 1.0 + 0.5 * a3
        a5 = min(p["rsfac"] * dtr, 0.25)
        a4 = a4 - 1.0
        if a4 > a5:
            a4 = a5
        else:
            a4 = max(a4, -a5)
        if irskip == 0:
            a3 = a4 / 3.0
            a1 = 1.0 + a3 - a3 * a3
            if nnb < znbmin and nbp > znbmin:
                if a1 < 1.0:
                    a1 = 1.05
            if abs(a1 - 1.0) > 0.003:
                if s["rs"][i] ** 2 > ri2 and s["rs"][i] ** 2 < 2.0 * ri2 and nnb > 5:
                    a1 = math.sqrt(a1)
                s["rs"][i] = a1 * s["rs"][i]
            if nnb > nbave:
                if ridot < 0.0:
                    drs = (float(nnb) - nbave) / (3.0 * nnb)
                    s["rs"][i] = s["rs"][i] * (1.0 - drs)
        if p["m_flag"] == 0:                 # :237-252
            if nnb <= 3 and ri2 < 100.0 * rh2:
                a1 = 2.0 * s["rs"][i]
                for l in range(1, nnb + 1):
                    j = nlist[l] - 1
                    e = [xi[k] - s["x"][j, k] for k in range(3)]
                    rij = math.sqrt(e[0] ** 2 + e[1] ** 2 + e[2] ** 2)
                    rsdot = sum(e[k] * (vi[k] - s["xdot"][j, k]) for k in range(3)) / rij
                    a1 = min(a1, rij + rsdot * dtr)
                s["rs"][i] = max(a1, 1.1 * s["rs"][i])
        dfirr = [0.0, 0.0, 0.0]
        dfd = [0.0, 0.0, 0.0]

    # :262 onwards -- lists as Fortran arrays with 1-based positions
    L_ = [0] + [int(v) for v in lst[:lmax]]          # L_[q] = LIST(q, I), q = 1..lmax
    NL = [0] + list(nlist) + [0] * (lmax + 2 - len(nlist))   # NL[q] = NLIST(q)
    jj = [0] * (2 * lmax + 2)                         # JJLIST(1..)
    nbloss = nbgain = 0
    if nnb0 == 0:
        nbgain = nnb
        for l in range(1, nnb + 1):
            jj[l] = NL[l + 1]
    else:
        jmin = 0
        L, LG = 2, 2
        NL[nnb + 2] = ntot + 1
        NL[1] = L_[nnb0 + 1]
        while True:                                   # label 56
            if L_[L] != NL[LG]:
                if L_[L] >= NL[LG]:
                    nbgain += 1
                    jj[nnb0 + nbgain] = NL[LG]
                    L -= 1
                else:
                    nbloss += 1
                    j = L_[L]
                    jj[nbloss] = j
                    if step_nb[j - 1] < p["smin"]:
                        jmin = j
                    LG -= 1
            if L <= nnb0:                             # label 58
                L += 1
                LG += 1
                continue
            elif LG <= nnb:
                LG += 1
                L_[L] = ntot + 1
                continue
            break
        if jmin != 0:
            K = 1
            while True:                               # label 60
                if nnb > p["nnbmax"] or i1 > p["n"]:
                    break
                j = jj[K]
                skip = (step_nb[j - 1] > p["smin"] or j < p["ifirst"] or j > p["n"])
                if not skip:
                    rij2 = sum((xi[k] - s["x"][j - 1, k]) ** 2 for k in range(3))
                    skip = rij2 > 4.0 * rs2
                if not skip:
                    L = nnb + 1
                    # With NNB = 0 the reference's loop starts at L = 1 and
                    # compares NLIST(1), which then holds the saved last old
                    # member: the first kept body is displaced by that member
                    # (:386-392), leaving the list and the force split
                    # inconsistent.  Here, as on the device, a body is
                    # inserted into an empty list like into any other.
                    while L > 1:                      # label 62
                        if NL[L] < j:
                            break
                        NL[L + 1] = NL[L]
                        L -= 1
                    NL[L + 1] = j                     # label 64
                    nnb += 1
                    nbloss -= 1
                    L_[nnb0 + 1] = NL[1]
                    counters[1] += 1
                    f, fd = _pair(xi, vi, s["x"][j - 1], s["xdot"][j - 1], s["body"][j - 1])
                    for k in range(3):
                        freg[k] -= f[k]
                        fdr[k] -= fd[k]
                    if K > nbloss:
                        break
                    for l in range(K, nbloss + 1):
                        jj[l] = jj[l + 1]
                    K -= 1
                K += 1                                # label 68
                if K > nbloss:
                    break
    for l in range(1, nbloss + 1):                    # label 70
        j = jj[l]
        f, fd = _pair(xi, vi, s["x"][j - 1], s["xdot"][j - 1], s["body"][j - 1])
        for k in range(3):
            dfirr[k] -= f[k]
            dfd[k] -= fd[k]
    for l in range(1, nbgain + 1):
        j = jj[nnb0 + l]
        f, fd = _pair(xi, vi, s["x"][j - 1], s["xdot"][j - 1], s["body"][j - 1])
        for k in range(3):
            dfirr[k] += f[k]
            dfd[k] += fd[k]
    dtsq = dtr ** 2
    dt6 = 6.0 / (dtr * dtsq)
    dt2 = 2.0 / dtsq
    dtsq12 = dtsq / 12.0
    dtr13 = dtr / 3.0
    s["t0r"][i] = p["time"]
    if s["step"][i] < 5.0 * p["dtmin"] and dtr > 50.0 * s["step"][i]:
        dtr13 = 0.0
        dtsq12 = 0.0
    for k in range(3):
        dfr = s["fr"][i, k] - freg[k] - dfirr[k]
        fdr0 = fdr[k] + dfd[k]
        frd = s["frdot"][i, k]
        sm = frd + fdr0
        at3 = 2.0 * dfr + dtr * sm
        bt2 = -3.0 * dfr - dtr * (sm + frd)
        s["xn"][i, k] = s["x0"][i, k] + (0.6 * at3 + bt2) * dtsq12
        s["xndot"][i, k] = s["x0dot"][i, k] + (0.75 * at3 + bt2) * dtr13
        s["fi"][i, k] += dfirr[k]
        s["fr"][i, k] = freg[k]
        s["fidot"][i, k] += dfd[k]
        s["frdot"][i, k] = fdr[k]
        if p["kz14"] <= 2:
            if k == 1:
                s["fidot"][i, 0] -= p["tidal4"] * dfr
            if k == 0:
                s["fidot"][i, 1] += p["tidal4"] * dfr
        s["d0"][i, k] = s["fi"][i, k]
        s["d0r"][i, k] = freg[k]
        s["d1r"][i, k] = fdr[k]
        s["d3r"][i, k] = at3 * dt6
        s["d2r"][i, k] = (3.0 * at3 + bt2) * dt2
    if nbloss + nbgain > 0:                           # :608-616
        L_[1] = nnb
        for l in range(2, nnb + 2):
            L_[l] = NL[l]
        counters[2] += nbloss + nbgain
    s["list"][i, :] = L_[1:lmax + 1]
    nlist[:] = [nnb] + NL[2:nnb + 2]
    fr2 = freg[0] ** 2 + freg[1] ** 2 + freg[2] ** 2  # :618
    w1 = fdr[0] ** 2 + fdr[1] ** 2 + fdr[2] ** 2
    w2 = float(np.sum(s["d2r"][i] ** 2))
    w3 = float(np.sum(s["d3r"][i] ** 2))
    w0 = (math.sqrt(fr2 * w2) + w1) / (math.sqrt(w1 * w3) + w2)
    w0 = p["etar"] * w0
    ttmp = math.sqrt(w0)
    dt0 = ttmp
    t = p["time"]
    if ttmp > 2.0 * s["stepr"][i]:
        if math.fmod(t, 2.0 * dtr) == 0.0:
            ttmp = min(2.0 * dtr, p["smax"])
            while dt0 > 2.0 * ttmp and 2.0 * ttmp < p["smax"] and math.fmod(t, 2.0 * ttmp) == 0.0:
                ttmp = 2.0 * ttmp
        else:
            ttmp = s["stepr"][i]
    elif ttmp < dtr:
        ttmp = 0.5 * dtr
        if ttmp > dt0:
            ttmp = 0.5 * ttmp
    else:
        ttmp = s["stepr"][i]
    if ttmp > 0.1 and ttmp > dtr:
        dv2 = sum((vi[k] - s["xndot"][i, k]) ** 2 for k in range(3))
        dtj = dtr * (1.0e-4 * dtr ** 2 * fr2 / dv2) ** 0.1
        if dtj < ttmp:
            ttmp = dtr
    ttmp = min(ttmp, p["smax"])
    s["stepr"][i] = ttmp
    if nnb0 == 0 and nnb >= 0:
        s["step"][i] = 0.125 * s["step"][i]
        s["timenw"][i] = s["t0"][i] + s["step"][i]
    while ttmp < s["step"][i]:                        # label 110
        s["step"][i] = 0.5 * s["step"][i]
        s["timenw"][i] = s["t0"][i] + s["step"][i]
        counters[3] += 1


def regcor_block(iact, freg, fdr, nlist_rows, s, p):
    """All bodies of an active block in order; freg, fdr [ni, 3] and
    nlist_rows [ni, lmax] are modified like the device corrector's inputs.
    The neighbours' STEP is read as it was at the start of the block (the
    reference's OpenMP loop leaves that order open; the device corrector
    defines it so).  Returns the counters (NBVOID, NBSMIN, NBFLUX, NICONV)."""
    counters = [0, 0, 0, 0]
    step_entry = s["step"].copy()
    for k, i1 in enumerate(iact):
        fr = [float(v) for v in freg[k]]
        fd = [float(v) for v in fdr[k]]
        row = [int(v) for v in nlist_rows[k, :int(nlist_rows[k, 0]) + 1]]
        regcor_body(int(i1), fr, fd, row, s, p, counters, step_entry)
        freg[k] = fr
        fdr[k] = fd
        nlist_rows[k, :] = 0
        nlist_rows[k, :len(row)] = row
    return counters
