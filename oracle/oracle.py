"""ctypes front end of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
module, as the checker or the timed CPU baseline; the product never imports it.

    regf_fp64(...)  FP64 truth with the gpunb_regf_ contract (oracle_fp64.c)
    pot_fp64(...)   FP64 gpupot_ semantics
    Port            portable FP32 restatement of src/Main/reg.avx.cpp / pot.avx.cpp
    RefAVX          the reference's own reg.avx.cpp / pot.avx.cpp compiled from
                    its sources into oracle/_ref (x86_64 hosts only)
    irr_fp64(...)   FP64 irregular force of src/Main/irr.avx.cpp (irr_fp64.c)
    irr_abs_sums()  its per-particle sums of pair-term magnitudes (parity bound)
    RefIrrAVX       the reference's own irr.avx.cpp compiled into oracle/_ref
"""
from __future__ import annotations

import ctypes as C
import os
import platform
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int)
_lib = None


def build(ref_dir: str | os.PathLike | None = None) -> None:
    """make liboracle.so, and the reference AVX libraries when ref_dir names
    the reference's source tree (x86_64 hosts only)."""
    subprocess.run(["make", "-s", "-C", str(HERE), "liboracle.so"], check=True)
    if ref_dir and platform.machine() == "x86_64" and Path(ref_dir).joinpath(
            "src/Main/reg.avx.cpp").exists():
        subprocess.run(["make", "-s", "-C", str(HERE), "ref", f"REF={ref_dir}"], check=True,
                       capture_output=True)


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        path = HERE / "liboracle.so"
        srcs = [HERE / "oracle_fp64.c", HERE / "port_fp32.c", HERE / "irr_fp64.c",
                HERE / "Makefile"]
        if not path.exists() or any(s.stat().st_mtime > path.stat().st_mtime for s in srcs):
            build()
        _lib = C.CDLL(str(path))
        _lib.oracle_regf_fp64.argtypes = [C.c_int, _D, _D, _D, C.c_int, _D, _D, _D, _D, _D, _D,
                                          _D, C.c_int, C.c_int, _I, C.c_int, _D, _D]
        _lib.oracle_pot_fp64.argtypes = [C.c_int, C.c_int, C.c_int, _D, _D, _D]
        _lib.port_send_fp32.argtypes = [C.c_int, _D, _D, _D]
        _lib.port_regf_fp32.argtypes = [C.c_int, _D, _D, _D, _D, _D, _D, _D, C.c_int, C.c_int,
                                        _I, C.c_int]
        _lib.port_pot_fp32.argtypes = [C.c_int, C.c_int, C.c_int, _D, _D, _D]
        _lib.oracle_num_threads.restype = C.c_int
        _lib.oracle_irr_fp64.argtypes = [C.c_int, _D, _D, _D, _D, _D, _D, C.c_int, _I, C.c_double,
                                         C.c_int, _I, _D, _D, _I]
    return _lib


def _c(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a.reshape(shape) if shape is not None else a


def _dp(a):
    return a.ctypes.data_as(_D)


def num_threads() -> int:
    return lib().oracle_num_threads()


def regf_fp64(m, x, v, h2, dtr, xi, vi, lmax, nnbmax, m_flag=0, with_abs=False):
    """FP64 oracle of gpunb_regf_ against the j-set (m, x, v).
    Returns acc, jrk, pot, list [, accabs, jrkabs]."""
    m = _c(m); n = m.shape[0]
    x = _c(x, (n, 3)); v = _c(v, (n, 3))
    h2 = _c(h2); ni = h2.shape[0]
    dtr = _c(dtr, (ni,)); xi = _c(xi, (ni, 3)); vi = _c(vi, (ni, 3))
    acc = np.empty((ni, 3)); jrk = np.empty((ni, 3)); pot = np.empty(ni)
    lst = np.zeros((ni, lmax), dtype=np.int32)
    aa = np.empty(ni); ja = np.empty(ni)
    lib().oracle_regf_fp64(n, _dp(m), _dp(x), _dp(v), ni, _dp(h2), _dp(dtr), _dp(xi), _dp(vi),
                           _dp(acc), _dp(jrk), _dp(pot), lmax, nnbmax,
                           lst.ctypes.data_as(_I), int(m_flag), _dp(aa), _dp(ja))
    if with_abs:
        return acc, jrk, pot, lst, aa, ja
    return acc, jrk, pot, lst


def pot_fp64(m, x, istart=1, ni=None):
    m = _c(m); n = m.shape[0]; x = _c(x, (n, 3))
    if ni is None:
        ni = n - istart + 1
    pot = np.empty(ni)
    lib().oracle_pot_fp64(int(istart), int(ni), n, _dp(m), _dp(x), _dp(pot))
    return pot


# ---------------------------------------------------------------------------
# Parity bound of the split-precision regular force (the FP64 oracle as truth).
#
# A regular force or jerk is a sum of N pair terms q_ij.  FP32 arithmetic
# errs per term by a few units of 2^-24 of |q_ij|, so the error of the sum
# scales with S_i = sum_j |q_ij|, not with |Q_i|: for a particle whose terms
# cancel (kappa_i = S_i / |Q_i| large) the plain relative error grows with
# kappa_i whatever the FP32 formulation.  The bound therefore measures each
# particle against max(|Q_i|, S_i / KAPPA0): the plain relative error
# wherever the sum cancels by less than KAPPA0, and 1e-6 S_i / KAPPA0 for a
# residue of stronger cancellation.  The potential (all terms positive) is
# held to the plain relative error.
SPLIT_TOL = 1e-6
KAPPA0 = 8.0


def parity_errors(acc, jrk, pot, ref_acc, ref_jrk, ref_pot, accabs, jrkabs) -> dict:
    """Per-particle errors of (acc, jrk, pot) against the FP64 oracle's
    (ref_acc, ref_jrk, ref_pot) with its term sums accabs, jrkabs (the
    with_abs outputs of regf_fp64).  Returns the plain relative maxima and
    99th percentiles, the cancellation-aware maxima (the bound), the maxima
    normalised by S_i, and the particles above SPLIT_TOL in plain terms with
    the smallest cancellation ratio among them."""
    acc, jrk, ref_acc, ref_jrk = (np.asarray(a, dtype=np.float64).reshape(-1, 3)
                                  for a in (acc, jrk, ref_acc, ref_jrk))
    pot, ref_pot, accabs, jrkabs = (np.asarray(a, dtype=np.float64).ravel()
                                    for a in (pot, ref_pot, accabs, jrkabs))
    out = {"n": int(acc.shape[0]), "kappa0": KAPPA0}
    for name, got, ref, s in (("acc", acc, ref_acc, accabs), ("jrk", jrk, ref_jrk, jrkabs)):
        d = np.linalg.norm(got - ref, axis=1)
        q = np.linalg.norm(ref, axis=1)
        rel = d / np.maximum(q, 1e-300)
        kap = s / np.maximum(q, 1e-300)
        bound = d / np.maximum(np.maximum(q, s / KAPPA0), 1e-300)
        above = rel > SPLIT_TOL
        out[name] = {"max": float(rel.max()), "p99": float(np.percentile(rel, 99)),
                     "bound_max": float(bound.max()),
                     "sum_norm_max": float((d / np.maximum(s, 1e-300)).max()),
                     "above_tol": int(above.sum()),
                     "min_kappa_above_tol": float(kap[above].min()) if above.any() else None}
    ep = np.abs(pot - ref_pot) / np.maximum(np.abs(ref_pot), 1e-300)
    out["pot"] = {"max": float(ep.max()), "p99": float(np.percentile(ep, 99))}
    return out


class Port:
    """Portable FP32 restatement of the reference CPU path (the CPU baseline)."""

    def send(self, m, x, v):
        m = _c(m); n = m.shape[0]
        self._keep = (m, _c(x, (n, 3)), _c(v, (n, 3)))
        lib().port_send_fp32(n, _dp(self._keep[0]), _dp(self._keep[1]), _dp(self._keep[2]))

    def regf(self, h2, dtr, xi, vi, lmax, nnbmax, m_flag=0):
        h2 = _c(h2); ni = h2.shape[0]
        dtr = _c(dtr, (ni,)); xi = _c(xi, (ni, 3)); vi = _c(vi, (ni, 3))
        acc = np.empty((ni, 3)); jrk = np.empty((ni, 3)); pot = np.empty(ni)
        lst = np.zeros((ni, lmax), dtype=np.int32)
        lib().port_regf_fp32(ni, _dp(h2), _dp(dtr), _dp(xi), _dp(vi), _dp(acc), _dp(jrk),
                             _dp(pot), lmax, nnbmax, lst.ctypes.data_as(_I), int(m_flag))
        return acc, jrk, pot, lst

    @staticmethod
    def pot(m, x, istart=1, ni=None):
        m = _c(m); n = m.shape[0]; x = _c(x, (n, 3))
        if ni is None:
            ni = n - istart + 1
        pot = np.empty(ni)
        lib().port_pot_fp32(int(istart), int(ni), n, _dp(m), _dp(x), _dp(pot))
        return pot


class RefAVX:
    """The reference's own CPU regular-force and potential code, compiled from
    src/Main/reg.avx.cpp and pot.avx.cpp into oracle/_ref (x86_64 only)."""

    REG = HERE / "_ref" / "libref_reg_avx.so"
    POT = HERE / "_ref" / "libref_pot_avx.so"

    @classmethod
    def available(cls) -> bool:
        return cls.REG.exists() and cls.POT.exists() and platform.machine() == "x86_64"

    def __init__(self, nbmax: int):
        self.reg = C.CDLL(str(self.REG))
        self.potlib = C.CDLL(str(self.POT))
        ip = C.POINTER(C.c_int)
        self.reg.gpunb_open_.argtypes = [ip, ip]
        self.reg.gpunb_send_.argtypes = [ip, _D, _D, _D]
        self.reg.gpunb_regf_.argtypes = [ip, _D, _D, _D, _D, _D, _D, _D, ip, ip, ip, ip]
        self.potlib.gpupot_.argtypes = [ip, ip, ip, ip, _D, _D, _D]
        a, r = C.c_int(nbmax), C.c_int(0)
        self.reg.gpunb_open_(C.byref(a), C.byref(r))

    def close(self):
        self.reg.gpunb_close_()

    def send(self, m, x, v):
        m = _c(m); n = m.shape[0]
        self._keep = (m, _c(x, (n, 3)), _c(v, (n, 3)))
        nj = C.c_int(n)
        self.reg.gpunb_send_(C.byref(nj), *[_dp(a) for a in self._keep])

    def regf(self, h2, dtr, xi, vi, lmax, nnbmax, m_flag=0):
        """The AVX loop reads and writes i in groups of 4: pad the arrays."""
        h2 = _c(h2); ni = h2.shape[0]
        pad = (ni + 3) // 4 * 4 + 4
        def padded(a, shape):
            out = np.zeros(shape)
            out[:ni] = a
            return out
        h2p = padded(h2, (pad,)); dtp = padded(_c(dtr, (ni,)), (pad,))
        xp = padded(_c(xi, (ni, 3)), (pad, 3)); vp = padded(_c(vi, (ni, 3)), (pad, 3))
        acc = np.zeros((pad, 3)); jrk = np.zeros((pad, 3)); pot = np.zeros(pad)
        lst = np.zeros((pad, lmax), dtype=np.int32)
        a = [C.c_int(ni), C.c_int(lmax), C.c_int(nnbmax), C.c_int(m_flag)]
        self.reg.gpunb_regf_(C.byref(a[0]), _dp(h2p), _dp(dtp), _dp(xp), _dp(vp), _dp(acc),
                             _dp(jrk), _dp(pot), C.byref(a[1]), C.byref(a[2]),
                             lst.ctypes.data_as(_I), C.byref(a[3]))
        return acc[:ni], jrk[:ni], pot[:ni], lst[:ni]

    def pot(self, m, x, istart=1, ni=None):
        """pot.avx.cpp reads particles and writes results 8 at a time, and
        indexes its output by absolute i (pot.avx.cpp:87-137), unlike the GPU
        version (gpupot.gpu.cu:101-105) whose output starts at istart; the
        result is returned istart-relative here."""
        m = _c(m); n = m.shape[0]
        if ni is None:
            ni = n - istart + 1
        mp = np.zeros(n + 16); mp[:n] = m
        xp = np.zeros((n + 16, 3)); xp[:n] = _c(x, (n, 3))
        pot = np.zeros(istart - 1 + ni + 16)
        a = [C.c_int(0), C.c_int(istart), C.c_int(ni), C.c_int(n)]
        self.potlib.gpupot_(*[C.byref(v) for v in a], _dp(mp), _dp(xp), _dp(pot))
        return pot[istart - 1:istart - 1 + ni]


def irr_fp64(x0, v0, a2, j6, m, t0, lists, ti, addr):
    """FP64 irregular force (irr.avx.cpp semantics) of the particles addr
    (0-based) at time ti; lists[n][lmax]: count then 0-based ids.
    Returns acc [ni, 3], jrk [ni, 3], nnbid [ni] (1-based, 0 if no list)."""
    m = _c(m); n = m.shape[0]
    x0 = _c(x0, (n, 3)); v0 = _c(v0, (n, 3)); a2 = _c(a2, (n, 3)); j6 = _c(j6, (n, 3))
    t0 = _c(t0)
    lists = np.ascontiguousarray(lists, dtype=np.int32)
    addr = np.ascontiguousarray(addr, dtype=np.int32)
    ni = addr.shape[0]
    acc = np.empty((ni, 3)); jrk = np.empty((ni, 3)); nid = np.empty(ni, dtype=np.int32)
    lib().oracle_irr_fp64(n, _dp(x0), _dp(v0), _dp(a2), _dp(j6), _dp(m), _dp(t0),
                          lists.shape[1], lists.ctypes.data_as(_I), float(ti), ni,
                          addr.ctypes.data_as(_I), _dp(acc), _dp(jrk), nid.ctypes.data_as(_I))
    return acc, jrk, nid


def irr_abs_sums(x0, v0, a2, j6, m, t0, lists, ti, addr):
    """Sums of the magnitudes of the pair terms of the irregular force and
    of its derivative, S_i = sum_j |q_ij|, for the particles addr (the same
    prediction and terms as irr_fp64; listed bodies at zero distance add
    nothing).  With them, parity_errors gives the cancellation-aware bound
    of the split-precision irregular force.  FP64 numpy, rows processed in
    chunks."""
    m = np.asarray(m, dtype=np.float64)
    n = m.shape[0]
    x0, v0, a2, j6 = (np.asarray(a, dtype=np.float64).reshape(n, 3) for a in (x0, v0, a2, j6))
    dt = (float(ti) - np.asarray(t0, dtype=np.float64))[:, None]
    x = x0 + dt * (v0 + dt * (a2 + dt * j6))            # irr.avx.cpp:162-176
    v = v0 + 2.0 * dt * (a2 + 1.5 * dt * j6)
    lists = np.asarray(lists)
    addr = np.asarray(addr, dtype=np.int64)
    accabs = np.zeros(addr.shape[0])
    jrkabs = np.zeros(addr.shape[0])
    lmax = lists.shape[1]
    for s in range(0, addr.shape[0], 1024):
        a = addr[s:s + 1024]
        cnt = np.maximum(lists[a, 0], 0)
        w = int(min(max(int(cnt.max()) if cnt.size else 0, 1), lmax - 1))
        k = np.arange(1, w + 1)[None, :]
        valid = k <= cnt[:, None]
        j = np.where(valid, lists[a, 1:w + 1], 0)
        dx = x[j] - x[a][:, None, :]
        dv = v[j] - v[a][:, None, :]
        r2 = np.einsum("ijk,ijk->ij", dx, dx)
        use = valid & (r2 > 0.0)
        r2s = np.where(use, r2, 1.0)
        rinv = 1.0 / np.sqrt(r2s)
        mr3 = np.where(use, m[j] * rinv ** 3, 0.0)
        al = -3.0 * np.einsum("ijk,ijk->ij", dx, dv) * rinv ** 2
        accabs[s:s + 1024] = (mr3 * np.sqrt(r2s)).sum(axis=1)
        jt = mr3[:, :, None] * (dv + al[:, :, None] * dx)
        jrkabs[s:s + 1024] = np.linalg.norm(jt, axis=2).sum(axis=1)
    return accabs, jrkabs


class RefIrrAVX:
    """The reference's src/Main/irr.avx.cpp built into oracle/_ref (x86_64
    only), driven through its own Fortran-style entry points (1-based
    addresses and ids)."""

    PATH = HERE / "_ref" / "libref_irr_avx.so"

    @classmethod
    def available(cls) -> bool:
        return cls.PATH.exists()

    def __init__(self, nmax: int, lmax: int):
        self.lib = C.CDLL(str(self.PATH))
        for name in ("irr_simd_open_", "irr_simd_close_", "irr_simd_set_jp_",
                     "irr_simd_set_list_", "irr_simd_firr_vec_"):
            getattr(self.lib, name).restype = None
        self.nmax, self.lmax = nmax, lmax
        self.lib.irr_simd_open_(C.byref(C.c_int(nmax)), C.byref(C.c_int(lmax)),
                                C.byref(C.c_int(0)))

    def close(self):
        self.lib.irr_simd_close_(C.byref(C.c_int(0)))

    def set_jp(self, x0, v0, a2, j6, m, t0):
        n = len(m)
        for i in range(n):
            xs = [np.ascontiguousarray(a[i], dtype=np.float64) for a in (x0, v0, a2, j6)]
            self.lib.irr_simd_set_jp_(C.byref(C.c_int(i + 1)), *[_dp(a) for a in xs],
                                      C.byref(C.c_double(m[i])), C.byref(C.c_double(t0[i])))

    def set_lists(self, lists):
        """lists[n][lmax] with 0-based ids; passed as the Fortran LIST rows
        (count, then 1-based ids)."""
        for i in range(lists.shape[0]):
            row = np.ascontiguousarray(lists[i], dtype=np.int32).copy()
            c = int(row[0])
            row[1:1 + c] += 1
            # the library reads whole groups of 8 ids
            buf = np.zeros(1 + 8 * ((c + 7) // 8 + 1), dtype=np.int32)
            buf[:1 + c] = row[:1 + c]
            self.lib.irr_simd_set_list_(C.byref(C.c_int(i + 1)), buf.ctypes.data_as(_I))

    def firr(self, ti, addr):
        a = np.ascontiguousarray(np.asarray(addr) + 1, dtype=np.int32)
        ni = a.shape[0]
        acc = np.empty((ni, 3)); jrk = np.empty((ni, 3)); nid = np.empty(ni, dtype=np.int32)
        self.lib.irr_simd_firr_vec_(C.byref(C.c_double(ti)), C.byref(C.c_int(ni)),
                                    a.ctypes.data_as(_I), _dp(acc), _dp(jrk),
                                    nid.ctypes.data_as(_I))
        return acc, jrk, nid
