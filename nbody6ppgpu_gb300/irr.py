"""Python binding of the GPU irregular-force library (include/irr.h), the
drop-in for NBODY6++'s SIMD library src/Main/irr.avx.cpp.

    with IrrSimd(nmax, lmax) as irr:
        irr.set_jp(x0, v0, f, fdot, m, t0)        # all particles (or a subset)
        irr.set_lists(lists)                      # rows: count, 0-based ids
        acc, jrk, nnbid = irr.firr(ti, active)    # 0-based active indices

The calls go through the reference's own Fortran-style entry points
(1-based addresses and ids), one particle per set call, as the Fortran
integrator makes them.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from .gpunb import GpunbError, _check, load

_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int)


def _dp(a):
    return a.ctypes.data_as(_D)


def _bind(lib):
    for name, args, res in [
        ("irr_simd_open_", [_I, _I, _I], None),
        ("irr_simd_close_", [_I], None),
        ("irr_simd_profile_", [_I], None),
        ("irr_simd_set_jp_", [_I, _D, _D, _D, _D, _D, _D], None),
        ("irr_simd_set_list_", [_I, _I], None),
        ("irr_simd_firr_vec_", [_D, _I, _I, _D, _D, _I], None),
        ("irr_set_host_path", [C.c_int], C.c_int),
        ("irr_set_precision", [C.c_int], C.c_int),
    ]:
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = res


class IrrSimd:
    """One open irregular-force library (the process-wide state of the C ABI)."""

    def __init__(self, nmax: int, lmax: int, rank: int = 0, precision: int | None = None):
        self.lib = load()
        _bind(self.lib)
        if precision is not None:
            self.lib.irr_set_precision(int(precision))
        self.nmax, self.lmax = nmax, lmax
        self.lib.irr_simd_open_(C.byref(C.c_int(nmax)), C.byref(C.c_int(lmax)),
                                C.byref(C.c_int(rank)))
        _check(self.lib)

    def close(self) -> None:
        self.lib.irr_simd_close_(C.byref(C.c_int(0)))
        _check(self.lib)

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_host_path(self, direct: bool) -> int:
        return self.lib.irr_set_host_path(1 if direct else 0)

    def set_precision(self, mode: int) -> int:
        """irr_set_precision: 2 = double-float (the default), 1 = FP64, 0 = split FP32."""
        return self.lib.irr_set_precision(int(mode))

    def set_jp(self, x0, v0, f, fdot, m, t0, idx=None) -> None:
        """irr_simd_set_jp_ for the particles idx (0-based; default all):
        position, velocity, F (force/2), FDOT (derivative/6), mass, time."""
        x0 = np.ascontiguousarray(x0, dtype=np.float64)
        v0 = np.ascontiguousarray(v0, dtype=np.float64)
        f = np.ascontiguousarray(f, dtype=np.float64)
        fdot = np.ascontiguousarray(fdot, dtype=np.float64)
        m = np.ascontiguousarray(m, dtype=np.float64)
        t0 = np.ascontiguousarray(t0, dtype=np.float64)
        idx = range(len(m)) if idx is None else idx
        fn = self.lib.irr_simd_set_jp_
        a = C.c_int(0)
        mm = C.c_double(0.0)
        tt = C.c_double(0.0)
        for i in idx:
            i = int(i)
            a.value = i + 1
            mm.value = float(m[i])
            tt.value = float(t0[i])
            fn(C.byref(a), _dp(x0[i]), _dp(v0[i]), _dp(f[i]), _dp(fdot[i]), C.byref(mm),
               C.byref(tt))
        _check(self.lib)

    def set_lists(self, lists, idx=None) -> None:
        """irr_simd_set_list_ for the rows idx (default all) of lists[n][lmax]
        (count, then 0-based ids), passed as Fortran LIST rows."""
        lists = np.asarray(lists, dtype=np.int32)
        idx = range(lists.shape[0]) if idx is None else idx
        fn = self.lib.irr_simd_set_list_
        a = C.c_int(0)
        for i in idx:
            i = int(i)
            row = lists[i]
            c = int(row[0])
            buf = np.empty(1 + c, dtype=np.int32)
            buf[0] = c
            buf[1:] = row[1:1 + c] + 1
            a.value = i + 1
            fn(C.byref(a), buf.ctypes.data_as(_I))
        _check(self.lib)

    def firr(self, ti: float, active, out=None) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
        """Irregular force, its derivative and the nearest neighbour (1-based,
        0 for an empty list) of the 0-based particles `active` at time ti.
        out: optional (acc [>=ni, 3] float64, jrk [>=ni, 3] float64, nnbid
        [>=ni] int32) C-contiguous arrays to write into, kept between calls as
        a Fortran caller keeps its arrays."""
        addr = np.ascontiguousarray(np.asarray(active) + 1, dtype=np.int32)
        ni = addr.shape[0]
        if out is None:
            acc = np.zeros((max(ni, 1), 3))
            jrk = np.zeros((max(ni, 1), 3))
            nid = np.zeros(max(ni, 1), dtype=np.int32)
        else:
            acc, jrk, nid = out
            if not (acc.dtype == np.float64 and jrk.dtype == np.float64 and nid.dtype == np.int32
                    and acc.flags.c_contiguous and jrk.flags.c_contiguous
                    and nid.flags.c_contiguous and acc.shape[1:] == (3,)
                    and jrk.shape[1:] == (3,) and min(len(acc), len(jrk), len(nid)) >= ni):
                raise ValueError("out must be C-contiguous float64 [ni,3] x2 and int32 [ni]")
        self.lib.irr_simd_firr_vec_(C.byref(C.c_double(ti)), C.byref(C.c_int(ni)),
                                    addr.ctypes.data_as(_I), _dp(acc), _dp(jrk),
                                    nid.ctypes.data_as(_I))
        _check(self.lib)
        return acc[:ni], jrk[:ni], nid[:ni]

    def profile(self) -> None:
        self.lib.irr_simd_profile_(C.byref(C.c_int(0)))


__all__ = ["IrrSimd", "GpunbError", "send_predicted"]


def send_predicted(time: float, body, ifirst: int = 1, ntot: int | None = None):
    """gpunb_send_predicted_: predict bodies ifirst..ntot (1-based) to `time`
    from the state stored with IrrSimd.set_jp and upload them as the
    regular-force j-set (needs an open GpuNb and an open IrrSimd).  Returns
    the predicted X and XDOT of those bodies."""
    lib = load()
    fn = lib.gpunb_send_predicted_
    fn.argtypes = [_I, _I, _D, _D, _D, _D]
    fn.restype = None
    body = np.ascontiguousarray(body, dtype=np.float64)
    if ntot is None:
        ntot = ifirst + len(body) - 1
    n = ntot - ifirst + 1
    x = np.zeros((max(n, 1), 3))
    xd = np.zeros((max(n, 1), 3))
    fn(C.byref(C.c_int(ifirst)), C.byref(C.c_int(ntot)), C.byref(C.c_double(time)), _dp(body),
       _dp(x), _dp(xd))
    _check(lib)
    return x[:n], xd[:n]
