"""Python host side of libgpunb.so, mirroring the reference's gpunb_* / gpupot_
interface (src/Main/gpunb.velocity.cu:904-939, src/Main/gpupot.gpu.cu:116-127)
with the argument meaning of its Fortran callers (src/Main/util_gpu.F:60,
src/Main/fpoly0.F:31,76,125, src/Main/energy.F:38).

Every call goes through the C ABI in include/gpunb.h with host numpy buffers,
exactly as the Fortran integrator calls it.  There is no CPU fallback: if the
CUDA library is missing or no GPU is visible, the calls raise.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass
from pathlib import Path

import numpy as np

_LIB = None
_PKG = Path(__file__).resolve().parent

ERRORS = {0: "ok", 1: "not open", 2: "bad argument", 3: "NaN input", 4: "CUDA error",
          5: "capacity", 6: "device wait timed out", 7: "no device", 8: "allocation failed"}


class GpunbError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"gpunb error {code} ({ERRORS.get(code, '?')}): {msg}")
        self.code = code


_P = C.POINTER
_D = _P(C.c_double)
_I = _P(C.c_int)


def library_path() -> Path:
    return Path(os.environ.get("GPUNB_LIBRARY", _PKG / "libgpunb.so"))


def load(build_if_missing: bool = True) -> C.CDLL:
    """Load libgpunb.so (building it in-tree first if it is absent)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = library_path()
    if not path.exists() and build_if_missing:
        from . import build as _build
        _build.build()
    if not path.exists():
        raise GpunbError(4, f"{path} not built")
    lib = C.CDLL(str(path))
    ip = C.POINTER(C.c_int)
    sig = {
        "gpunb_devinit_": ([ip], None),
        "gpunb_open_": ([ip, ip], None),
        "gpunb_close_": ([], None),
        "gpunb_send_": ([ip, _D, _D, _D], None),
        "gpunb_regf_": ([ip, _D, _D, _D, _D, _D, _D, _D, ip, ip, ip, ip], None),
        "gpunb_profile_": ([ip], None),
        "gpupot_": ([ip, ip, ip, ip, _D, _D, _D], None),
        "gpunb_last_error": ([], C.c_int),
        "gpunb_last_error_message": ([], C.c_char_p),
        "gpunb_clear_error": ([], None),
        "gpunb_set_abort_on_error": ([C.c_int], None),
        "gpunb_set_precision": ([C.c_int], None),
        "gpunb_set_launch": ([C.c_int, C.c_int], None),
        "gpunb_num_variants": ([], C.c_int),
        "gpunb_variant_info": ([C.c_int, ip, ip, ip], C.c_int),
        "gpunb_autotune": ([C.c_int, C.c_int, ip, _P(C.c_float)], C.c_int),
        "gpunb_set_autotune": ([C.c_int], C.c_int),
        "gpunb_set_resort_interval": ([C.c_int], C.c_int),
        "gpunb_rsmlp_label_device": ([C.c_int] + [C.c_void_p] * 12, C.c_int),
        "gpunb_sort_count": ([], C.c_longlong),
        "gpunb_tune_load": ([C.c_char_p], C.c_int),
        "gpunb_tune_save": ([C.c_char_p], C.c_int),
        "gpunb_set_timing": ([C.c_int], None),
        "gpunb_set_host_path": ([C.c_int], C.c_int),
        "gpunb_kernel_times": ([_P(C.c_float), C.c_int], C.c_int),
        "gpunb_last_kernel_ms": ([], C.c_float),
        "gpunb_last_launch": ([ip, ip, ip], None),
        "gpunb_send_device": ([C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
        "gpunb_regf_device": ([C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                               C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                               C.c_void_p, C.c_size_t, C.c_int, C.c_int, C.c_void_p], C.c_int),
        "gpunb_batch_send_device": ([C.c_int, ip, C.c_void_p, C.c_void_p, C.c_void_p,
                                     C.c_void_p], C.c_int),
        "gpunb_batch_regf_device": ([C.c_int, ip, C.c_void_p, C.c_void_p, C.c_void_p,
                                     C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                     C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t, C.c_int,
                                     C.c_int, C.c_void_p], C.c_int),
        "gpunb_batch_last_plan": ([ip, ip], C.c_int),
        "gpunb_set_graphs": ([C.c_int], None),
        "gpunb_device_status": ([C.c_void_p], C.c_int),
        "gpunb_test_bounded_wait": ([C.c_int, C.c_void_p], C.c_int),
        "gpunb_test_fail_allocs": ([C.c_int], None),
    }
    for name, (args, res) in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    lib.gpunb_set_abort_on_error(0)  # Python callers get exceptions instead
    _LIB = lib
    return lib


def _check(lib) -> None:
    code = lib.gpunb_last_error()
    if code:
        msg = lib.gpunb_last_error_message().decode()
        lib.gpunb_clear_error()
        raise GpunbError(code, msg)


def _dp(a: np.ndarray):
    return a.ctypes.data_as(_D)


def _ip(a: np.ndarray):
    return a.ctypes.data_as(_I)


def _c64(a, shape=None) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.float64)
    if shape is not None:
        a = a.reshape(shape)
    return a


@dataclass
class RegfResult:
    acc: np.ndarray      # [ni, 3]
    jrk: np.ndarray      # [ni, 3]
    pot: np.ndarray      # [ni]
    list: np.ndarray     # [ni, lmax] int32, Fortran LISTGP layout

    @property
    def nnb(self) -> np.ndarray:
        return self.list[:, 0]

    def neighbours(self, i: int) -> np.ndarray:
        c = int(self.list[i, 0])
        return self.list[i, 1:1 + c] if c >= 0 else np.empty(0, np.int32)


class GpuNb:
    """The gpunb_* lifecycle: open -> send -> regf ... -> close.

    Mirrors GPUNB_open/send/regf/close/profile of
    src/Main/gpunb.velocity.cu:628-902 through the C ABI."""

    def __init__(self, nbmax: int, rank: int = 0):
        self.lib = load()
        self.rank = rank
        self.nbmax = int(nbmax)
        nb = C.c_int(self.nbmax)
        rk = C.c_int(rank)
        self.lib.gpunb_open_(C.byref(nb), C.byref(rk))
        _check(self.lib)
        self.nj = 0

    # -- lifecycle ---------------------------------------------------------
    def close(self) -> None:
        self.lib.gpunb_close_()
        _check(self.lib)

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def profile(self) -> None:
        rk = C.c_int(self.rank)
        self.lib.gpunb_profile_(C.byref(rk))

    # -- configuration -----------------------------------------------------
    def set_precision(self, mode: str) -> None:
        self.lib.gpunb_set_precision({"split": 0, "fp64": 1, "double_float": 2}[mode])

    def set_launch(self, variant: int = -1, splits: int = 0) -> None:
        self.lib.gpunb_set_launch(int(variant), int(splits))

    def autotune(self, ni: int, m_flag: int = 0):
        s = C.c_int(0)
        ms = C.c_float(0)
        v = self.lib.gpunb_autotune(int(ni), int(m_flag), C.byref(s), C.byref(ms))
        _check(self.lib)
        return v, s.value, ms.value

    def set_autotune(self, on: bool) -> bool:
        """gpunb_set_autotune: tune each new (N, ni) bucket on its first call's
        own block; returns the previous setting."""
        return bool(self.lib.gpunb_set_autotune(1 if on else 0))

    def tune_save(self, path) -> int:
        return self.lib.gpunb_tune_save(str(path).encode())

    def tune_load(self, path) -> int:
        return self.lib.gpunb_tune_load(str(path).encode())

    def last_launch(self):
        v, s, g = C.c_int(), C.c_int(), C.c_int()
        self.lib.gpunb_last_launch(C.byref(v), C.byref(s), C.byref(g))
        return v.value, s.value, g.value

    def set_host_path(self, direct: bool) -> int:
        """1: copy straight from/to the caller's arrays, rows written by the
        device (where the device reads pageable memory coherently); 0: staged
        through pinned buffers.  Returns the mode in effect."""
        return self.lib.gpunb_set_host_path(1 if direct else 0)

    def set_graphs(self, on: bool) -> None:
        """gpunb_set_graphs: replay each call shape as a CUDA graph."""
        self.lib.gpunb_set_graphs(1 if on else 0)

    def set_timing(self, on: bool) -> None:
        self.lib.gpunb_set_timing(1 if on else 0)

    def kernel_times(self, max_n: int = 4096) -> np.ndarray:
        buf = (C.c_float * max_n)()
        n = self.lib.gpunb_kernel_times(buf, max_n)
        return np.frombuffer(buf, dtype=np.float32, count=n).copy()

    # -- the hot path --------------------------------------------------------
    def send(self, m, x, v) -> None:
        """gpunb_send_(nj, mj, xj, vj): upload the (predicted) j-set."""
        m = _c64(m)
        n = m.shape[0]
        x = _c64(x, (n, 3))
        v = _c64(v, (n, 3))
        nj = C.c_int(n)
        self.lib.gpunb_send_(C.byref(nj), _dp(m), _dp(x), _dp(v))
        _check(self.lib)
        self.nj = n

    def regf(self, h2, dtr, xi, vi, lmax: int, nnbmax: int, m_flag: int = 0,
             out: RegfResult | None = None) -> RegfResult:
        """gpunb_regf_(ni, h2, dtr, xi, vi, acc, jrk, pot, lmax, nnbmax, list, m_flag)."""
        h2 = _c64(h2)
        ni = h2.shape[0]
        dtr = _c64(dtr, (ni,))
        xi = _c64(xi, (ni, 3))
        vi = _c64(vi, (ni, 3))
        if out is None or out.acc.shape[0] != ni or out.list.shape[1] != lmax:
            out = RegfResult(acc=np.empty((ni, 3)), jrk=np.empty((ni, 3)), pot=np.empty(ni),
                             list=np.zeros((ni, lmax), dtype=np.int32))
        a_ni, a_lmax, a_nnb, a_mf = C.c_int(ni), C.c_int(lmax), C.c_int(nnbmax), C.c_int(m_flag)
        self.lib.gpunb_regf_(C.byref(a_ni), _dp(h2), _dp(dtr), _dp(xi), _dp(vi), _dp(out.acc),
                             _dp(out.jrk), _dp(out.pot), C.byref(a_lmax), C.byref(a_nnb),
                             _ip(out.list), C.byref(a_mf))
        _check(self.lib)
        return out


def gpupot(m, x, istart: int = 1, ni: int | None = None, rank: int = 0) -> np.ndarray:
    """gpupot_(rank, istart, ni, n, m, x, pot): +sum_j m_j/r_ij for i = istart..istart+ni-1
    (1-based), all j with r_ij > 0."""
    lib = load()
    m = _c64(m)
    n = m.shape[0]
    x = _c64(x, (n, 3))
    if ni is None:
        ni = n - istart + 1
    pot = np.empty(max(ni, 0))
    a = [C.c_int(v) for v in (rank, istart, ni, n)]
    lib.gpupot_(*[C.byref(v) for v in a], _dp(m), _dp(x), _dp(pot))
    _check(lib)
    return pot


def list_to_sets(lst: np.ndarray) -> list:
    """Rows of a LISTGP array -> list of id arrays (None for overflowed rows)."""
    out = []
    for row in lst:
        c = int(row[0])
        out.append(row[1:1 + c].copy() if c >= 0 else None)
    return out
