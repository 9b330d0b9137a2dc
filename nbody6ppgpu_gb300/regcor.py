"""Python host side of gpunb_regcor_device (include/gpunb.h): the regular
corrector of src/Main/regcor_gpu.F for a whole active block on the device.

`regcor_device(iact, freg, fdr, nlist, params, state)` takes torch CUDA
tensors in the Fortran COMMON layout of NBODY6++ (all NTOT bodies, index
I - 1, vectors [NTOT, 3], LIST as [NTOT, LMAX] with 1-based members) and
updates them in place, as REGCOR_GPU does body by body on the host.
"""
from __future__ import annotations

import ctypes as C

from .gpunb import load
from .rsmlp import RSParamsC

STATE_DOUBLE = ("x", "xdot", "body", "h", "x0", "x0dot", "t0r", "stepr", "step", "t0", "timenw",
                "fi", "fidot", "fr", "frdot", "d0", "d0r", "d1r", "d2r", "d3r", "xn", "xndot",
                "rs")


class RegcorParamsC(C.Structure):
    """gpunb_regcor_params"""
    _fields_ = [("time", C.c_double), ("dtmin", C.c_double), ("smin", C.c_double),
                ("smax", C.c_double), ("etar", C.c_double), ("tidal4", C.c_double),
                ("kz14", C.c_int), ("m_flag", C.c_int), ("nnbmax", C.c_int), ("n", C.c_int),
                ("ntot", C.c_int), ("ifirst", C.c_int), ("lmax", C.c_int),
                ("rs", RSParamsC)]


class RegcorStateC(C.Structure):
    """gpunb_regcor_state"""
    _fields_ = [(name, C.c_void_p) for name in STATE_DOUBLE] + [("list", C.c_void_p),
                                                                 ("counters", C.c_void_p)]


def _ptr(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def regcor_device(iact, freg, fdr, nlist, params: dict, state: dict, counters=None,
                  stream=None) -> None:
    """gpunb_regcor_device.  iact: int32 [ni] (1-based body indices, distinct);
    freg, fdr: float64 [ni, 3]; nlist: int32 [ni, lmax] (count, 1-based
    members, self removed; updated for retained neighbours); params: the
    fields of gpunb_regcor_params plus the RS rule's (nnbopt, nb_flag, rscale,
    rc, rsfac, bodym, rdens); state: the arrays named in STATE_DOUBLE plus
    "list" (int32 [NTOT, LMAX]); "h" may be absent.  counters: optional int32
    [4] tensor accumulating NBVOID, NBSMIN, NBFLUX, NICONV."""
    lib = load()
    fn = lib.gpunb_regcor_device
    fn.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                   C.POINTER(RegcorParamsC), C.POINTER(RegcorStateC), C.c_void_p]
    fn.restype = C.c_int
    rs = RSParamsC(nnbopt=int(params["nnbopt"]), nnbmax=int(params["nnbmax"]),
                   nb_flag=int(params["nb_flag"]), few_nb_rule=0,
                   rscale=float(params["rscale"]), rc=float(params["rc"]),
                   rsfac=float(params["rsfac"]), bodym=float(params["bodym"]),
                   rdens=(C.c_double * 3)(*[float(v) for v in params["rdens"]]),
                   band_lo=0.0, band_hi=0.0)
    p = RegcorParamsC(time=float(params["time"]), dtmin=float(params["dtmin"]),
                      smin=float(params["smin"]), smax=float(params["smax"]),
                      etar=float(params["etar"]), tidal4=float(params["tidal4"]),
                      kz14=int(params["kz14"]), m_flag=int(params["m_flag"]),
                      nnbmax=int(params["nnbmax"]), n=int(params["n"]),
                      ntot=int(params["ntot"]), ifirst=int(params["ifirst"]),
                      lmax=int(params["lmax"]), rs=rs)
    s = RegcorStateC(**{name: _ptr(state.get(name)) for name in STATE_DOUBLE},
                     list=_ptr(state["list"]), counters=_ptr(counters))
    rc = fn(int(iact.numel()), _ptr(iact), _ptr(freg), _ptr(fdr), _ptr(nlist), C.byref(p),
            C.byref(s), None if stream is None else C.c_void_p(stream.cuda_stream))
    if rc != 0:
        raise RuntimeError(f"gpunb_regcor_device failed with code {rc}")
