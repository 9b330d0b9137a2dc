"""GB300-native (sm_103a) regular-force library for NBODY6++: the
gpunb_open/send/regf/close/profile and gpupot C ABI, re-implemented with
hand-written CUDA kernels (libgpunb.so), plus its Python host side."""
from .gpunb import GpuNb, GpunbError, RegfResult, gpupot, load  # noqa: F401

__all__ = ["GpuNb", "GpunbError", "RegfResult", "gpupot", "load"]
