"""gpupot_device_noalloc: the potential for callers that cannot allocate
device memory (graph-captured energy checks, hosts whose caching allocator
already holds the free device memory).  It must give the same potentials as
the gpupot_ entry point, call after call, from its fixed in-library scratch.

Kept in a file of its own that pytest collects last."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

POT_TOL = 1e-6   # the relative tolerance of the other potential tests


def _noalloc_fn():
    from nbody6ppgpu_gb300.gpunb import load
    lib = load()
    fn = lib.gpupot_device_noalloc
    fn.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    fn.restype = C.c_int
    return fn


def test_noalloc_matches_gpupot_on_two_calls_in_a_row():
    torch = pytest.importorskip("torch")
    from nbody6ppgpu_gb300 import ics
    from nbody6ppgpu_gb300.gpunb import gpupot
    fn = _noalloc_fn()
    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(dev)
    # a full set, then a sub-range of a different, larger set: the second call
    # reuses the scratch left by the first one
    for n, seed, istart, ni in [(8192, 11, 1, 8192), (20000, 12, 501, 3000)]:
        c = ics.plummer(n, seed=seed, masses="kroupa", nb_target=20.0)
        ref = gpupot(c.m, c.x, istart=istart, ni=ni)
        m = torch.tensor(c.m, dtype=torch.float64, device=dev)
        x = torch.tensor(c.x, dtype=torch.float64, device=dev)
        pot = torch.full((ni,), float("nan"), dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        rc = fn(istart, ni, n, m.data_ptr(), x.data_ptr(), pot.data_ptr(), stream.cuda_stream)
        assert rc == 0
        stream.synchronize()
        out = pot.cpu().numpy()
        assert np.all(np.isfinite(out))
        assert (np.abs(out - ref) / np.abs(ref)).max() <= POT_TOL


def test_noalloc_rejects_sizes_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    fn = _noalloc_fn()
    dev = torch.device("cuda", 0)
    n = 65537
    m = torch.zeros(n, dtype=torch.float64, device=dev)
    x = torch.zeros((n, 3), dtype=torch.float64, device=dev)
    pot = torch.zeros(1, dtype=torch.float64, device=dev)
    assert fn(1, 1, n, m.data_ptr(), x.data_ptr(), pot.data_ptr(), None) == 2
    assert fn(3, 2, 3, m.data_ptr(), x.data_ptr(), pot.data_ptr(), None) == 2
