"""gpupot_device_noalloc: the potential for callers that cannot allocate device
memory (a host whose own caching allocator already holds the free device
memory, or a step loop that cannot afford the device-wide synchronisation of
cudaFree).  It must give the potentials of the FP64 oracle, and the same ones
as the gpupot_ entry point, call after call from its fixed in-library
scratch, report the errors its kernels raise, and leave the device's memory
use unchanged.

Kept in a file of its own that pytest collects last."""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

POT_TOL = 1e-6   # the relative tolerance of the other potential tests
E_ARG, E_NAN = 2, 3


def _lib():
    from nbody6ppgpu_gb300.gpunb import load
    lib = load()
    fn = lib.gpupot_device_noalloc
    fn.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    fn.restype = C.c_int
    return lib, fn


def _sampled_oracle(m, x, istart, ni, step):
    rows = np.arange(0, ni, step)
    return rows, np.array([O.pot_fp64(m, x, istart + int(k), 1)[0] for k in rows])


def test_noalloc_matches_oracle_and_gpupot_on_two_calls_in_a_row():
    torch = pytest.importorskip("torch")
    from nbody6ppgpu_gb300 import ics
    from nbody6ppgpu_gb300.gpunb import gpupot
    _, fn = _lib()
    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(dev)
    # a full set, then a sub-range of a different, larger set: the second call
    # reuses the scratch left by the first one
    for n, seed, istart, ni in [(8192, 11, 1, 8192), (20000, 12, 501, 3000)]:
        c = ics.plummer(n, seed=seed, masses="kroupa", nb_target=20.0)
        m = torch.tensor(c.m, dtype=torch.float64, device=dev)
        x = torch.tensor(c.x, dtype=torch.float64, device=dev)
        pot = torch.full((ni,), float("nan"), dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        rc = fn(istart, ni, n, m.data_ptr(), x.data_ptr(), pot.data_ptr(), stream.cuda_stream)
        assert rc == 0
        out = pot.cpu().numpy()
        assert np.all(np.isfinite(out))
        rows, ref = _sampled_oracle(c.m, c.x, istart, ni, 37)
        assert (np.abs(out[rows] - ref) / ref).max() <= POT_TOL
        same = gpupot(c.m, c.x, istart=istart, ni=ni)
        assert (np.abs(out - same) / np.abs(same)).max() <= POT_TOL


def test_noalloc_at_its_size_limit_allocates_nothing():
    torch = pytest.importorskip("torch")
    from nbody6ppgpu_gb300 import ics
    lib, fn = _lib()
    dev = torch.device("cuda", 0)
    n = 65536
    c = ics.plummer(n, seed=21, masses="kroupa", nb_target=20.0)
    m = torch.tensor(c.m, dtype=torch.float64, device=dev)
    x = torch.tensor(c.x, dtype=torch.float64, device=dev)
    pot = torch.empty(n, dtype=torch.float64, device=dev)
    stream = torch.cuda.Stream(dev)
    torch.cuda.synchronize()
    assert fn(1, n, n, m.data_ptr(), x.data_ptr(), pot.data_ptr(), stream.cuda_stream) == 0
    # later calls change nothing in the device's memory use, also while the
    # library's own allocations are made to fail
    free0, _ = torch.cuda.mem_get_info(dev)
    lib.gpunb_test_fail_allocs(1000)
    try:
        for _ in range(2):
            assert fn(1, n, n, m.data_ptr(), x.data_ptr(), pot.data_ptr(),
                      stream.cuda_stream) == 0
    finally:
        lib.gpunb_test_fail_allocs(0)
    free1, _ = torch.cuda.mem_get_info(dev)
    assert free1 == free0
    out = pot.cpu().numpy()
    rows, ref = _sampled_oracle(c.m, c.x, 1, n, 499)
    assert (np.abs(out[rows] - ref) / ref).max() <= POT_TOL


def test_noalloc_reports_a_nan_body_and_poisons_the_output():
    torch = pytest.importorskip("torch")
    from nbody6ppgpu_gb300 import ics
    _, fn = _lib()
    dev = torch.device("cuda", 0)
    n = 4096
    c = ics.plummer(n, seed=5, masses="kroupa", nb_target=20.0)
    x = c.x.copy()
    x[123, 1] = np.nan
    m = torch.tensor(c.m, dtype=torch.float64, device=dev)
    xd = torch.tensor(x, dtype=torch.float64, device=dev)
    pot = torch.zeros(n, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    assert fn(1, n, n, m.data_ptr(), xd.data_ptr(), pot.data_ptr(), None) == E_NAN
    assert np.all(np.isnan(pot.cpu().numpy()))
    # the next call on clean inputs starts from a cleared error word
    xd = torch.tensor(c.x, dtype=torch.float64, device=dev)
    assert fn(1, n, n, m.data_ptr(), xd.data_ptr(), pot.data_ptr(), None) == 0
    out = pot.cpu().numpy()
    rows, ref = _sampled_oracle(c.m, c.x, 1, n, 61)
    assert (np.abs(out[rows] - ref) / ref).max() <= POT_TOL


def test_noalloc_rejects_sizes_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    _, fn = _lib()
    dev = torch.device("cuda", 0)
    n = 65537
    m = torch.zeros(n, dtype=torch.float64, device=dev)
    x = torch.zeros((n, 3), dtype=torch.float64, device=dev)
    pot = torch.zeros(1, dtype=torch.float64, device=dev)
    assert fn(1, 1, n, m.data_ptr(), x.data_ptr(), pot.data_ptr(), None) == E_ARG
    assert fn(3, 2, 3, m.data_ptr(), x.data_ptr(), pot.data_ptr(), None) == E_ARG
