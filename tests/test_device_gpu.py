"""The single-set device entry points (gpunb_send_device / gpunb_regf_device):
the same results as the host-array ABI, CUDA-graph replay that reproduces
eager calls bit for bit on changed inputs, and device-side errors read back
through gpunb_device_status."""
import numpy as np
import pytest

from conftest import rows_equal
from nbody6ppgpu_gb300 import ics
from nbody6ppgpu_gb300.gpunb import GpuNb, load

pytestmark = pytest.mark.gpu

N = 8192
NNBMAX = 256


@pytest.fixture(scope="module")
def case():
    c = ics.plummer(N, seed=31, masses="kroupa", nb_target=60.0)
    return c, c.h2()


class DeviceCall:
    """Device copies of one j-set and one active block, and the outputs."""

    def __init__(self, c, h2, act):
        import torch
        self.torch = torch
        dev = torch.device("cuda", 0)
        T = lambda a: torch.as_tensor(np.ascontiguousarray(a)).to(dev, dtype=torch.float64)
        self.m, self.x, self.v = T(c.m), T(c.x), T(c.v)
        self.h2, self.dtr, self.xi, self.vi = T(h2[act]), T(c.dtr[act]), T(c.x[act]), T(c.v[act])
        ni = len(act)
        self.ni = ni
        self.acc = torch.empty((ni, 3), dtype=torch.float64, device=dev)
        self.jrk = torch.empty((ni, 3), dtype=torch.float64, device=dev)
        self.pot = torch.empty(ni, dtype=torch.float64, device=dev)
        self.nnb = torch.empty(ni, dtype=torch.int32, device=dev)
        self.off = torch.empty(ni + 1, dtype=torch.int32, device=dev)
        self.lst = torch.empty(ni * NNBMAX, dtype=torch.int32, device=dev)

    def run(self, lib):
        self.torch.cuda.synchronize()   # the library works on its own stream
        rc = lib.gpunb_send_device(N, self.m.data_ptr(), self.x.data_ptr(), self.v.data_ptr(), None)
        assert rc == 0
        rc = lib.gpunb_regf_device(self.ni, self.h2.data_ptr(), self.dtr.data_ptr(),
                                   self.xi.data_ptr(), self.vi.data_ptr(), self.acc.data_ptr(),
                                   self.jrk.data_ptr(), self.pot.data_ptr(), self.nnb.data_ptr(),
                                   self.off.data_ptr(), self.lst.data_ptr(), self.ni * NNBMAX,
                                   NNBMAX, 0, None)
        assert rc == 0
        assert lib.gpunb_device_status(None) == 0
        off = self.off.cpu().numpy()
        lst = self.lst.cpu().numpy()
        return (self.acc.cpu().numpy(), self.jrk.cpu().numpy(), self.pot.cpu().numpy(),
                self.nnb.cpu().numpy(), [lst[off[i]:off[i + 1]].copy() for i in range(self.ni)])


@pytest.mark.parametrize("ni", [37, 1024, N])
def test_device_entry_points_match_host_abi(case, ni):
    c, h2 = case
    act = ics.active_set(N, ni, seed=ni)
    lib = load()
    with GpuNb(N) as nb:
        nb.send(c.m, c.x, c.v)
        host = nb.regf(h2[act], c.dtr[act], c.x[act], c.v[act], NNBMAX + 1, NNBMAX)
        acc, jrk, pot, nnb, rows = DeviceCall(c, h2, act).run(lib)
    assert np.array_equal(acc, host.acc) and np.array_equal(jrk, host.jrk)
    assert np.array_equal(pot, host.pot)
    assert np.array_equal(nnb, host.list[:, 0])
    for i in range(ni):
        k = host.list[i, 0]
        assert np.array_equal(rows[i], host.list[i, 1:1 + k] if k > 0 else []), i


@pytest.mark.parametrize("ni", [37, 4096])
def test_graph_replay_matches_eager_calls(case, ni):
    """Eager results for inputs A and B; then, with graphs on, A (eager run
    and capture), B and A again (replays): the same bits every time."""
    c, h2 = case
    act = ics.active_set(N, ni, seed=ni + 1)
    lib = load()
    with GpuNb(N) as nb:
        d = DeviceCall(c, h2, act)
        a_eager = d.run(lib)
        x0, xi0 = d.x.clone(), d.xi.clone()
        d.x.add_(1e-3)          # B: the whole system shifted and the j-set perturbed
        d.x[::7].mul_(1.01)
        d.xi.copy_(d.x[d.torch.as_tensor(act, device=d.x.device)])
        b_eager = d.run(lib)
        lib.gpunb_set_graphs(1)
        try:
            d.x.copy_(x0); d.xi.copy_(xi0)
            a_cap = d.run(lib)
            d.x.add_(1e-3)
            d.x[::7].mul_(1.01)
            d.xi.copy_(d.x[d.torch.as_tensor(act, device=d.x.device)])
            b_rep = d.run(lib)
            d.x.copy_(x0); d.xi.copy_(xi0)
            a_rep = d.run(lib)
        finally:
            lib.gpunb_set_graphs(0)
    for got, want in ((a_cap, a_eager), (b_rep, b_eager), (a_rep, a_eager)):
        for g_, w_ in zip(got[:4], want[:4]):
            assert np.array_equal(g_, w_)
        assert all(np.array_equal(p, q) for p, q in zip(got[4], want[4]))
    assert not np.array_equal(a_eager[0], b_eager[0])


def test_device_status_reports_nan(case):
    c, h2 = case
    act = ics.active_set(N, 64, seed=5)
    lib = load()
    with GpuNb(N) as nb:
        d = DeviceCall(c, h2, act)
        d.xi[3, 1] = float("nan")
        d.torch.cuda.synchronize()
        lib.gpunb_clear_error()
        rc = lib.gpunb_send_device(N, d.m.data_ptr(), d.x.data_ptr(), d.v.data_ptr(), None)
        assert rc == 0
        rc = lib.gpunb_regf_device(d.ni, d.h2.data_ptr(), d.dtr.data_ptr(), d.xi.data_ptr(),
                                   d.vi.data_ptr(), d.acc.data_ptr(), d.jrk.data_ptr(),
                                   d.pot.data_ptr(), d.nnb.data_ptr(), d.off.data_ptr(),
                                   d.lst.data_ptr(), d.ni * NNBMAX, NNBMAX, 0, None)
        assert rc == 0                                    # queued; the kernel flags the NaN
        assert lib.gpunb_device_status(None) == 3         # GPUNB_E_NAN
        assert lib.gpunb_last_error() == 3
        lib.gpunb_clear_error()
        assert lib.gpunb_device_status(None) == 0         # the word was cleared


def test_host_abi_graph_replay_matches_eager(case):
    """gpunb_send_ / gpunb_regf_ replayed as graphs (device reading the host
    arrays directly) give the eager results bit for bit on changed inputs."""
    c, h2 = case
    act = ics.active_set(N, 2000, seed=7)
    with GpuNb(N) as nb:
        if not nb.set_host_path(True):
            pytest.skip("the device does not read host memory directly here")
        x = c.x.copy()
        xi = x[act].copy()
        vi = c.v[act].copy()
        h2a, dtra = h2[act].copy(), c.dtr[act].copy()

        def call(out=None):
            nb.send(c.m, x, c.v)
            r = nb.regf(h2a, dtra, xi, vi, NNBMAX + 1, NNBMAX, out=out)
            return r.acc.copy(), r.jrk.copy(), r.pot.copy(), r.list.copy(), r

        a_eager = call()
        x += 1e-3
        x[::5] *= 1.01
        xi[:] = x[act]
        b_eager = call()
        out = b_eager[4]
        nb.set_graphs(True)
        try:
            x[:] = c.x
            xi[:] = x[act]
            a_cap = call(out)
            x += 1e-3
            x[::5] *= 1.01
            xi[:] = x[act]
            b_rep = call(out)
            x[:] = c.x
            xi[:] = x[act]
            a_rep = call(out)
        finally:
            nb.set_graphs(False)
    for got, want in ((a_cap, a_eager), (b_rep, b_eager), (a_rep, a_eager)):
        for g_, w_ in zip(got[:3], want[:3]):
            assert np.array_equal(g_, w_)
        assert rows_equal(got[3], want[3]) == []   # entries past a row's count are unset
    assert not np.array_equal(a_eager[0], b_eager[0])


def test_graphs_follow_buffer_growth(case):
    """A call shape captured, then a larger j-set that makes the library grow
    its buffers, then the first shape again: the replay must not use the old
    buffers (results equal an eager call)."""
    c, h2 = case
    act = ics.active_set(N, 500, seed=11)
    big = ics.plummer(2 * N, seed=32, masses="kroupa", nb_target=60.0)
    lib = load()
    with GpuNb(2 * N) as nb:
        d = DeviceCall(c, h2, act)
        want = d.run(lib)
        lib.gpunb_set_graphs(1)
        try:
            d.run(lib)                                    # eager run + capture
            nb.send(big.m, big.x, big.v)                  # grows the library's buffers
            nb.regf(big.h2()[:4096], big.dtr[:4096], big.x[:4096], big.v[:4096],
                    NNBMAX + 1, NNBMAX)
            got = d.run(lib)
        finally:
            lib.gpunb_set_graphs(0)
    for g_, w_ in zip(got[:4], want[:4]):
        assert np.array_equal(g_, w_)
    assert all(np.array_equal(p, q) for p, q in zip(got[4], want[4]))
