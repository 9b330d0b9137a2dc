"""GPU irregular force (include/irr.h, drop-in for src/Main/irr.avx.cpp)
through its Fortran-style C ABI in its FP64 mode (irr_set_precision(1)),
against the FP64 oracle and the golden vectors of the reference's own
irr.avx.cpp.  The double-float default is tested in test_irr_df_gpu.py,
the split-FP32 mode in test_irr_split_gpu.py.

Tolerances: in FP64 mode, against the FP64 oracle the force and its
derivative agree to 1e-10 relative (the two differ only in fused
multiply-adds) and the nearest neighbours are identical; against the
reference's FP32 library they agree within its own error (2e-6 at the 99th
percentile, 2e-5 maximum)."""
import numpy as np
import pytest

from conftest import load_golden, rel_vec_err
from nbody6ppgpu_gb300.gpunb import GpunbError
from oracle import oracle as O

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10
REF_P99, REF_MAX = 2e-6, 2e-5


def _irr(g):
    from nbody6ppgpu_gb300.irr import IrrSimd
    n, lmax = len(g["m"]), g["lists"].shape[1]
    irr = IrrSimd(n, lmax, precision=1)
    irr.set_jp(g["x0"], g["v0"], g["f"], g["fdot"], g["m"], g["t0"])
    irr.set_lists(g["lists"])
    return irr


def _check_fp64(a, j, nid, oa, oj, on):
    ok = np.linalg.norm(oa, axis=1) > 0
    assert np.max(rel_vec_err(a[ok], oa[ok])) < FP64_TOL
    assert np.max(rel_vec_err(j[ok], oj[ok])) < FP64_TOL
    assert np.all(a[~ok] == 0)
    assert np.array_equal(nid, on)


@pytest.mark.parametrize("name", ["irr_plummer2048", "irr_ragged_n37"])
def test_golden_cases(name):
    g = load_golden(name)
    with _irr(g) as irr:
        a, j, nid = irr.firr(float(g["ti"]), g["active"])
    _check_fp64(a, j, nid, g["fp64_acc"], g["fp64_jrk"], g["fp64_nnbid"])
    ok = np.linalg.norm(a, axis=1) > 0
    for got, ref in ((a, g["ref_acc"]), (j, g["ref_jrk"])):
        e = rel_vec_err(ref[ok], got[ok])
        assert np.percentile(e, 99) < REF_P99 and e.max() < REF_MAX
    assert np.array_equal(nid, g["ref_nnbid"])


def test_host_paths_identical_and_deterministic():
    from nbody6ppgpu_gb300.irr import IrrSimd  # noqa: F401
    g = load_golden("irr_plummer2048")
    out = []
    with _irr(g) as irr:
        for mode in (1, 0, 1):
            irr.set_host_path(bool(mode))
            out.append(irr.firr(float(g["ti"]), g["active"]))
        irr.set_host_path(True)
    for a, b in zip(out, out[1:]):
        for u, v in zip(a, b):
            assert np.array_equal(u, v)


def test_updates_between_calls():
    """Only the changed particles are uploaded: later set calls win, new
    lists take effect, untouched particles keep their state."""
    g = load_golden("irr_plummer2048")
    n = len(g["m"])
    rng = np.random.default_rng(4)
    x0, v0, f, fdot, t0 = (g[k].copy() for k in ("x0", "v0", "f", "fdot", "t0"))
    lists = g["lists"].copy()
    ti = float(g["ti"])
    with _irr(g) as irr:
        irr.firr(ti, g["active"])
        for rnd in range(3):
            ch = rng.choice(n, 300, replace=False)
            # a first value that must be overwritten by the second
            irr.set_jp(x0 + 1.0, v0, f, fdot, g["m"], t0, idx=ch[:50])
            x0[ch] += rng.normal(0, 1e-3, (300, 3))
            v0[ch] += rng.normal(0, 1e-3, (300, 3))
            t0[ch] = ti - rng.uniform(0, 0.005, 300)
            irr.set_jp(x0, v0, f, fdot, g["m"], t0, idx=ch)
            rows = rng.choice(n, 40, replace=False)
            for i in rows:           # drop the last neighbour of some rows
                if lists[i, 0] > 0:
                    lists[i, 0] -= 1
            irr.set_lists(lists, idx=rows)
            act = rng.choice(n, 700, replace=False)
            a, j, nid = irr.firr(ti, act)
            oa, oj, on = O.irr_fp64(x0, v0, f, fdot, g["m"], t0, lists, ti, act)
            _check_fp64(a, j, nid, oa, oj, on)


def test_edge_cases():
    from nbody6ppgpu_gb300.irr import IrrSimd
    g = load_golden("irr_ragged_n37")
    n = len(g["m"])
    lists = g["lists"].copy()
    ti = float(g["ti"])
    with _irr(g) as irr:
        # empty call
        a, j, nid = irr.firr(ti, np.array([], dtype=int))
        assert a.shape == (0, 3)
        # the particle itself in its own list adds no force but is the nearest
        i = 3
        row = lists[i].copy()
        c = row[0]
        row[1 + c] = i
        row[0] = c + 1
        l2 = lists.copy()
        l2[i] = row
        irr.set_lists(l2, idx=[i])
        a, j, nid = irr.firr(ti, [i])
        oa, oj, _ = O.irr_fp64(g["x0"], g["v0"], g["f"], g["fdot"], g["m"], g["t0"], lists, ti,
                               [i])
        assert np.max(rel_vec_err(a, oa)) < FP64_TOL and nid[0] == i + 1
        irr.set_lists(lists, idx=[i])
        # an id outside the particle set is an error, not a fault
        bad = lists.copy()
        bad[5, 1] = n + 10
        irr.set_lists(bad, idx=[5])
        with pytest.raises(GpunbError):
            irr.firr(ti, [5])
        from nbody6ppgpu_gb300.gpunb import load
        load().gpunb_clear_error()
        irr.set_lists(lists, idx=[5])
        with pytest.raises(GpunbError):
            irr.firr(ti, [n + 3])
        load().gpunb_clear_error()
    assert IrrSimd  # the module stays importable


def test_device_resident_entry_point():
    torch = pytest.importorskip("torch")
    import ctypes as C
    from nbody6ppgpu_gb300.gpunb import load
    g = load_golden("irr_plummer2048")
    n = len(g["m"])
    rec = np.zeros((n, 16))
    rec[:, 0:3] = g["x0"]; rec[:, 3] = g["m"]; rec[:, 4:7] = g["v0"]; rec[:, 7] = g["t0"]
    rec[:, 8:11] = g["f"]; rec[:, 12:15] = g["fdot"]
    dev = torch.device("cuda", 0)
    st = torch.cuda.Stream(dev)
    R = torch.tensor(rec, device=dev)
    L = torch.tensor(g["lists"], device=dev)
    act = torch.tensor(g["active"].astype(np.int32), device=dev)
    ni = act.numel()
    A = torch.empty(ni, 3, dtype=torch.float64, device=dev)
    J = torch.empty_like(A)
    NID = torch.empty(ni, dtype=torch.int32, device=dev)
    lib = load()
    lib.irr_set_precision(1)
    fn = lib.irr_firr_device
    fn.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_double, C.c_int, C.c_void_p,
                   C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    fn.restype = C.c_int
    torch.cuda.synchronize()
    rc = fn(n, R.data_ptr(), L.shape[1], L.data_ptr(), float(g["ti"]), ni, act.data_ptr(),
            A.data_ptr(), J.data_ptr(), NID.data_ptr(), st.cuda_stream)
    assert rc == 0
    st.synchronize()
    _check_fp64(A.cpu().numpy(), J.cpu().numpy(), NID.cpu().numpy(), g["fp64_acc"],
                g["fp64_jrk"], g["fp64_nnbid"])


def test_send_predicted_equals_host_prediction_then_send():
    """gpunb_send_predicted_ returns the xbpredall.f prediction and leaves the
    library in the state gpunb_send_ of those arrays would: the next regular
    force is the same, bit for bit."""
    from nbody6ppgpu_gb300.gpunb import GpuNb
    from nbody6ppgpu_gb300.irr import send_predicted
    g = load_golden("irr_plummer2048")
    n = len(g["m"])
    ti = float(g["ti"])
    x0, v0, f, fdot, m, t0 = (g[k] for k in ("x0", "v0", "f", "fdot", "m", "t0"))
    s = (ti - t0)[:, None]
    X = ((fdot * s + f) * s + v0) * s + x0          # xbpredall.f:21-26
    XD = (fdot * 1.5 * s + f) * 2.0 * s + v0
    ifirst = 5                                        # bodies 1-4 stand for KS components
    sl = slice(ifirst - 1, n)
    act = np.arange(0, n - ifirst + 1, 7)
    h2 = np.full(act.size, 0.01)
    dtr = np.full(act.size, 1e-3)
    with _irr(g), GpuNb(n) as nb:
        xp, vp = send_predicted(ti, m[sl], ifirst, n)
        np.testing.assert_allclose(xp, X[sl], rtol=1e-13, atol=1e-15)
        np.testing.assert_allclose(vp, XD[sl], rtol=1e-13, atol=1e-15)
        r1 = nb.regf(h2, dtr, xp[act], vp[act], 129, 128)
        nb.send(m[sl], xp, vp)
        r2 = nb.regf(h2, dtr, xp[act], vp[act], 129, 128)
    for a, b in ((r1.acc, r2.acc), (r1.jrk, r2.jrk), (r1.pot, r2.pot), (r1.list, r2.list)):
        assert np.array_equal(a, b)


def test_whole_set_prediction_gives_the_same_bits():
    """Blocks of at least n/32 particles predict every particle once before the
    force loop; smaller blocks predict each listed neighbour in the loop.  The
    arithmetic is the same, so a particle's result does not depend on which
    path its block took."""
    g = load_golden("irr_plummer2048")
    n = len(g["m"])
    small = np.arange(0, n, 97)[:40]            # 40 < n/32: per-listing prediction
    large = np.arange(n)                        # whole-set prediction
    with _irr(g) as irr:
        a_s, j_s, n_s = irr.firr(float(g["ti"]), small)
        a_l, j_l, n_l = irr.firr(float(g["ti"]), large)
    assert np.array_equal(a_s, a_l[small]) and np.array_equal(j_s, j_l[small])
    assert np.array_equal(n_s, n_l[small])
