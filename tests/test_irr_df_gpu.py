"""GPU irregular force in double-float arithmetic, the default of
include/irr.h: every quantity a hi + lo pair of floats, every operation an
error-free transform on the FP32 pipe, after an FP64 prediction.  Through the
Fortran-style C ABI against the FP64 oracle (oracle/irr_fp64.c): force and
derivative within DF_TOL = 1e-10 relative (measured ~4e-12), nearest
neighbours identical; against the reference's own FP32 library (golden
vectors): within its error (2e-6 at the 99th percentile, 2e-5 maximum)."""
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

from conftest import load_golden, rel_vec_err
from oracle import oracle as O

pytestmark = pytest.mark.gpu

DF_TOL = 1e-10
REF_P99, REF_MAX = 2e-6, 2e-5
ROOT = Path(__file__).resolve().parents[1]


def _irr(g, precision=2):
    from nbody6ppgpu_gb300.irr import IrrSimd
    n, lmax = len(g["m"]), g["lists"].shape[1]
    irr = IrrSimd(n, lmax, precision=precision)
    irr.set_jp(g["x0"], g["v0"], g["f"], g["fdot"], g["m"], g["t0"])
    irr.set_lists(g["lists"])
    return irr


def _check_df(a, j, nid, oa, oj, on):
    ok = np.linalg.norm(oa, axis=1) > 0
    assert np.max(rel_vec_err(a[ok], oa[ok])) < DF_TOL
    assert np.max(rel_vec_err(j[ok], oj[ok])) < DF_TOL
    assert np.all(a[~ok] == 0) and np.all(j[~ok] == 0)
    assert np.array_equal(nid, on)


@pytest.mark.parametrize("name", ["irr_plummer2048", "irr_ragged_n37"])
def test_golden_cases(name):
    g = load_golden(name)
    with _irr(g) as irr:
        a, j, nid = irr.firr(float(g["ti"]), g["active"])
    _check_df(a, j, nid, g["fp64_acc"], g["fp64_jrk"], g["fp64_nnbid"])
    ok = np.linalg.norm(a, axis=1) > 0
    for got, ref in ((a, g["ref_acc"]), (j, g["ref_jrk"])):
        e = rel_vec_err(ref[ok], got[ok])
        assert np.percentile(e, 99) < REF_P99 and e.max() < REF_MAX
    assert np.array_equal(nid, g["ref_nnbid"])


_DEFAULT_CHILD = r"""
import sys
sys.path.insert(0, {root!r}); sys.path.insert(0, {tests!r})
import numpy as np
from conftest import load_golden
from nbody6ppgpu_gb300.irr import IrrSimd
g = load_golden("irr_plummer2048")
irr = IrrSimd(len(g["m"]), g["lists"].shape[1])
irr.set_jp(g["x0"], g["v0"], g["f"], g["fdot"], g["m"], g["t0"])
irr.set_lists(g["lists"])
a, j, nid = irr.firr(float(g["ti"]), g["active"])
irr.close()
np.savez({out!r}, a=a, j=j, nid=nid)
"""


def test_a_fresh_process_defaults_to_double_float(tmp_path):
    out = tmp_path / "fresh.npz"
    src = _DEFAULT_CHILD.format(root=str(ROOT), tests=str(ROOT / "tests"), out=str(out))
    r = subprocess.run([sys.executable, "-c", src], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    fresh = np.load(out)
    g = load_golden("irr_plummer2048")
    with _irr(g, precision=2) as irr:
        a, j, nid = irr.firr(float(g["ti"]), g["active"])
    assert np.array_equal(fresh["a"], a) and np.array_equal(fresh["j"], j)
    assert np.array_equal(fresh["nid"], nid)


def test_host_paths_identical_and_whole_set_prediction_same_bits():
    g = load_golden("irr_plummer2048")
    n = len(g["m"])
    out = []
    with _irr(g) as irr:
        for mode in (1, 0, 1):
            irr.set_host_path(bool(mode))
            out.append(irr.firr(float(g["ti"]), g["active"]))
        irr.set_host_path(True)
        small = np.arange(0, n, 97)[:40]                 # per-listing prediction
        a_s, j_s, n_s = irr.firr(float(g["ti"]), small)
        a_l, j_l, n_l = irr.firr(float(g["ti"]), np.arange(n))   # whole-set prediction
    for a, b in zip(out, out[1:]):
        for u, v in zip(a, b):
            assert np.array_equal(u, v)
    assert np.array_equal(a_s, a_l[small]) and np.array_equal(j_s, j_l[small])
    assert np.array_equal(n_s, n_l[small])


def test_device_resident_entry_point_matches_the_host_form():
    torch = pytest.importorskip("torch")
    import ctypes as C
    from nbody6ppgpu_gb300.gpunb import load
    g = load_golden("irr_plummer2048")
    n = len(g["m"])
    rec = np.zeros((n, 16))
    rec[:, 0:3] = g["x0"]; rec[:, 3] = g["m"]; rec[:, 4:7] = g["v0"]; rec[:, 7] = g["t0"]
    rec[:, 8:11] = g["f"]; rec[:, 12:15] = g["fdot"]
    act_h = g["active"][:50]
    with _irr(g) as irr:
        ha, hj, hn = irr.firr(float(g["ti"]), act_h)
    dev = torch.device("cuda", 0)
    st = torch.cuda.Stream(dev)
    R = torch.tensor(rec, device=dev)
    L = torch.tensor(g["lists"], device=dev)
    act = torch.tensor(act_h.astype(np.int32), device=dev)
    ni = act.numel()
    A = torch.empty(ni, 3, dtype=torch.float64, device=dev)
    J = torch.empty_like(A)
    NID = torch.empty(ni, dtype=torch.int32, device=dev)
    lib = load()
    assert lib.irr_set_precision(2) == 2
    fn = lib.irr_firr_device
    fn.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_double, C.c_int, C.c_void_p,
                   C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    fn.restype = C.c_int
    torch.cuda.synchronize()
    assert fn(n, R.data_ptr(), L.shape[1], L.data_ptr(), float(g["ti"]), ni, act.data_ptr(),
              A.data_ptr(), J.data_ptr(), NID.data_ptr(), st.cuda_stream) == 0
    st.synchronize()
    assert np.array_equal(A.cpu().numpy(), ha) and np.array_equal(J.cpu().numpy(), hj)
    assert np.array_equal(NID.cpu().numpy(), hn)


def test_bench_cluster_and_long_lists_against_the_oracle():
    """Plummer N = 65536 with the lists of its own regular force (~110
    neighbours; blocks of 1024 and all 65536) and Plummer N = 8192 with ~300
    neighbours (all rows, both lane layouts), against the FP64 oracle."""
    from nbody6ppgpu_gb300 import ics
    from nbody6ppgpu_gb300.gpunb import GpuNb
    from nbody6ppgpu_gb300.irr import IrrSimd
    rng = np.random.default_rng(12)
    for n, target, lmax, blocks in ((65536, 100.0, 513, (1024, 65536)),
                                    (8192, 300.0, 1025, (300, 8192))):
        c = ics.plummer(n, seed=3, masses="kroupa", nb_target=target)
        with GpuNb(c.n) as nb:
            nb.send(c.m, c.x, c.v)
            r = nb.regf(c.h2(), c.dtr, c.x, c.v, lmax, lmax - 1)
        lists = np.zeros((c.n, lmax), dtype=np.int32)
        for i in range(c.n):
            ids = r.list[i, 1:1 + max(int(r.list[i, 0]), 0)]
            ids = ids[ids != i]
            lists[i, 0] = len(ids)
            lists[i, 1:1 + len(ids)] = ids
        f = rng.normal(0.0, 0.5, (c.n, 3))
        fdot = rng.normal(0.0, 0.5, (c.n, 3))
        ti = 1.0
        t0 = ti - rng.uniform(0.0, 2e-3, c.n)
        st = (c.x, c.v, f, fdot, c.m, t0, lists, ti)
        with IrrSimd(c.n, lmax, precision=2) as irr:
            irr.set_jp(c.x, c.v, f, fdot, c.m, t0)
            irr.set_lists(lists)
            for ni in blocks:
                act = rng.permutation(c.n)[:ni]
                a, j, nid = irr.firr(ti, act)
                oa, oj, on = O.irr_fp64(*st, act)
                _check_df(a, j, nid, oa, oj, on)
