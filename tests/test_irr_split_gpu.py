"""GPU irregular force in split precision (irr_set_precision(0) of
include/irr.h: the reference's own scheme, src/Main/irr.avx.cpp:58-176 --
double-single positions, FP32 velocities, masses and force arithmetic --
here after an FP64 prediction), through the Fortran-style C ABI.

Parity, against the FP64 oracle (oracle/irr_fp64.c), to the accuracy class
of the reference's own FP32 library (its golden vectors: 2e-6 at the 99th
percentile, 2e-5 maximum): force and derivative within IRR_P99 = 2e-6
relative at the 99th percentile, and per particle within IRR_BOUND = 5e-6 of
max(|Q_i|, S_i / 8), S_i the sum of the pair terms' magnitudes
(oracle.irr_abs_sums).  The regular force's bound is 1e-6: an irregular
force sums a few dominant terms whose FP32 roundings do not average out the
way a regular force's thousands do; that accuracy is the double-float (the
default) and FP64 modes'.  Against the golden vectors of the reference's library: within
its error.  The nearest neighbour is the FP64
oracle's, except where the two nearest listed bodies lie within 1e-6 of each
other in r^2 (the choice is made on the FP32 r^2)."""
import numpy as np
import pytest

from conftest import load_golden, rel_vec_err
from oracle import oracle as O

pytestmark = pytest.mark.gpu

REF_P99, REF_MAX = 2e-6, 2e-5
IRR_P99, IRR_BOUND = 2e-6, 5e-6
TIE = 1e-6


def _irr(g, precision=0):
    from nbody6ppgpu_gb300.irr import IrrSimd
    n, lmax = len(g["m"]), g["lists"].shape[1]
    irr = IrrSimd(n, lmax, precision=precision)
    irr.set_jp(g["x0"], g["v0"], g["f"], g["fdot"], g["m"], g["t0"])
    irr.set_lists(g["lists"])
    return irr


def _state(g):
    return (g["x0"], g["v0"], g["f"], g["fdot"], g["m"], g["t0"], g["lists"], float(g["ti"]))


def _check_nnbid(nid, on, st, act):
    """nid == on except for ties within TIE in FP64 r^2 (both 1-based ids)."""
    x0, v0, a2, j6, m, t0, lists, ti = st
    dt = (ti - t0)[:, None]
    x = x0 + dt * (v0 + dt * (a2 + dt * j6))
    bad = np.nonzero(nid != on)[0]
    for k in bad:
        i = int(act[k])
        assert nid[k] > 0 and on[k] > 0, (k, nid[k], on[k])
        ra = float(np.sum((x[nid[k] - 1] - x[i]) ** 2))
        rb = float(np.sum((x[on[k] - 1] - x[i]) ** 2))
        assert abs(ra - rb) <= TIE * rb, (k, ra, rb)
    return len(bad)


def _check_vs_oracle(a, j, nid, st, act):
    oa, oj, on = O.irr_fp64(*st, act)
    sa, sj = O.irr_abs_sums(*st, act)
    ones = np.ones(len(act))
    e = O.parity_errors(a, j, ones, oa, oj, ones, sa, sj)
    for q in ("acc", "jrk"):
        assert e[q]["p99"] <= IRR_P99 and e[q]["bound_max"] <= IRR_BOUND, (q, e[q])
    empty = st[6][np.asarray(act), 0] == 0
    assert np.all(a[empty] == 0) and np.all(j[empty] == 0) and np.all(nid[empty] == 0)
    _check_nnbid(nid, on, st, act)
    return e


@pytest.mark.parametrize("name", ["irr_plummer2048", "irr_ragged_n37"])
def test_golden_cases(name):
    g = load_golden(name)
    with _irr(g) as irr:
        a, j, nid = irr.firr(float(g["ti"]), g["active"])
    _check_vs_oracle(a, j, nid, _state(g), g["active"])
    ok = np.linalg.norm(a, axis=1) > 0
    for got, ref in ((a, g["ref_acc"]), (j, g["ref_jrk"])):
        e = rel_vec_err(ref[ok], got[ok])
        assert np.percentile(e, 99) < REF_P99 and e.max() < REF_MAX
    assert np.array_equal(nid, g["ref_nnbid"])


def test_precision_switch():
    g = load_golden("irr_plummer2048")
    from nbody6ppgpu_gb300.gpunb import load
    lib = load()
    assert lib.irr_set_precision(0) == 0
    with _irr(g, precision=None) as irr:
        a0, j0, _ = irr.firr(float(g["ti"]), g["active"])
        assert irr.set_precision(1) == 1
        a1, j1, n1 = irr.firr(float(g["ti"]), g["active"])
        assert irr.set_precision(0) == 0
    ok = np.linalg.norm(g["fp64_acc"], axis=1) > 0
    assert np.max(rel_vec_err(a1[ok], g["fp64_acc"][ok])) < 1e-10
    assert np.array_equal(n1, g["fp64_nnbid"])
    # split results are FP32-accurate, not FP64-accurate
    assert 0 < np.max(rel_vec_err(a0[ok], g["fp64_acc"][ok])) < 1e-5


def test_host_paths_identical_and_deterministic():
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


def test_whole_set_prediction_gives_the_same_bits():
    """Blocks of at least n/32 particles split the whole set's FP64
    prediction once; smaller blocks predict and split each listed body in
    the force loop.  Same arithmetic, so the same bits either way."""
    g = load_golden("irr_plummer2048")
    n = len(g["m"])
    small = np.arange(0, n, 97)[:40]
    large = np.arange(n)
    with _irr(g) as irr:
        a_s, j_s, n_s = irr.firr(float(g["ti"]), small)
        a_l, j_l, n_l = irr.firr(float(g["ti"]), large)
    assert np.array_equal(a_s, a_l[small]) and np.array_equal(j_s, j_l[small])
    assert np.array_equal(n_s, n_l[small])


def test_updates_between_calls():
    g = load_golden("irr_plummer2048")
    n = len(g["m"])
    rng = np.random.default_rng(14)
    x0, v0, f, fdot, t0 = (g[k].copy() for k in ("x0", "v0", "f", "fdot", "t0"))
    lists = g["lists"].copy()
    ti = float(g["ti"])
    with _irr(g) as irr:
        for _ in range(3):
            ch = rng.choice(n, 300, replace=False)
            x0[ch] += rng.normal(0, 1e-3, (300, 3))
            v0[ch] += rng.normal(0, 1e-3, (300, 3))
            t0[ch] = ti - rng.uniform(0, 0.005, 300)
            irr.set_jp(x0, v0, f, fdot, g["m"], t0, idx=ch)
            rows = rng.choice(n, 40, replace=False)
            for i in rows:
                if lists[i, 0] > 0:
                    lists[i, 0] -= 1
            irr.set_lists(lists, idx=rows)
            act = rng.choice(n, 700, replace=False)
            a, j, nid = irr.firr(ti, act)
            _check_vs_oracle(a, j, nid, (x0, v0, f, fdot, g["m"], t0, lists, ti), act)


def test_self_in_list_and_empty_rows():
    g = load_golden("irr_ragged_n37")
    lists = g["lists"].copy()
    ti = float(g["ti"])
    i = 3
    c = lists[i, 0]
    l2 = lists.copy()
    l2[i, 1 + c] = i
    l2[i, 0] = c + 1
    l2[7, 0] = 0                     # an empty row
    with _irr(g) as irr:
        irr.set_lists(l2, idx=[i, 7])
        a, j, nid = irr.firr(ti, [i, 7])
        irr.set_lists(lists, idx=[i])
        b, k, _ = irr.firr(ti, [i])
    assert np.array_equal(a[0], b[0]) and np.array_equal(j[0], k[0])   # self adds nothing
    assert nid[0] == i + 1                                             # and is the nearest
    assert np.all(a[1] == 0) and np.all(j[1] == 0) and nid[1] == 0


def test_device_resident_entry_point_matches_the_host_form():
    torch = pytest.importorskip("torch")
    import ctypes as C
    from nbody6ppgpu_gb300.gpunb import load
    g = load_golden("irr_plummer2048")
    n = len(g["m"])
    rec = np.zeros((n, 16))
    rec[:, 0:3] = g["x0"]; rec[:, 3] = g["m"]; rec[:, 4:7] = g["v0"]; rec[:, 7] = g["t0"]
    rec[:, 8:11] = g["f"]; rec[:, 12:15] = g["fdot"]
    act_h = g["active"][:50]         # a small block: per-listing prediction in both forms
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
    assert lib.irr_set_precision(0) == 0
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


def test_bench_cluster_against_the_oracle():
    """Plummer N = 65536 (Kroupa) with the neighbour lists of its own
    regular force (self removed): blocks of 1024 and 65536 particles against
    the FP64 oracle, every row."""
    from nbody6ppgpu_gb300 import ics
    from nbody6ppgpu_gb300.gpunb import GpuNb
    c = ics.plummer(65536, seed=3, masses="kroupa", nb_target=100.0)
    lmax = 513
    with GpuNb(c.n) as nb:
        nb.send(c.m, c.x, c.v)
        r = nb.regf(c.h2(), c.dtr, c.x, c.v, lmax, 512)
    lists = np.zeros((c.n, lmax), dtype=np.int32)
    for i in range(c.n):
        ids = r.list[i, 1:1 + max(int(r.list[i, 0]), 0)]
        ids = ids[ids != i]
        lists[i, 0] = len(ids)
        lists[i, 1:1 + len(ids)] = ids
    rng = np.random.default_rng(8)
    f = rng.normal(0.0, 0.5, (c.n, 3))
    fdot = rng.normal(0.0, 0.5, (c.n, 3))
    ti = 1.0
    t0 = ti - rng.uniform(0.0, 2e-3, c.n)
    from nbody6ppgpu_gb300.irr import IrrSimd
    st = (c.x, c.v, f, fdot, c.m, t0, lists, ti)
    with IrrSimd(c.n, lmax, precision=0) as irr:
        irr.set_jp(c.x, c.v, f, fdot, c.m, t0)
        irr.set_lists(lists)
        for ni in (1024, c.n):
            act = rng.permutation(c.n)[:ni]
            a, j, nid = irr.firr(ti, act)
            _check_vs_oracle(a, j, nid, st, act)


def test_profile_counts_the_listed_pairs(capfd):
    """irr_simd_profile_ reports the calls' listed pairs, counted on the
    device (the line of irr.avx.cpp:403-416: Ncall, <NI> = pairs per call,
    <NB> = pairs per particle)."""
    g = load_golden("irr_plummer2048")
    act = g["active"]
    pairs = int(np.maximum(g["lists"][act, 0], 0).sum())
    with _irr(g) as irr:
        irr.profile()                     # reset the counters
        capfd.readouterr()
        irr.firr(float(g["ti"]), act)
        irr.firr(float(g["ti"]), act)
        irr.profile()
    err = capfd.readouterr().err
    line = [ln for ln in err.splitlines() if "Irr.F" in ln][-1]
    f = line.split()
    assert int(f[f.index("Ncall:") + 1]) == 2
    assert int(f[f.index("<NI>:") + 1]) == pairs
    assert abs(float(f[f.index("<NB>:") + 1]) - pairs / len(act)) < 1e-6 * pairs


@pytest.mark.parametrize("precision", [0, 1])
def test_long_lists_both_lane_layouts(precision):
    """Lists of ~300 neighbours (many chunks per lane), a block large enough
    for 8 lanes per particle and a small one with 32, both precisions,
    against the FP64 oracle."""
    from nbody6ppgpu_gb300 import ics
    from nbody6ppgpu_gb300.gpunb import GpuNb
    from nbody6ppgpu_gb300.irr import IrrSimd
    c = ics.plummer(8192, seed=9, masses="kroupa", nb_target=300.0)
    lmax = 1025
    with GpuNb(c.n) as nb:
        nb.send(c.m, c.x, c.v)
        r = nb.regf(c.h2(), c.dtr, c.x, c.v, lmax, 1024)
    lists = np.zeros((c.n, lmax), dtype=np.int32)
    for i in range(c.n):
        ids = r.list[i, 1:1 + max(int(r.list[i, 0]), 0)]
        ids = ids[ids != i]
        lists[i, 0] = len(ids)
        lists[i, 1:1 + len(ids)] = ids
    assert lists[:, 0].mean() > 200
    rng = np.random.default_rng(10)
    f = rng.normal(0.0, 0.5, (c.n, 3))
    fdot = rng.normal(0.0, 0.5, (c.n, 3))
    ti = 0.5
    t0 = ti - rng.uniform(0.0, 1e-3, c.n)
    st = (c.x, c.v, f, fdot, c.m, t0, lists, ti)
    with IrrSimd(c.n, lmax, precision=precision) as irr:
        irr.set_jp(c.x, c.v, f, fdot, c.m, t0)
        irr.set_lists(lists)
        for act in (np.arange(c.n), rng.permutation(c.n)[:300]):
            a, j, nid = irr.firr(ti, act)
            if precision == 0:
                _check_vs_oracle(a, j, nid, st, act)
            else:
                oa, oj, on = O.irr_fp64(*st, act)
                assert np.max(rel_vec_err(a, oa)) < 1e-10 and np.max(rel_vec_err(j, oj)) < 1e-10
                assert np.array_equal(nid, on)
