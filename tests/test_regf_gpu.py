"""GPU parity of gpunb_regf_ / gpupot_ (through the C ABI) against the FP64
oracle and the golden vectors of the reference's CPU path.

Tolerances (FP64 oracle as truth):
  * split precision, per particle: force and jerk within 1e-6 of
    max(|Q_i|, S_i / 8), S_i = sum_j |q_ij| (the plain relative error
    wherever the sum cancels by less than a factor 8; oracle.parity_errors),
    the potential within 1e-6 relative, and the plain relative errors of
    force and jerk within 1e-6 at the 99th percentile;
  * plain FP64 kernel: <= 1e-12;
  * neighbour lists: identical to the oracle, bit for bit (counts, overflow
    flags and ids in ascending order).
"""
import numpy as np
import pytest

from conftest import check_split, load_golden, rel_vec_err, rows_equal, unpack_list
from nbody6ppgpu_gb300 import ics
from nbody6ppgpu_gb300.gpunb import GpuNb, GpunbError, gpupot, load
from oracle import oracle as O

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
DF_TOL = 1e-10   # the double-float kernel against the FP64 oracle, every particle


@pytest.fixture(scope="module")
def lib():
    return load()


def check_forces(res, acc, jrk, pot, accabs, jrkabs):
    """split-precision bound on the accepted rows of a regf result"""
    ok = res.list[:, 0] >= 0
    return check_split(res.acc, res.jrk, res.pot, acc, jrk, pot, accabs, jrkabs, ok=ok)


def run_golden(g, precision="split", variant=-1, splits=0):
    n = len(g["m"])
    with GpuNb(max(n, 1)) as nb:
        nb.set_precision(precision)
        nb.set_launch(variant, splits)
        nb.send(g["m"], g["x"], g["v"])
        ii = g["ii"]
        return nb.regf(g["h2"], g["dtr"], g["x"][ii], g["v"][ii], int(g["lmax"]),
                       int(g["nnbmax"]), int(g["m_flag"]))


@pytest.mark.parametrize("name", ["plummer2048_equal", "mflag_plummer512",
                                  "overflow_plummer512", "ragged_n37"])
@pytest.mark.parametrize("precision", ["split", "fp64", "double_float"])
def test_golden_cases(lib, name, precision):
    g = load_golden(name)
    res = run_golden(g, precision)
    lmax = int(g["lmax"])
    assert rows_equal(res.list, unpack_list(g["fp64_cnt"], g["fp64_ids"], lmax)) == []
    # and therefore identical to the reference CPU path's lists too
    assert rows_equal(res.list, unpack_list(g["ref_cnt"], g["ref_ids"], lmax)) == []
    if precision == "split":
        check_forces(res, g["fp64_acc"], g["fp64_jrk"], g["fp64_pot"], g["fp64_accabs"],
                     g["fp64_jrkabs"])
    else:
        ok = res.list[:, 0] >= 0
        if precision == "fp64":
            np.testing.assert_allclose(res.acc[ok], g["fp64_acc"][ok], rtol=FP64_TOL, atol=1e-14)
            np.testing.assert_allclose(res.pot[ok], g["fp64_pot"][ok], rtol=FP64_TOL)
        else:   # double-float: every particle's vectors and potential
            assert rel_vec_err(res.acc[ok], g["fp64_acc"][ok]).max() < DF_TOL
            assert rel_vec_err(res.jrk[ok], g["fp64_jrk"][ok]).max() < DF_TOL
            np.testing.assert_allclose(res.pot[ok], g["fp64_pot"][ok], rtol=DF_TOL)


def test_all_launch_shapes_agree_and_are_deterministic(lib):
    g = load_golden("plummer2048_equal")
    base = run_golden(g, "split", 0, 0)
    again = run_golden(g, "split", 0, 0)
    assert np.array_equal(base.acc, again.acc) and np.array_equal(base.list, again.list)
    nv = lib.gpunb_num_variants()
    for v in range(nv):
        for s in (1, 3, 16):
            r = run_golden(g, "split", v, s)
            assert rows_equal(r.list, base.list) == [], (v, s)
            check_forces(r, g["fp64_acc"], g["fp64_jrk"], g["fp64_pot"], g["fp64_accabs"],
                         g["fp64_jrkabs"])


@pytest.fixture(scope="module")
def plummer64k():
    c = ics.plummer(65536, seed=2, masses="kroupa", nb_target=100.0)
    return c


@pytest.mark.parametrize("ni", [1, 32, 1024, 16384, 65536])
def test_config2_block_sizes(lib, plummer64k, ni):
    """Plummer N=65536, Kroupa masses, target 100, nbmax 512, every block size
    of the workload; the oracle is evaluated on (512 sampled rows of) the
    same active block."""
    c = plummer64k
    act = ics.active_set(c.n, ni, seed=ni)
    with GpuNb(c.n) as nb:
        nb.send(c.m, c.x, c.v)
        res = nb.regf(c.h2()[act], c.dtr[act], c.x[act], c.v[act], 513, 512)
    samp = np.arange(ni) if ni <= 1024 else np.linspace(0, ni - 1, 512).astype(int)
    a = act[samp]
    acc, jrk, pot, lst, aa, ja = O.regf_fp64(c.m, c.x, c.v, c.h2()[a], c.dtr[a], c.x[a], c.v[a],
                                             513, 512, with_abs=True)
    sub = type(res)(acc=res.acc[samp], jrk=res.jrk[samp], pot=res.pot[samp], list=res.list[samp])
    assert rows_equal(sub.list, lst) == []
    check_forces(sub, acc, jrk, pot, aa, ja)


@pytest.mark.parametrize("ni", [1024, 16384])
def test_config2_mass_weighted_criterion(lib, plummer64k, ni):
    """The mass-weighted neighbour criterion (m_flag: r^2 < m_j h2 with
    h2 = RS^2 / <m>, util_gpu.F:48) on the Plummer N = 65536 Kroupa cluster:
    512 sampled rows of the block against the FP64 oracle, lists identical,
    the named bound."""
    c = plummer64k
    act = ics.active_set(c.n, ni, seed=ni + 7)
    h2m = c.h2() / c.m.mean()
    with GpuNb(c.n) as nb:
        nb.send(c.m, c.x, c.v)
        res = nb.regf(h2m[act], c.dtr[act], c.x[act], c.v[act], 513, 512, m_flag=1)
    samp = np.arange(ni) if ni <= 1024 else np.linspace(0, ni - 1, 512).astype(int)
    a = act[samp]
    acc, jrk, pot, lst, aa, ja = O.regf_fp64(c.m, c.x, c.v, h2m[a], c.dtr[a], c.x[a], c.v[a],
                                             513, 512, m_flag=1, with_abs=True)
    sub = type(res)(acc=res.acc[samp], jrk=res.jrk[samp], pot=res.pot[samp], list=res.list[samp])
    assert rows_equal(sub.list, lst) == []
    check_forces(sub, acc, jrk, pot, aa, ja)


def test_autotune_on_the_callers_block_is_cached_saved_and_loaded(lib, plummer64k, tmp_path):
    """gpunb_set_autotune(1): the first call of an (N, ni) bucket times every
    launch shape on that call's own block and keeps the fastest.  The tuned
    call is parity-green, forcing the chosen shape gives the same bits, and a
    saved cache loaded back restores the choice."""
    c = plummer64k
    ni = 4096
    act = ics.active_set(c.n, ni, seed=41)
    h2 = c.h2()[act]
    args = (h2, c.dtr[act], c.x[act], c.v[act], 513, 512)
    empty = tmp_path / "empty.txt"
    empty.write_text("")
    saved = tmp_path / "tune.txt"
    with GpuNb(c.n) as nb:
        nb.send(c.m, c.x, c.v)
        assert nb.tune_load(empty) == 0
        prev = nb.set_autotune(True)
        try:
            r1 = nb.regf(*args)
            chosen = nb.last_launch()[:2]
        finally:
            nb.set_autotune(prev)
        assert nb.tune_save(saved) == 1
        nb.set_launch(*chosen)
        r2 = nb.regf(*args)
        nb.set_launch(-1, 0)
        assert np.array_equal(r1.acc, r2.acc) and np.array_equal(r1.jrk, r2.jrk)
        assert np.array_equal(r1.list, r2.list)
        # without the entry the heuristic applies; the saved cache restores it
        assert nb.tune_load(empty) == 0
        nb.regf(*args)
        assert nb.tune_load(saved) == 1
        nb.regf(*args)
        assert nb.last_launch()[:2] == chosen
    samp = np.linspace(0, ni - 1, 256).astype(int)
    a = act[samp]
    acc, jrk, pot, lst, aa, ja = O.regf_fp64(c.m, c.x, c.v, h2[samp], c.dtr[a], c.x[a], c.v[a],
                                             513, 512, with_abs=True)
    sub = type(r1)(acc=r1.acc[samp], jrk=r1.jrk[samp], pot=r1.pot[samp], list=r1.list[samp])
    assert rows_equal(sub.list, lst) == []
    check_forces(sub, acc, jrk, pot, aa, ja)


def test_reordering_interval_keeps_results(lib, plummer64k):
    """Sends between two re-orderings of the j-set reuse its Morton
    permutation and re-pack the tiles from the current positions: after the
    bodies have drifted for three sends the lists equal the oracle's and the
    forces meet the parity bound.  Re-orderings happen on every 4th send and
    whenever nj changes."""
    import ctypes as C
    lib.gpunb_sort_count.restype = C.c_longlong
    c = plummer64k
    act = ics.active_set(c.n, 2048, seed=77)
    h2 = c.h2()[act]
    with GpuNb(c.n) as nb:
        prev = lib.gpunb_set_resort_interval(4)
        try:
            n0 = lib.gpunb_sort_count()
            nb.send(c.m, c.x, c.v)                      # re-orders
            for k in range(1, 4):                       # drift, same permutation
                x = c.x + c.v * (2e-3 * k)
                nb.send(c.m, x, c.v)
            assert lib.gpunb_sort_count() - n0 == 1
            r = nb.regf(h2, c.dtr[act], x[act], c.v[act], 513, 512)
            nb.send(c.m, x, c.v)                        # the 5th send re-orders
            assert lib.gpunb_sort_count() - n0 == 2
            nb.send(c.m[:-1], x[:-1], c.v[:-1])         # a new nj re-orders
            assert lib.gpunb_sort_count() - n0 == 3
        finally:
            lib.gpunb_set_resort_interval(prev)
    samp = np.linspace(0, act.size - 1, 256).astype(int)
    a = act[samp]
    acc, jrk, pot, lst, aa, ja = O.regf_fp64(c.m, x, c.v, h2[samp], c.dtr[a], x[a], c.v[a],
                                             513, 512, with_abs=True)
    sub = type(r)(acc=r.acc[samp], jrk=r.jrk[samp], pot=r.pot[samp], list=r.list[samp])
    assert rows_equal(sub.list, lst) == []
    check_forces(sub, acc, jrk, pot, aa, ja)


def test_fp64_kernel_matches_oracle(lib, plummer64k):
    c = plummer64k
    act = ics.active_set(c.n, 300, seed=5)
    with GpuNb(c.n) as nb:
        nb.set_precision("fp64")
        nb.send(c.m, c.x, c.v)
        res = nb.regf(c.h2()[act], c.dtr[act], c.x[act], c.v[act], 513, 512)
    acc, jrk, pot, lst = O.regf_fp64(c.m, c.x, c.v, c.h2()[act], c.dtr[act], c.x[act], c.v[act],
                                     513, 512)
    assert rows_equal(res.list, lst) == []
    assert rel_vec_err(res.acc, acc).max() < FP64_TOL
    assert rel_vec_err(res.jrk, jrk).max() < 1e-10


@pytest.mark.parametrize("m_flag", [0, 1])
def test_double_float_kernel_meets_fp64_accuracy_at_every_particle(lib, plummer64k, m_flag):
    """gpunb_set_precision(2): force, jerk and potential of every sampled
    particle (512 rows) of a 16384 block of the Plummer 65536 cluster within
    1e-10 of the FP64 oracle in plain relative terms -- no cancellation
    allowance -- and the lists identical (the golden cases run in this mode
    too, test_golden_cases)."""
    c = plummer64k
    act = ics.active_set(c.n, 16384, seed=9)
    h2 = c.h2() / (c.m.mean() if m_flag else 1.0)
    samp = np.linspace(0, act.size - 1, 512).astype(int)
    with GpuNb(c.n) as nb:
        nb.set_precision("double_float")
        nb.send(c.m, c.x, c.v)
        res = nb.regf(h2[act], c.dtr[act], c.x[act], c.v[act], 513, 512, m_flag=m_flag)
        nb.set_precision("split")
    a = act[samp]
    acc, jrk, pot, lst = O.regf_fp64(c.m, c.x, c.v, h2[a], c.dtr[a], c.x[a], c.v[a], 513, 512,
                                     m_flag=m_flag)
    assert rows_equal(res.list[samp], lst) == []
    assert rel_vec_err(res.acc[samp], acc).max() < DF_TOL
    assert rel_vec_err(res.jrk[samp], jrk).max() < DF_TOL
    assert (np.abs(res.pot[samp] - pot) / pot).max() < DF_TOL


_PRECISION_CHILD = """
import sys, hashlib
sys.path[:0] = [{root!r}, {tests!r}]
from conftest import load_golden
from nbody6ppgpu_gb300.gpunb import GpuNb
g = load_golden("plummer2048_equal")
ii = g["ii"]
for explicit in (None, {name!r}):
    with GpuNb(len(g["m"])) as nb:
        if explicit:
            nb.set_precision(explicit)
        nb.send(g["m"], g["x"], g["v"])
        r = nb.regf(g["h2"], g["dtr"], g["x"][ii], g["v"][ii], int(g["lmax"]),
                    int(g["nnbmax"]), int(g["m_flag"]))
    print("DIGEST", hashlib.sha256(r.acc.tobytes() + r.jrk.tobytes() + r.pot.tobytes()
                                   + r.list.tobytes()).hexdigest())
"""


def test_precision_from_the_environment_at_open(lib):
    """gpunb_open_ takes the pair kernel from GPUNB_PRECISION: a process that
    sets it to 1 (or 2) and never calls gpunb_set_precision gets the bits of
    the FP64 (or double-float) kernel; unset or 0 gives the split kernel."""
    import os
    import subprocess
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parents[1]
    seen = []
    for mode, name in ((None, "split"), ("0", "split"), ("1", "fp64"), ("2", "double_float")):
        env = dict(os.environ)
        env.pop("GPUNB_PRECISION", None)
        if mode is not None:
            env["GPUNB_PRECISION"] = mode
        src = _PRECISION_CHILD.format(root=str(root), tests=str(root / "tests"), name=name)
        r = subprocess.run([sys.executable, "-c", src], capture_output=True, text=True,
                           timeout=600, env=env)
        assert r.returncode == 0, r.stderr[-2000:]
        from_env, explicit = [ln.split()[1] for ln in r.stdout.splitlines()
                              if ln.startswith("DIGEST")]
        assert from_env == explicit, mode
        seen.append(from_env)
    assert seen[0] == seen[1] and len(set(seen)) == 3


def test_edge_cases(lib):
    c = ics.plummer(300, seed=8, nb_target=10.0)
    with GpuNb(1000) as nb:
        # empty j-set: no force, no neighbours
        nb.send(np.zeros(0), np.zeros((0, 3)), np.zeros((0, 3)))
        r = nb.regf(c.h2()[:3], c.dtr[:3], c.x[:3], c.v[:3], 8, 7)
        assert np.all(r.acc == 0) and np.all(r.pot == 0) and np.all(r.list[:, 0] == 0)
        # a single body: only itself as neighbour
        nb.send(c.m[:1], c.x[:1], c.v[:1])
        r = nb.regf(c.h2()[:1], c.dtr[:1], c.x[:1], c.v[:1], 8, 7)
        assert list(r.list[0, :2]) == [1, 0] and np.all(r.acc == 0)
        # ragged ni, tiny h2 (self only), nnbmax = 0 -> every row overflows (-1)
        nb.send(c.m, c.x, c.v)
        h2 = np.full(7, 1e-30)
        r = nb.regf(h2, c.dtr[:7], c.x[:7], c.v[:7], 4, 3)
        assert np.all(r.list[:, 0] == 1) and np.array_equal(r.list[:, 1], np.arange(7))
        r = nb.regf(h2, c.dtr[:7], c.x[:7], c.v[:7], 4, 0)
        assert np.all(r.list[:, 0] == -1)
        acc, jrk, pot, lst, aa, ja = O.regf_fp64(c.m, c.x, c.v, h2, c.dtr[:7], c.x[:7],
                                                 c.v[:7], 4, 3, with_abs=True)
        r = nb.regf(h2, c.dtr[:7], c.x[:7], c.v[:7], 4, 3)
        check_forces(r, acc, jrk, pot, aa, ja)
        # i-particles not in the j-set (no self) and h2 on an exact boundary
        xi = c.x[:2] + 0.5
        acc, jrk, pot, lst = O.regf_fp64(c.m, c.x, c.v, c.h2()[:2], c.dtr[:2], xi, c.v[:2], 64, 63)
        r = nb.regf(c.h2()[:2], c.dtr[:2], xi, c.v[:2], 64, 63)
        assert rows_equal(r.list, lst) == []
        d2 = np.sum((c.x[5] - c.x[0]) ** 2)   # body 5 exactly at r2 == h2: not a neighbour
        acc, jrk, pot, lst = O.regf_fp64(c.m, c.x, c.v, [d2], [0.0], c.x[:1], c.v[:1], 64, 63)
        r = nb.regf([d2], [0.0], c.x[:1], c.v[:1], 64, 63)
        assert rows_equal(r.list, lst) == [] and 5 not in r.neighbours(0)


def test_errors_are_reported(lib):
    c = ics.plummer(64, seed=1, nb_target=5.0)
    with GpuNb(64) as nb:
        with pytest.raises(GpunbError) as e:
            nb.send(np.ones(65), np.zeros((65, 3)), np.zeros((65, 3)))
        assert e.value.code == 5
        x = c.x.copy()
        x[3, 1] = np.nan
        with pytest.raises(GpunbError) as e:
            nb.send(c.m, x, c.v)
        assert e.value.code == 3
        nb.send(c.m, c.x, c.v)
        with pytest.raises(GpunbError) as e:
            nb.regf(c.h2()[:4], c.dtr[:4], c.x[:4], c.v[:4], 8, 8)   # nnbmax > lmax-1
        assert e.value.code == 2
        xi = c.x[:4].copy()
        xi[0, 0] = np.nan
        with pytest.raises(GpunbError) as e:
            nb.regf(c.h2()[:4], c.dtr[:4], xi, c.v[:4], 8, 7)
        assert e.value.code == 3
        # the library stays usable after a reported error
        r = nb.regf(c.h2()[:4], c.dtr[:4], c.x[:4], c.v[:4], 8, 7)
        assert np.all(np.isfinite(r.acc))


def test_bounded_wait_gives_up_and_the_context_stays_usable(lib):
    """A device wait that nothing completes gives up after its poll limit and
    records GPUNB_E_TIMEOUT; the host reads it and the next calls work."""
    g = load_golden("plummer2048_equal")
    lib.gpunb_clear_error()
    with GpuNb(len(g["m"])):
        assert lib.gpunb_test_bounded_wait(1000, None) == 0
        assert lib.gpunb_device_status(None) == 6           # GPUNB_E_TIMEOUT
        lib.gpunb_clear_error()
        assert lib.gpunb_device_status(None) == 0
    res = run_golden(g)
    assert rows_equal(res.list, unpack_list(g["fp64_cnt"], g["fp64_ids"], int(g["lmax"]))) == []
    check_forces(res, g["fp64_acc"], g["fp64_jrk"], g["fp64_pot"], g["fp64_accabs"],
                 g["fp64_jrkabs"])


def test_allocation_failure_is_reported_and_recovered(lib):
    g = load_golden("plummer2048_equal")
    lib.gpunb_clear_error()
    with GpuNb(len(g["m"])) as nb:
        lib.gpunb_test_fail_allocs(1)          # the first send's tile buffer
        try:
            with pytest.raises(GpunbError) as e:
                nb.send(g["m"], g["x"], g["v"])
            assert e.value.code == 8
        finally:
            lib.gpunb_test_fail_allocs(0)
        nb.send(g["m"], g["x"], g["v"])
        ii = g["ii"]
        res = nb.regf(g["h2"], g["dtr"], g["x"][ii], g["v"][ii], int(g["lmax"]),
                      int(g["nnbmax"]), int(g["m_flag"]))
    assert rows_equal(res.list, unpack_list(g["fp64_cnt"], g["fp64_ids"], int(g["lmax"]))) == []
    check_forces(res, g["fp64_acc"], g["fp64_jrk"], g["fp64_pot"], g["fp64_accabs"],
                 g["fp64_jrkabs"])


def test_gpupot_golden(lib):
    g = load_golden("pot_plummer2048")
    p = gpupot(g["m"], g["x"])
    assert (np.abs(p - g["fp64_all"]) / g["fp64_all"]).max() < 1e-6
    p = gpupot(g["m"], g["x"], istart=int(g["istart"]), ni=int(g["ni"]))
    assert (np.abs(p - g["fp64_sub"]) / g["fp64_sub"]).max() < 1e-6


def test_gpupot_coincident_and_large(lib):
    c = ics.plummer(20000, seed=3, masses="kroupa")
    m, x = c.m.copy(), c.x.copy()
    x[10] = x[11]                      # coincident pair: skipped both ways
    p = gpupot(m, x)
    samp = np.arange(0, 20000, 97)
    o = np.array([O.pot_fp64(m, x, int(i) + 1, 1)[0] for i in samp])
    assert (np.abs(p[samp] - o) / o).max() < 1e-6
    assert np.isfinite(p[10]) and np.isfinite(p[11])


def test_gpupot_morton_tiles(lib, plummer64k):
    """gpupot_ runs on Morton-ordered tiles with tile-relative coordinates for
    far tiles: the whole set, a sub-range (its own order), a clump of bodies
    at one point (a tile of radius 0), against the FP64 oracle; and a call
    between gpunb_send_ and gpunb_regf_ leaves the regular force unchanged,
    bit for bit."""
    c = plummer64k
    p = gpupot(c.m, c.x)
    samp = np.arange(0, c.n, 211)
    o = np.array([O.pot_fp64(c.m, c.x, int(i) + 1, 1)[0] for i in samp])
    assert (np.abs(p[samp] - o) / o).max() < 1e-6
    istart, ni = 12345, 20000
    q = gpupot(c.m, c.x, istart=istart, ni=ni)
    ref = p[istart - 1:istart - 1 + ni]
    assert (np.abs(q - ref) / ref).max() < 1e-6
    qs = np.arange(0, ni, 97)
    o = np.array([O.pot_fp64(c.m, c.x, istart + int(k), 1)[0] for k in qs])
    assert (np.abs(q[qs] - o) / o).max() < 1e-6
    # 300 bodies at one point: they see each other at r = 0 (skipped)
    m, x = c.m[:4096].copy(), c.x[:4096].copy()
    x[:300] = x[300]
    r = gpupot(m, x)
    idx = np.r_[0:5, 295:305, 4000:4096:7]
    o = np.array([O.pot_fp64(m, x, int(i) + 1, 1)[0] for i in idx])
    assert np.all(np.isfinite(r)) and (np.abs(r[idx] - o) / o).max() < 1e-6
    # tiny and ragged sets: one body (nothing at r > 0), two, one tile plus one
    assert gpupot(c.m[:1], c.x[:1])[0] == 0.0
    for k in (2, 129):
        r = gpupot(c.m[:k], c.x[:k])
        o = O.pot_fp64(c.m[:k], c.x[:k], 1, k)
        assert (np.abs(r - o) / o).max() < 1e-6
    act = ics.active_set(c.n, 1024, seed=5)
    h2 = c.h2()
    with GpuNb(c.n) as nb:
        nb.send(c.m, c.x, c.v)
        r1 = nb.regf(h2[act], c.dtr[act], c.x[act], c.v[act], 513, 512)
        gpupot(c.m[::2], c.x[::2])
        r2 = nb.regf(h2[act], c.dtr[act], c.x[act], c.v[act], 513, 512)
    for a, b in ((r1.acc, r2.acc), (r1.jrk, r2.jrk), (r1.pot, r2.pot), (r1.list, r2.list)):
        assert np.array_equal(a, b)


def test_profile_counters(lib, capfd):
    """gpunb_profile_ prints the reference's line (gpunb.velocity.cu:882-902):
    sends and regular calls since the last profile, <Ni> = active particles
    per send, a positive rate; then resets, so a second call prints nothing."""
    c = ics.plummer(4096, seed=8, nb_target=50.0)
    h2 = c.h2()
    with GpuNb(c.n) as nb:
        nb.profile()
        capfd.readouterr()
        nb.send(c.m, c.x, c.v)
        nb.send(c.m, c.x, c.v)
        for k in (100, 200, 300):
            nb.regf(h2[:k], c.dtr[:k], c.x[:k], c.v[:k], 129, 128)
        nb.profile()
        err = capfd.readouterr().err
        nb.profile()
        again = capfd.readouterr().err
    line = [ln for ln in err.splitlines() if "Reg.F" in ln][-1]
    f = line.replace("(s)", "").split()
    assert int(f[f.index("Nsend") + 1]) == 2 and int(f[f.index("Ngrav") + 1]) == 3
    assert int(f[f.index("<Ni>") + 1]) == 300
    assert float(f[f.index("Perf.(Gflops)") + 1]) > 0
    assert "Reg.F" not in again


def test_host_paths_identical(lib, plummer64k):
    """Direct host arrays (device writes the rows) and pinned staging give the
    same bytes, including overflow rows and blocks above the host-scatter
    threshold."""
    c = plummer64k
    g = load_golden("overflow_plummer512")
    ii = g["ii"]
    act = ics.active_set(c.n, 16384, seed=3)
    h2 = c.h2()
    cases = [(g["m"], g["x"], g["v"], g["h2"], g["dtr"], g["x"][ii], g["v"][ii],
              int(g["lmax"]), int(g["nnbmax"])),
             (c.m, c.x, c.v, h2[act], c.dtr[act], c.x[act], c.v[act], 257, 256)]
    with GpuNb(c.n) as nb:
        for m, x, v, hh, dtr, xi, vi, lmax, nnbmax in cases:
            out = []
            for mode in (1, 0):
                nb.set_host_path(bool(mode))
                nb.send(m, x, v)
                out.append(nb.regf(hh, dtr, xi, vi, lmax, nnbmax))
            nb.set_host_path(True)
            a, b = out
            assert np.array_equal(a.list, b.list)
            assert np.array_equal(a.acc, b.acc) and np.array_equal(a.jrk, b.jrk)
            assert np.array_equal(a.pot, b.pot)
