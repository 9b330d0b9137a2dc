"""Batched clusters (one persistent launch for many independent j-sets):
every set's forces, potentials and neighbour lists against the FP64 oracle of
that set alone, and bit-for-bit repeatability."""
import numpy as np
import pytest

from conftest import check_split, rows_equal
from nbody6ppgpu_gb300 import ics
from oracle import oracle as O

pytestmark = pytest.mark.gpu

SPECS = [  # (N, seed, nb_target, active count)
    (512, 21, 20.0, 1), (777, 22, 30.0, 777), (2048, 23, 50.0, 100), (3001, 24, 40.0, 3001),
    (8192, 25, 80.0, 2048), (600, 26, 25.0, 37), (130, 27, 10.0, 129),
]
NNBMAX = 256


@pytest.fixture(scope="module")
def batch_case():
    sets, act, h2s, dtrs = [], [], [], []
    for n, seed, tgt, k in SPECS:
        c = ics.plummer(n, seed=seed, masses="kroupa", nb_target=tgt)
        a = ics.active_set(n, k, seed=seed)
        sets.append((c.m, c.x, c.v))
        act.append(a)
        h2s.append(c.h2()[a])
        dtrs.append(c.dtr[a])
    return sets, act, h2s, dtrs


def run_batch(batch_case, variant=-1):
    from nbody6ppgpu_gb300.batch import DeviceBatch
    from nbody6ppgpu_gb300.gpunb import GpuNb
    sets, act, h2s, dtrs = batch_case
    with GpuNb(1 << 16) as nb:
        nb.set_launch(variant, 0)
        b = DeviceBatch(sets, act, NNBMAX)
        b.set_radii(h2s, dtrs)
        b.send()
        b.regf()
        res = b.results()
        plan = b.last_plan()
    return res, plan


def test_batch_matches_oracle_per_set(batch_case):
    sets, act, h2s, dtrs = batch_case
    res, plan = run_batch(batch_case)
    assert plan[1] > len(SPECS)
    for c, ((m, x, v), a) in enumerate(zip(sets, act)):
        acc, jrk, pot, lst, aa, ja = O.regf_fp64(m, x, v, h2s[c], dtrs[c], x[a], v[a],
                                                 NNBMAX + 1, NNBMAX, with_abs=True)
        got = np.zeros_like(lst)
        for i, ids in enumerate(res.lists[c]):
            got[i, 0] = res.nnb[c][i]
            if res.nnb[c][i] > 0:
                got[i, 1:1 + len(ids)] = ids
        assert rows_equal(got, lst) == [], c
        check_split(res.acc[c], res.jrk[c], res.pot[c], acc, jrk, pot, aa, ja,
                    ok=lst[:, 0] >= 0)


@pytest.mark.parametrize("variant", [2, 4])
def test_batch_repeatable_and_shape_independent_lists(batch_case, variant):
    r1, _ = run_batch(batch_case, variant)
    r2, _ = run_batch(batch_case, variant)
    for c in range(len(SPECS)):
        assert np.array_equal(r1.acc[c], r2.acc[c]) and np.array_equal(r1.nnb[c], r2.nnb[c])
        for a, b in zip(r1.lists[c], r2.lists[c]):
            assert np.array_equal(a, b)


def test_batch_graph_replay_matches_eager(batch_case):
    from nbody6ppgpu_gb300.batch import DeviceBatch
    from nbody6ppgpu_gb300.gpunb import GpuNb
    sets, act, h2s, dtrs = batch_case
    eager, _ = run_batch(batch_case)
    with GpuNb(1 << 16) as nb:
        nb.lib.gpunb_set_graphs(1)
        try:
            b = DeviceBatch(sets, act, NNBMAX)
            b.set_radii(h2s, dtrs)
            for _ in range(3):        # eager + capture, then two replays
                b.send()
                b.regf()
                r = b.results()
                for c in range(len(SPECS)):
                    assert np.array_equal(r.acc[c], eager.acc[c])
                    assert np.array_equal(r.pot[c], eager.pot[c])
                    assert np.array_equal(r.nnb[c], eager.nnb[c])
                    for a, e in zip(r.lists[c], eager.lists[c]):
                        assert np.array_equal(a, e)
        finally:
            nb.lib.gpunb_set_graphs(0)


def test_batch_autotune_picks_a_shape_on_the_batch_and_keeps_it(batch_case, tmp_path):
    """gpunb_set_autotune(1): the first call of a batch shape times every
    (variant, work items per block) on that batch and keeps the fastest; the
    results stay within the parity bound and equal a second call's bit for
    bit, and the choice lands in the saved cache under the batch's bucket."""
    from nbody6ppgpu_gb300.batch import DeviceBatch
    from nbody6ppgpu_gb300.gpunb import GpuNb
    sets, act, h2s, dtrs = batch_case
    empty = tmp_path / "empty.txt"
    empty.write_text("")
    with GpuNb(1 << 16) as nb:
        assert nb.tune_load(empty) == 0
        prev = nb.set_autotune(True)
        try:
            b = DeviceBatch(sets, act, NNBMAX)
            b.set_radii(h2s, dtrs)
            b.send()
            b.regf()
            r1 = b.results()
            plan1 = b.last_plan()
            b.regf()
            r2 = b.results()
            plan2 = b.last_plan()
        finally:
            nb.set_autotune(prev)
        saved = tmp_path / "tune.txt"
        assert nb.tune_save(saved) >= 1
    assert plan1 == plan2 and plan1[0] in (2, 4, 6)
    key_flags = [int(l.split()[0]) >> 62 for l in saved.read_text().splitlines()]
    assert 1 in key_flags                       # an entry under the batch flag
    for c, ((m, x, v), a) in enumerate(zip(sets, act)):
        assert np.array_equal(r1.acc[c], r2.acc[c]) and np.array_equal(r1.nnb[c], r2.nnb[c])
        acc, jrk, pot, lst, aa, ja = O.regf_fp64(m, x, v, h2s[c], dtrs[c], x[a], v[a],
                                                 NNBMAX + 1, NNBMAX, with_abs=True)
        assert np.array_equal(np.asarray(r1.nnb[c]), lst[:, 0]), c
        check_split(r1.acc[c], r1.jrk[c], r1.pot[c], acc, jrk, pot, aa, ja, ok=lst[:, 0] >= 0)


_PLAN_CHILD = r"""
import sys
sys.path.insert(0, {root!r})
sys.path.insert(0, {tests!r})
import numpy as np
from nbody6ppgpu_gb300 import ics
from nbody6ppgpu_gb300.batch import DeviceBatch
from nbody6ppgpu_gb300.gpunb import GpuNb
from test_batch_gpu import SPECS, NNBMAX
sets, act, h2s, dtrs = [], [], [], []
for n, seed, tgt, k in SPECS:
    c = ics.plummer(n, seed=seed, masses="kroupa", nb_target=tgt)
    a = ics.active_set(n, k, seed=seed)
    sets.append((c.m, c.x, c.v)); act.append(a); h2s.append(c.h2()[a]); dtrs.append(c.dtr[a])
with GpuNb(1 << 16) as nb:
    if {warm}:
        c = ics.plummer(4096, seed=1, nb_target=50.0)
        nb.send(c.m, c.x, c.v)
        for v in range(nb.lib.gpunb_num_variants()):
            nb.set_launch(v, 0)
            nb.regf(c.h2(), c.dtr, c.x, c.v, 257, 256)
        nb.set_launch(-1, 0)
    b = DeviceBatch(sets, act, NNBMAX)
    b.set_radii(h2s, dtrs)
    b.send()
    b.regf()
    print("PLAN", *b.last_plan())
"""


def test_first_launch_plans_with_full_residency():
    """A batch whose plan is made before any pair kernel has run in the
    process (so before any kernel's shared-memory opt-in) gets the same work
    items as one made after every kernel shape has run: the occupancy
    behind the plan counts every resident block from the first call."""
    import subprocess
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parents[1]
    plans = []
    for warm in (False, True):
        src = _PLAN_CHILD.format(root=str(root), tests=str(root / "tests"), warm=warm)
        r = subprocess.run([sys.executable, "-c", src], capture_output=True, text=True,
                           timeout=600)
        assert r.returncode == 0, r.stderr[-2000:]
        line = [ln for ln in r.stdout.splitlines() if ln.startswith("PLAN")][-1]
        plans.append(tuple(int(t) for t in line.split()[1:]))
    assert plans[0] == plans[1], plans
