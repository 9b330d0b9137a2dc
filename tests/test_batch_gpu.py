"""Batched clusters (one persistent launch for many independent j-sets):
every set's forces, potentials and neighbour lists against the FP64 oracle of
that set alone, and bit-for-bit repeatability."""
import numpy as np
import pytest

from conftest import rel_vec_err, rows_equal
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
        ok = lst[:, 0] >= 0
        ea = rel_vec_err(res.acc[c][ok], acc[ok])
        ep = np.abs(res.pot[c][ok] - pot[ok]) / pot[ok]
        na = np.linalg.norm(res.acc[c][ok] - acc[ok], axis=1) / aa[ok]
        nj = np.linalg.norm(res.jrk[c][ok] - jrk[ok], axis=1) / ja[ok]
        assert np.percentile(ea, 99) < 1e-6 and ea.max() < 1e-5, (c, ea.max())
        assert ep.max() < 1e-6, c
        assert na.max() < 1e-6 and nj.max() < 1e-6, c


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
