"""Sharding of the regular-force path over processes (i-split and j-split),
on CPU: the partition rules against the Fortran/C formulas, the j-split merge
against one unsharded computation, and two gloo ranks running both schemes
end to end.  The per-rank computation here is the FP64 oracle; on GPUs it is
the library."""
import os
import socket
import tempfile

import numpy as np
import pytest

from nbody6ppgpu_gb300 import ics, shard
from nbody6ppgpu_gb300.gpunb import RegfResult
from oracle import oracle as O

LMAX, NNBMAX = 129, 128


def _case(n=700, seed=3):
    c = ics.plummer(n, seed=seed, nb_target=30.0)
    act = ics.active_set(n, 301, seed=5)
    return c, act


def _oracle(m, x, v, *args):
    return RegfResult(*O.regf_fp64(m, x, v, *args))


def _oracle_fn(m, x, v):
    return lambda h2, dtr, xi, vi, lmax, nnbmax, m_flag=0: _oracle(
        m, x, v, h2, dtr, xi, vi, lmax, nnbmax, m_flag)


def test_i_split_blocks():
    s, c = shard.i_split(10, 4)
    assert list(c) == [3, 3, 2, 2] and list(s) == [0, 3, 6, 8]
    s, c = shard.i_split(2, 4)
    assert list(c) == [1, 1, 0, 0] and list(s) == [0, 1, 2, 2]
    s, c = shard.i_split(0, 3)
    assert list(c) == [0, 0, 0]


def test_j_offsets():
    assert list(shard.j_offsets(10, 3)) == [0, 3, 6, 10]
    assert list(shard.j_offsets(2, 4)) == [0, 0, 1, 1, 2]


@pytest.mark.parametrize("size", [2, 3, 5])
def test_j_split_merge_equals_unsharded(size):
    c, act = _case()
    h2 = c.h2()
    args = (h2[act], c.dtr[act], c.x[act], c.v[act], LMAX, NNBMAX)
    ref = _oracle(c.m, c.x, c.v, *args)
    joff = shard.j_offsets(c.n, size)
    parts = [_oracle(c.m[a:b], c.x[a:b], c.v[a:b], *args) for a, b in zip(joff, joff[1:])]
    got = shard.merge_j_parts(parts, joff, NNBMAX)
    assert np.array_equal(got.list, ref.list)
    for k in ("acc", "jrk"):
        a, b = getattr(got, k), getattr(ref, k)
        assert np.max(np.linalg.norm(a - b, axis=1) / np.linalg.norm(b, axis=1)) < 1e-13
    assert np.max(np.abs(got.pot - ref.pot) / ref.pot) < 1e-13


def test_j_split_merge_overflow():
    c, act = _case()
    h2 = c.h2()
    small = 31
    args = (h2[act], c.dtr[act], c.x[act], c.v[act], LMAX, small)
    ref = _oracle(c.m, c.x, c.v, *args)
    joff = shard.j_offsets(c.n, 3)
    parts = [_oracle(c.m[a:b], c.x[a:b], c.v[a:b], *args) for a, b in zip(joff, joff[1:])]
    got = shard.merge_j_parts(parts, joff, small)
    assert np.any(ref.list[:, 0] < 0) and np.any(ref.list[:, 0] > 0)
    assert np.array_equal(got.list[:, 0], ref.list[:, 0])
    ok = ref.list[:, 0] >= 0
    assert np.array_equal(got.list[ok], ref.list[ok])


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, size, port, out):
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=size)
    try:
        c, act = _case()
        h2 = c.h2()
        args = (h2[act], c.dtr[act], c.x[act], c.v[act], LMAX, NNBMAX)
        full = shard.ShardedRegf(_oracle_fn(c.m, c.x, c.v))
        ri = full.i_split(*args)
        joff = shard.j_offsets(c.n, size)
        a, b = int(joff[rank]), int(joff[rank + 1])
        sl = shard.ShardedRegf(_oracle_fn(c.m[a:b], c.x[a:b], c.v[a:b]))
        rj = sl.j_split(joff, *args)
        np.savez(os.path.join(out, f"r{rank}.npz"), ia=ri.acc, ij=ri.jrk, ip=ri.pot, il=ri.list,
                 ja=rj.acc, jj=rj.jrk, jp=rj.pot, jl=rj.list)
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_i_and_j_split():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    c, act = _case()
    h2 = c.h2()
    ref = _oracle(c.m, c.x, c.v, h2[act], c.dtr[act], c.x[act], c.v[act], LMAX, NNBMAX)
    with tempfile.TemporaryDirectory() as out:
        mp.start_processes(_rank_main, args=(2, _free_port(), out), nprocs=2, join=True,
                           start_method="spawn")
        res = [dict(np.load(os.path.join(out, f"r{r}.npz"))) for r in range(2)]
    for r in res:
        # i-split: exactly the unsharded rows on every rank
        assert np.array_equal(r["il"], ref.list)
        assert np.array_equal(r["ia"], ref.acc) and np.array_equal(r["ip"], ref.pot)
        # j-split: same lists, sums to FP64 rounding
        assert np.array_equal(r["jl"], ref.list)
        assert np.max(np.abs(r["ja"] - ref.acc)) < 1e-12 * np.max(np.abs(ref.acc))
    assert np.array_equal(res[0]["ja"], res[1]["ja"])
