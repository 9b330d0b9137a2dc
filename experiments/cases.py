"""One regular-force block on a seeded cluster, through the host ABI: the
case the kernel profiles are taken on.

    python -m experiments.cases --model plummer --n 65536 --ni 65536 --reps 4

Sends the j-set once and calls gpunb_regf_ `reps` times on the same active
set (the first call warms the library up; a profiler is pointed at a later
one).  Prints the per-call kernel time from the library's CUDA events and
the mean neighbour count.

    python -m experiments.cases --irr 0 --n 65536 --ni 65536 --reps 4

adds, after the regular block, `reps` irregular-force calls (irr_simd_*,
precision 0 = split FP32, 1 = FP64) of `ni` particles with the neighbour
lists of a full regular block (self removed).

    python -m experiments.cases --batched --reps 4

runs instead `reps` steps (batched send + regf, graphs on) of the 256-cluster
workload of the bench, a 256 MB fill between steps marking the step bounds
in a launch list.
"""
from __future__ import annotations

import argparse

from nbody6ppgpu_gb300 import ics
from nbody6ppgpu_gb300.gpunb import GpuNb


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--model", default="plummer", choices=["plummer", "king"])
    ap.add_argument("--n", type=int, default=65536)
    ap.add_argument("--ni", type=int, default=65536)
    ap.add_argument("--reps", type=int, default=4)
    ap.add_argument("--nnbmax", type=int, default=512)
    ap.add_argument("--target", type=float, default=100.0)
    ap.add_argument("--irr", type=int, default=-1, help="irregular force precision (0, 1)")
    ap.add_argument("--batched", action="store_true", help="the 256-cluster batched step")
    a = ap.parse_args()
    if a.batched:
        batched(a)
        return
    if a.model == "king":
        c = ics.king(a.n, seed=4, nb_target=a.target)
    else:
        c = ics.plummer(a.n, seed=2, masses="kroupa", nb_target=a.target)
    act = ics.active_set(c.n, a.ni, seed=a.ni)
    h2 = c.h2()
    with GpuNb(c.n) as nb:
        nb.send(c.m, c.x, c.v)
        nb.set_timing(True)
        for _ in range(a.reps):
            r = nb.regf(h2[act], c.dtr[act], c.x[act], c.v[act], a.nnbmax + 1, a.nnbmax)
        times = nb.kernel_times()
    print(f"{a.model} N={c.n} ni={a.ni}: kernel ms per call {[round(t, 4) for t in times]}, "
          f"mean count {r.list[:, 0].mean():.1f}")
    if a.irr >= 0:
        irregular(c, h2, a)


def batched(a):
    import time

    import torch

    from nbody6ppgpu_gb300 import workloads
    from nbody6ppgpu_gb300.batch import DeviceBatch
    from nbody6ppgpu_gb300.gpunb import load
    lib = load()
    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(dev)
    sets, active, h2, dtr, _ = workloads.clusters256()
    nb = GpuNb(sum(len(s[0]) for s in sets))   # the library open, as the integrator has it
    b = DeviceBatch(sets, active, 512, device=0, stream=stream)
    b.set_radii(h2, dtr)
    lib.gpunb_set_graphs(1)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    ms = []
    for _ in range(a.reps):
        with torch.cuda.stream(stream):
            flush.fill_(1)
        torch.cuda.synchronize()
        t = time.perf_counter()
        b.send()
        b.regf()
        torch.cuda.synchronize()
        ms.append(1e3 * (time.perf_counter() - t))
    print(f"batched 256 clusters: {b.total_ni} active, plan {b.last_plan()}, "
          f"ms per step {[round(t, 3) for t in ms]}")
    nb.close()


def irregular(c, h2, a):
    import time

    import numpy as np

    from nbody6ppgpu_gb300.irr import IrrSimd
    lmax = a.nnbmax + 1
    with GpuNb(c.n) as nb:
        nb.send(c.m, c.x, c.v)
        r = nb.regf(h2, c.dtr, c.x, c.v, lmax, a.nnbmax)
    lists = np.zeros_like(r.list)
    for i in range(c.n):
        ids = r.list[i, 1:1 + max(int(r.list[i, 0]), 0)]
        ids = ids[ids != i]
        lists[i, 0] = len(ids)
        lists[i, 1:1 + len(ids)] = ids
    rng = np.random.default_rng(7)
    f = rng.normal(0.0, 0.5, (c.n, 3))
    fdot = rng.normal(0.0, 0.5, (c.n, 3))
    t0 = 1.0 - rng.uniform(0.0, 2e-3, c.n)
    act = rng.permutation(c.n)[:a.ni]
    out = (np.zeros((a.ni, 3)), np.zeros((a.ni, 3)), np.zeros(a.ni, dtype=np.int32))
    with IrrSimd(c.n, lmax, precision=a.irr) as irr:
        irr.set_jp(c.x, c.v, f, fdot, c.m, t0)
        irr.set_lists(lists)
        ms = []
        for _ in range(a.reps):
            t = time.perf_counter()
            irr.firr(1.0, act, out=out)
            ms.append(1e3 * (time.perf_counter() - t))
    print(f"irregular precision {a.irr} ni={a.ni}: {int(lists[act, 0].sum())} pairs, "
          f"host-ABI ms per call {[round(t, 3) for t in ms]}")


if __name__ == "__main__":
    main()
