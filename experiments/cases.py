"""One regular-force block on a seeded cluster, through the host ABI: the
case the kernel profiles are taken on.

    python -m experiments.cases --model plummer --n 65536 --ni 65536 --reps 4

Sends the j-set once and calls gpunb_regf_ `reps` times on the same active
set (the first call warms the library up; a profiler is pointed at a later
one).  Prints the per-call kernel time from the library's CUDA events and
the mean neighbour count.
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
    a = ap.parse_args()
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


if __name__ == "__main__":
    main()
