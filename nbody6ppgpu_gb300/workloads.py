"""Seeded benchmark and test workloads named after the configurations they
stand for (synthetic inputs with the distributions of the reference's
set-up; no public data set is involved)."""
from __future__ import annotations

import math

import numpy as np

from . import ics


def clusters256(seed: int = 1000, n_sets: int = 256, nmin: int = 512, nmax: int = 16384,
                fmin: float = 2.0 ** -10):
    """Independent Plummer clusters, each with its own seed: N log-uniform in
    [nmin, nmax], Kroupa masses, active fraction log-uniform in [fmin, 1]
    (at least one active body), mean neighbour target uniform in [50, 150].
    Returns (sets, active, h2, dtr, targets): sets = [(m, x, v)], active =
    index arrays of the active blocks, h2/dtr of the active bodies."""
    rng = np.random.default_rng(seed)
    sets, active, h2, dtr, targets = [], [], [], [], []
    for k in range(n_sets):
        n = int(round(math.exp(rng.uniform(math.log(nmin), math.log(nmax)))))
        frac = math.exp(rng.uniform(math.log(fmin), 0.0))
        tgt = float(rng.uniform(50.0, 150.0))
        c = ics.plummer(n, seed=seed + 1 + k, masses="kroupa", nb_target=tgt,
                        exact_energy_max=0)
        ni = max(1, int(round(frac * n)))
        a = ics.active_set(n, ni, seed=seed + 1 + k)
        sets.append((c.m, c.x, c.v))
        active.append(a)
        h2.append(c.h2()[a])
        dtr.append(c.dtr[a])
        targets.append(tgt)
    return sets, active, h2, dtr, targets
