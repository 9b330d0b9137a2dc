import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running")


def load_golden(name):
    return dict(np.load(GOLDEN / f"{name}.npz"))


def unpack_list(cnt, ids, lmax):
    """compact (counts, ids) -> LISTGP rows"""
    lst = np.zeros((len(cnt), lmax), dtype=np.int32)
    o = 0
    for i, c in enumerate(cnt):
        lst[i, 0] = c
        if c > 0:
            lst[i, 1:1 + c] = ids[o:o + c]
            o += c
    return lst


def rows_equal(a, b):
    """indices of rows whose count or accepted ids differ"""
    bad = []
    for i in range(a.shape[0]):
        ca, cb = int(a[i, 0]), int(b[i, 0])
        if ca != cb or (ca > 0 and not np.array_equal(a[i, 1:1 + ca], b[i, 1:1 + cb])):
            bad.append(i)
    return bad


def rel_vec_err(a, b):
    return np.linalg.norm(a - b, axis=1) / np.maximum(np.linalg.norm(b, axis=1), 1e-300)


def check_split(acc, jrk, pot, ref_acc, ref_jrk, ref_pot, accabs, jrkabs, ok=None):
    """The split-precision parity bound (oracle.parity_errors): per particle,
    force and jerk within 1e-6 of max(|Q_i|, S_i / KAPPA0), the potential
    within 1e-6 relative, and the plain relative errors of force and jerk
    within 1e-6 at the 99th percentile.  ok selects rows (accepted lists)."""
    from oracle import oracle as O
    if ok is not None:
        acc, jrk, pot, ref_acc, ref_jrk, ref_pot, accabs, jrkabs = (
            np.asarray(a)[ok] for a in (acc, jrk, pot, ref_acc, ref_jrk, ref_pot, accabs, jrkabs))
    e = O.parity_errors(acc, jrk, pot, ref_acc, ref_jrk, ref_pot, accabs, jrkabs)
    for q in ("acc", "jrk"):
        assert e[q]["bound_max"] <= O.SPLIT_TOL, (q, e[q])
        assert e[q]["p99"] <= O.SPLIT_TOL, (q, e[q])
    assert e["pot"]["max"] <= O.SPLIT_TOL, e["pot"]
    return e
