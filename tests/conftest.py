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
