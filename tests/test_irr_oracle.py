"""The FP64 oracle of the irregular force (oracle/irr_fp64.c) against the
golden vectors of the reference's own src/Main/irr.avx.cpp (FP32 with
double-single positions), and against the reference library itself where it
was compiled (x86_64 hosts with the reference sources)."""
import numpy as np
import pytest

from conftest import load_golden, rel_vec_err
from oracle import oracle as O

REF_P99 = 2e-6    # the reference's FP32 arithmetic against FP64
REF_MAX = 2e-5

CASES = ["irr_plummer2048", "irr_ragged_n37"]


def _run_oracle(g):
    return O.irr_fp64(g["x0"], g["v0"], g["f"], g["fdot"], g["m"], g["t0"], g["lists"],
                      float(g["ti"]), g["active"])


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_stored_fp64(name):
    g = load_golden(name)
    a, j, nid = _run_oracle(g)
    ok = np.linalg.norm(g["fp64_acc"], axis=1) > 0
    assert np.max(rel_vec_err(a[ok], g["fp64_acc"][ok])) < 1e-13
    assert np.max(rel_vec_err(j[ok], g["fp64_jrk"][ok])) < 1e-13
    assert np.array_equal(nid, g["fp64_nnbid"])


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference_irr_avx(name):
    g = load_golden(name)
    a, j, nid = _run_oracle(g)
    ok = np.linalg.norm(a, axis=1) > 0
    ea = rel_vec_err(g["ref_acc"][ok], a[ok])
    ej = rel_vec_err(g["ref_jrk"][ok], j[ok])
    assert np.percentile(ea, 99) < REF_P99 and ea.max() < REF_MAX
    assert np.percentile(ej, 99) < REF_P99 and ej.max() < REF_MAX
    assert np.array_equal(nid, g["ref_nnbid"])
    # empty lists: zero force, nearest id 0 (irr.avx.cpp:257-273)
    empty = g["lists"][g["active"], 0] == 0
    assert np.all(a[empty] == 0) and np.all(nid[empty] == 0)
    assert np.all(g["ref_nnbid"][empty] == 0)


def test_reference_library_if_built():
    if not O.RefIrrAVX.available():
        pytest.skip("reference irr.avx.cpp not built on this host (x86_64 + sources only)")
    g = load_golden("irr_ragged_n37")
    n, lmax = len(g["m"]), g["lists"].shape[1]
    r = O.RefIrrAVX(n, lmax)
    try:
        r.set_jp(g["x0"], g["v0"], g["f"], g["fdot"], g["m"], g["t0"])
        r.set_lists(g["lists"])
        a, j, nid = r.firr(float(g["ti"]), g["active"])
    finally:
        r.close()
    assert np.array_equal(a, g["ref_acc"]) and np.array_equal(nid, g["ref_nnbid"])


def test_abs_sums_bound_the_force_and_match_a_plain_loop():
    """oracle.irr_abs_sums (the S_i of the split-precision parity bound): at
    least |Q_i| for every particle, and equal to a plain per-pair loop."""
    g = load_golden("irr_plummer2048")
    args = (g["x0"], g["v0"], g["f"], g["fdot"], g["m"], g["t0"], g["lists"], float(g["ti"]),
            g["active"])
    a, j, _ = O.irr_fp64(*args)
    sa, sj = O.irr_abs_sums(*args)
    assert np.all(np.linalg.norm(a, axis=1) <= sa * (1 + 1e-12))
    assert np.all(np.linalg.norm(j, axis=1) <= sj * (1 + 1e-12))
    dt = (float(g["ti"]) - g["t0"])[:, None]
    x = g["x0"] + dt * (g["v0"] + dt * (g["f"] + dt * g["fdot"]))
    v = g["v0"] + 2.0 * dt * (g["f"] + 1.5 * dt * g["fdot"])
    for k in range(0, len(g["active"]), 97):
        i = int(g["active"][k])
        ta = tj = 0.0
        for jj in g["lists"][i, 1:1 + g["lists"][i, 0]]:
            dx, dv = x[jj] - x[i], v[jj] - v[i]
            r2 = float(dx @ dx)
            if r2 > 0.0:
                ta += g["m"][jj] / r2
                tj += np.linalg.norm(g["m"][jj] / r2 ** 1.5 * (dv - 3.0 * (dx @ dv) / r2 * dx))
        assert abs(sa[k] - ta) <= 1e-12 * ta and abs(sj[k] - tj) <= 1e-12 * tj
