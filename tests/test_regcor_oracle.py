"""The host restatement of REGCOR_GPU (oracle/regcor_oracle.py) on small
hand-checkable cases: its Fortran-style list comparison (sentinels, JJLIST)
finds exactly the set differences of the old and new lists, the force change
it forms is the sum over gained minus lost neighbours, and the retention of
small-step neighbours keeps exactly the eligible ones."""
import math

import numpy as np

from oracle import regcor_oracle as R


def _state(n, lmax, rng):
    s = {k: np.zeros((n, 3)) for k in ("x", "xdot", "x0", "x0dot", "fi", "fidot", "fr", "frdot",
                                       "d0", "d0r", "d1r", "d2r", "d3r", "xn", "xndot")}
    s["x"] = rng.normal(0.0, 1.0, (n, 3))
    s["xdot"] = rng.normal(0.0, 0.5, (n, 3))
    s["x0"] = s["x"] - 0.01 * s["xdot"]
    s["x0dot"] = s["xdot"].copy()
    s["fr"] = rng.normal(0.0, 1.0, (n, 3))
    s["frdot"] = rng.normal(0.0, 1.0, (n, 3))
    for k in ("body", "t0r", "stepr", "step", "t0", "timenw", "rs"):
        s[k] = np.zeros(n)
    s["body"][:] = 1.0 / n
    s["t0r"][:] = 1.0 - 1.0 / 64
    s["stepr"][:] = 1.0 / 64
    s["step"][:] = 1.0 / 256
    s["t0"][:] = 1.0 - 1.0 / 256
    s["rs"][:] = 0.5
    s["list"] = np.zeros((n, lmax), dtype=np.int64)
    s["h"] = None
    return s


def _params(n, lmax):
    return dict(time=1.0, dtmin=1e-6, smin=1e-3, smax=0.125, etar=0.02, tidal4=0.0, kz14=0,
                m_flag=0, nnbmax=lmax - 2, n=n, ntot=n, ifirst=1, lmax=lmax, nnbopt=10,
                nb_flag=1, rscale=0.8, rc=0.3, rsfac=50.0, bodym=1.0 / n, rdens=[0.0, 0.0, 0.0])


def test_list_comparison_finds_the_set_differences():
    rng = np.random.default_rng(3)
    n, lmax = 200, 40
    for trial in range(200):
        s = _state(n, lmax, rng)
        p = _params(n, lmax)
        i1 = int(rng.integers(1, n + 1))
        pool = [j for j in range(1, n + 1) if j != i1]
        old = sorted(rng.choice(pool, int(rng.integers(0, 20)), replace=False).tolist())
        new = sorted(rng.choice(pool, int(rng.integers(1, 20)), replace=False).tolist())
        s["list"][i1 - 1, :len(old) + 1] = [len(old)] + old
        xi, vi = s["x"][i1 - 1], s["xdot"][i1 - 1]
        want = np.zeros(3)
        for j in set(new) - set(old):
            want += R._pair(xi, vi, s["x"][j - 1], s["xdot"][j - 1], s["body"][j - 1])[0]
        for j in set(old) - set(new):
            want -= R._pair(xi, vi, s["x"][j - 1], s["xdot"][j - 1], s["body"][j - 1])[0]
        fi0 = s["fi"][i1 - 1].copy()
        counters = [0, 0, 0, 0]
        row = [len(new)] + new
        R.regcor_body(i1, list(s["fr"][i1 - 1]), list(s["frdot"][i1 - 1]), row, s, p, counters)
        assert counters[2] == (len(set(new) ^ set(old)) if old else len(new))
        assert np.allclose(s["fi"][i1 - 1] - fi0, want, rtol=1e-12, atol=1e-12)
        got = s["list"][i1 - 1]
        assert got[0] == len(new) and list(got[1:1 + len(new)]) == new


def test_small_step_neighbours_inside_two_radii_are_kept():
    rng = np.random.default_rng(5)
    n, lmax = 60, 40
    s = _state(n, lmax, rng)
    p = _params(n, lmax)
    i1 = 7
    xi = s["x"][i1 - 1]
    s["rs"][i1 - 1] = 0.6
    old = [2, 3, 4, 5, 9]
    new = [3, 9]
    s["step"][[1, 3, 4]] = 1e-4           # bodies 2, 4, 5: steps below SMIN
    s["x"][1] = xi + [0.5, 0.0, 0.0]      # 2: inside 2 RS -> kept
    s["x"][3] = xi + [2.0, 0.0, 0.0]      # 4: outside 2 RS -> lost
    s["x"][4] = xi + [0.0, 0.9, 0.0]      # 5: inside -> kept
    s["list"][i1 - 1, :len(old) + 1] = [len(old)] + old
    fr0 = s["fr"][i1 - 1].copy()
    freg = list(fr0)
    f2 = R._pair(xi, s["xdot"][i1 - 1], s["x"][1], s["xdot"][1], s["body"][1])[0]
    f5 = R._pair(xi, s["xdot"][i1 - 1], s["x"][4], s["xdot"][4], s["body"][4])[0]
    row = [len(new)] + new
    counters = [0, 0, 0, 0]
    R.regcor_body(i1, freg, list(s["frdot"][i1 - 1]), row, s, p, counters)
    assert row == [4, 2, 3, 5, 9] and counters[1] == 2
    assert np.allclose(s["fr"][i1 - 1], fr0 - np.asarray(f2) - np.asarray(f5), rtol=1e-12,
                       atol=1e-14)
    assert s["list"][i1 - 1, 0] == 4 and list(s["list"][i1 - 1, 1:5]) == [2, 3, 5, 9]
    assert math.isclose(s["t0r"][i1 - 1], 1.0)


def test_kept_neighbours_enter_an_empty_new_list_in_order():
    """An empty new list with small-step old neighbours inside 2 RS: they are
    kept in ascending order, and the list matches the forces moved (the
    reference's loop would displace the first kept body by the last old
    member here)."""
    rng = np.random.default_rng(9)
    n, lmax = 40, 20
    s = _state(n, lmax, rng)
    p = _params(n, lmax)
    i1 = 4
    xi = s["x"][i1 - 1]
    s["rs"][i1 - 1] = 0.6
    old = [2, 3, 5, 8]
    s["step"][[1, 4]] = 1e-4                 # bodies 2 and 5
    s["x"][1] = xi + [0.3, 0.0, 0.0]
    s["x"][4] = xi + [0.0, -0.4, 0.0]
    s["list"][i1 - 1, :len(old) + 1] = [len(old)] + old
    row = [0]
    counters = [0, 0, 0, 0]
    R.regcor_body(i1, list(s["fr"][i1 - 1]), list(s["frdot"][i1 - 1]), row, s, p, counters)
    assert row == [2, 2, 5] and counters[1] == 2
    assert list(s["list"][i1 - 1, :3]) == [2, 2, 5]
