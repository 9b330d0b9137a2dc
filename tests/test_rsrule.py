"""The plain neighbour-radius rules (the predictor's fallback and baseline),
checked case by case against values worked out by hand from the Fortran:
src/Main/util_gpu.F:81-97 (overflow), src/Main/fpoly0.F:153-158 (fewer than
two members) and src/Main/regcor_gpu.F:120-253 (the update after a regular
step)."""
import math

import numpy as np
import pytest

from nbody6ppgpu_gb300 import rsrule


def params(**kw):
    p = dict(nnbopt=100, nnbmax=200, rscale=0.8, rc=0.3, rsfac=50.0, nb_flag=1, bodym=1.0)
    p.update(kw)
    return rsrule.RSParams(**p)


def one(rs, nnb, nnb0, x, v, dtr, p):
    out, tgt = rsrule.regcor_rs(np.array([rs]), np.array([nnb]), np.array([nnb0]),
                                np.array([x], dtype=float), np.array([v], dtype=float),
                                np.array([dtr]), p, return_target=True)
    return float(out[0]), float(tgt[0])


def test_overflow_rule():
    p = params()
    rs = np.ones(3)
    out = rsrule.overflow_rs(rs, np.array([-300, -80, -101]), p)
    assert out[0] == pytest.approx((100 / 300) ** 0.333, rel=1e-15)
    assert out[1] == pytest.approx((100 / 200) ** 0.4, rel=1e-15)
    assert out[2] == pytest.approx((100 / 101) ** 0.333, rel=1e-15)
    out0 = rsrule.overflow_rs(rs, np.array([-300, -80, -101]), params(nb_flag=0))
    assert np.all(out0 == 0.9)


def test_few_neighbours_rule():
    assert rsrule.few_nb_rs(np.array([0.2]))[0] == pytest.approx(0.3)


def test_growth_limited_by_rsfac():
    # inside the core (no radial-velocity factor): NNB 50 -> FAC 1.1, A3 55,
    # A4 1.1; A5 = 50 * 0.001 = 0.05 caps the volume change; second-order
    # cube root 1 + a - a^2 with a = 0.05/3; RS^2 = 0.04 is not in (RI2, 2 RI2)
    rs, tgt = one(0.2, 50, 50, (0.1, 0.0, 0.0), (0.0, 0.3, 0.0), 0.001, params())
    a = 0.05 / 3.0
    assert rs == pytest.approx(0.2 * (1.0 + a - a * a), rel=1e-14)
    assert tgt == pytest.approx(55.0)


def test_no_change_at_optimum():
    rs, tgt = one(0.2, 100, 100, (0.1, 0.0, 0.0), (0.0, 0.3, 0.0), 0.01, params())
    assert rs == 0.2 and tgt == pytest.approx(100.0)


def test_membership_cap_and_taper():
    # NBAVE = min(NNBOPT + 150, max(NNBMAX - 50, ZNBMIN)) = 60 for NNBMAX 110
    p = params(nnbmax=110)
    _, tgt = one(0.2, 100, 100, (0.1, 0.0, 0.0), (0.0, 0.0, 0.0), 0.01, p)
    assert tgt == pytest.approx(0.9 * 60)
    # outside the half-mass radius the target shrinks by RSCALE / r (>= 0.1)
    _, tgt = one(0.2, 100, 100, (1.6, 0.0, 0.0), (0.0, 0.0, 0.0), 0.01, params())
    assert tgt == pytest.approx(100.0 * 0.8 / 1.6)
    _, tgt = one(0.2, 100, 100, (20.0, 0.0, 0.0), (0.0, 0.0, 0.0), 0.01, params())
    assert tgt == pytest.approx(100.0 * 0.1)


def test_inertial_square_root_and_radial_factor():
    # r = 0.5: outside RC, inside 100 RH^2 -> A4 *= 1 + RIDOT DTR / RI2;
    # NNB0 above the target and NNB below it -> A4 = sqrt(A4)
    x, v, dtr = (0.5, 0.0, 0.0), (0.2, 0.0, 0.0), 0.002
    rs, _ = one(0.1, 80, 95, x, v, dtr, params())
    a3 = 80 * (1.0 + 0.1 * 20 / 80)          # 82
    a4 = math.sqrt(a3 / 80) * (1.0 + 0.5 * 0.2 * dtr / 0.25)
    a5 = min(50.0 * dtr, 0.25)
    d = min(a4 - 1.0, a5)
    a = d / 3.0
    assert rs == pytest.approx(0.1 * (1.0 + a - a * a), rel=1e-14)


def test_extra_reduction_for_inward_motion():
    # NNB 170 > NBAVE 150 and moving inward: RS *= 1 - (NNB - NBAVE) / (3 NNB)
    x, v, dtr = (0.1, 0.0, 0.0), (-0.3, 0.0, 0.0), 0.1
    rs, _ = one(0.05, 170, 170, x, v, dtr, params())
    a3 = min(170 * (1.0 + 0.1 * (100 - 170) / 170), 0.9 * 150)
    d = max(a3 / 170 - 1.0, -0.25)
    a = d / 3.0
    a1 = 1.0 + a - a * a
    assert rs == pytest.approx(0.05 * a1 * (1.0 - 20.0 / 510.0), rel=1e-14)


def test_zero_neighbours():
    p = params()
    out = rsrule.regcor_rs(np.array([0.2, 0.2, 0.01]), np.zeros(3, dtype=int), np.zeros(3),
                           np.array([[1.0, 0, 0], [1.0, 0, 0], [1.0, 0, 0]]),
                           np.array([[1.0, 0, 0], [-1.0, 0, 0], [1.0, 0, 0]]),
                           np.full(3, 0.01), p)
    assert out[0] == pytest.approx(0.15)
    assert out[1] == pytest.approx(0.22)
    assert out[2] == pytest.approx(0.08)     # max(0.75 RS, 0.1 RSCALE)
