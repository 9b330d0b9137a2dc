"""The RS update on the device (gpunb_rs_update_device): the plain rule
against rsrule.regcor_rs (itself checked against hand-worked cases of the
Fortran), and the fused MLP proposal against the host path of the harness
(features -> forward kernel -> band check -> fallback)."""
import numpy as np
import pytest

from nbody6ppgpu_gb300 import rsrule
from nbody6ppgpu_gb300.rsharness import PRED_BAND

pytestmark = pytest.mark.gpu


def _inputs(n, seed):
    rng = np.random.default_rng(seed)
    x = rng.normal(0, 0.8, (n, 3)) * rng.choice([0.1, 1.0, 5.0], (n, 1))
    v = rng.normal(0, 0.5, (n, 3))
    nnb = rng.integers(0, 260, n)
    nnb[:20] = 0                       # zero-neighbour branch
    nnb[20:40] = 1                     # few-member rule
    nnb0 = np.clip(nnb + rng.integers(-30, 30, n), 0, None)
    rs = np.exp(rng.uniform(np.log(0.02), np.log(0.5), n))
    r = np.linalg.norm(x, axis=1)
    rs[40:80] = r[40:80] * rng.uniform(1.05, 1.35, 40)   # RS^2 in (r^2, 2 r^2): shell rule
    dtr = rng.choice([0.0039, 0.0156, 0.0625, 0.125], n)
    acc = rng.normal(0, 1, (n, 3))
    jrk = rng.normal(0, 3, (n, 3))
    m_scaled = rng.uniform(0.1, 20, n)
    return x, v, m_scaled, rs, nnb, nnb0, acc, jrk, dtr


@pytest.mark.parametrize("nb_flag", [1, 0])
def test_plain_rule_matches_host(nb_flag):
    pytest.importorskip("torch")
    from nbody6ppgpu_gb300.rsmlp import rs_update_device
    p = rsrule.RSParams(nnbopt=100, nnbmax=200, nb_flag=nb_flag, bodym=1e-4)
    x, v, m, rs, nnb, nnb0, acc, jrk, dtr = _inputs(5000, 1 + nb_flag)
    host, tgt = rsrule.regcor_rs(rs, nnb, nnb0, x, v, dtr, p, return_target=True)
    got, gtgt, used = rs_update_device(p, x, v, m, rs, nnb, nnb0, acc, jrk, dtr,
                                       few_nb_rule=False)
    np.testing.assert_allclose(got, host, rtol=1e-13)
    np.testing.assert_allclose(gtgt, tgt, rtol=1e-13)
    assert not used.any()
    few, _, _ = rs_update_device(p, x, v, m, rs, nnb, nnb0, acc, jrk, dtr, few_nb_rule=True)
    want = np.where(nnb < 2, rsrule.few_nb_rs(rs), host)
    np.testing.assert_allclose(few, want, rtol=1e-13)


def test_fused_predictor_matches_host_path():
    pytest.importorskip("torch")
    from nbody6ppgpu_gb300.rsmlp import RSMLP, features, rs_update_device
    p = rsrule.RSParams(nnbopt=100, nnbmax=200, bodym=1e-4)
    x, v, m, rs, nnb, nnb0, acc, jrk, dtr = _inputs(4000, 7)
    F = features(x, v, m, rs, nnb, acc, jrk, dtr, p.nnbopt)
    mlp = RSMLP(seed=5)
    rng = np.random.default_rng(3)
    T = 0.2 * np.tanh(F[:, 1] - F[:, 1].mean()) + 0.05 * rng.normal(size=len(F))
    mlp.train(F, T, epochs=3)                       # any fitted network will do
    plain, tgt = rsrule.regcor_rs(rs, nnb, nnb0, x, v, dtr, p, return_target=True)
    plain = np.where(nnb < 2, rsrule.few_nb_rs(rs), plain)
    y = mlp.predict(F)
    pc = (np.maximum(nnb, 0) + 1.0) * np.exp(3.0 * y.astype(np.float64)) - 1.0
    lo, hi = PRED_BAND
    ok = (pc >= lo * tgt) & (pc <= hi * tgt) & np.isfinite(y)
    want = np.where(ok, rs * np.exp(y.astype(np.float64)), plain)
    got, gtgt, used = rs_update_device(p, x, v, m, rs, nnb, nnb0, acc, jrk, dtr, mlp=mlp,
                                       band=PRED_BAND)
    # both sides run the same tensor-core inference; features computed on the
    # host and on the device can differ in the last bit, which can flip the
    # BF16 rounding of an input (a change of y below 1e-2)
    edge = (np.abs(pc - lo * tgt) < 0.03 * tgt) | (np.abs(pc - hi * tgt) < 0.03 * tgt)
    assert np.array_equal(used.astype(bool)[~edge], ok[~edge])
    assert ok.sum() > 100 and (~ok).sum() > 100       # both branches exercised
    sel = ~edge
    np.testing.assert_allclose(got[sel], want[sel], rtol=1e-2)
    assert np.mean(np.isclose(got[sel], want[sel], rtol=1e-6, atol=0)) > 0.99


def test_fused_band_check_at_the_next_step_matches_host_path():
    """With the block's neighbour rows the device takes the larger of the
    count at the current density and the estimate at the next regular step
    (rsharness.motion_count), as the harness's default band check does, and
    makes the same choices away from the band edges."""
    pytest.importorskip("torch")
    cKDTree = pytest.importorskip("scipy.spatial").cKDTree
    from nbody6ppgpu_gb300.rsharness import motion_count
    from nbody6ppgpu_gb300.rsmlp import RSMLP, features, rs_update_device
    p = rsrule.RSParams(nnbopt=100, nnbmax=200, bodym=1e-4)
    x, v, m, rs, nnb, nnb0, acc, jrk, dtr = _inputs(4000, 7)
    n = len(x)
    # rows: each particle's nnb nearest bodies and itself (LISTGP layout and CSR)
    tree = cKDTree(x)
    rows = np.zeros((n, 262), dtype=np.int32)
    off = np.zeros(n + 1, dtype=np.int32)
    for i in range(n):
        _, ids = tree.query(x[i], k=int(nnb[i]) + 1)
        ids = np.sort(np.atleast_1d(ids))
        rows[i, 0] = len(ids)
        rows[i, 1:1 + len(ids)] = ids
        off[i + 1] = off[i] + len(ids)
    flat = np.concatenate([rows[i, 1:1 + rows[i, 0]] for i in range(n)]).astype(np.int32)
    F = features(x, v, m, rs, nnb, acc, jrk, dtr, p.nnbopt)
    mlp = RSMLP(seed=5)
    rng = np.random.default_rng(3)
    T = 0.3 * np.tanh(F[:, 1] - F[:, 1].mean()) + 0.1 * rng.normal(size=n)
    mlp.train(F, T, epochs=3)
    plain, tgt = rsrule.regcor_rs(rs, nnb, nnb0, x, v, dtr, p, return_target=True)
    plain = np.where(nnb < 2, rsrule.few_nb_rs(rs), plain)
    y = mlp.predict(F).astype(np.float64)
    pc = np.maximum(motion_count(x, v, np.arange(n), rows, dtr, rs * np.exp(y), rs),
                    (np.maximum(nnb, 0) + 1.0) * np.exp(3.0 * y) - 1.0)
    lo, hi = PRED_BAND
    ok = (pc >= lo * tgt) & (pc <= hi * tgt) & np.isfinite(y)
    want = np.where(ok, rs * np.exp(y), plain)
    got, gtgt, used = rs_update_device(p, x, v, m, rs, nnb, nnb0, acc, jrk, dtr, mlp=mlp,
                                       band=PRED_BAND, rows=(off, flat, x, v))
    # a key within rounding of R'^2 can move the count by one, a BF16 input
    # rounded the other way moves y by less than 1e-2
    edge = (np.abs(pc - lo * tgt) <= 1.5 + 0.1 * pc) | (np.abs(pc - hi * tgt) <= 1.5 + 0.1 * pc)
    assert np.array_equal(used.astype(bool)[~edge], ok[~edge])
    assert ok[~edge].sum() > 100 and (~ok[~edge]).sum() > 100
    np.testing.assert_allclose(got[~edge], want[~edge], rtol=1e-2)
    assert np.mean(np.isclose(got[~edge], want[~edge], rtol=1e-6, atol=0)) > 0.99
