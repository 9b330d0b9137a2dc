"""The learned neighbour-radius predictor on the GPU: the hand-written MLP
kernels (forward, backward, Adam) against the FP64 oracle, training on the
GPU, the invariance of the total force to the radius the predictor picks,
and what the trained predictor gains over the plain rule."""
import numpy as np
import pytest

from oracle import mlp_oracle

pytestmark = pytest.mark.gpu

# inference: BF16 inputs and activations (2^-9 relative each), FP32
# accumulation, hardware tanh; |y_gpu - y_fp64| / (1 + |y|) at most FWD_TOL,
# its root mean square at most FWD_RMS
FWD_TOL = 3e-2
FWD_RMS = 3e-3
GRAD_TOL = 1e-4     # ||g_gpu - g_fp64|| / ||g_fp64||: FP32 accumulation over the batch


@pytest.fixture(scope="module")
def mlp():
    pytest.importorskip("torch")
    from nbody6ppgpu_gb300.rsmlp import RSMLP
    return RSMLP(seed=7)


def _rand_inputs(B, seed):
    rng = np.random.default_rng(seed)
    return rng.normal(size=(B, 8)).astype(np.float32), \
        (0.3 * rng.normal(size=B)).astype(np.float32), rng.random(B).astype(np.float32)


def test_forward_matches_oracle(mlp):
    X, _, _ = _rand_inputs(1000, 1)
    y = mlp.forward_normalised(X)
    wf, wq = mlp.params()
    ref, _ = mlp_oracle.forward(wq, wf, X)
    e = np.abs(y - ref) / (1.0 + np.abs(ref))
    assert e.max() < FWD_TOL and np.sqrt(np.mean(e * e)) < FWD_RMS, (e.max(), np.sqrt(np.mean(e * e)))


@pytest.mark.parametrize("B,weighted", [(1000, False), (1000, True), (384, False), (1, True)])
def test_gradient_matches_oracle(mlp, B, weighted):
    X, T, W = _rand_inputs(B, 2 + B)
    g, loss = mlp.gradient(X, T, W if weighted else None)
    wf, wq = mlp.params()
    gref, lref = mlp_oracle.gradient(wq, wf, X, T, W if weighted else None)
    assert np.linalg.norm(g - gref) / np.linalg.norm(gref) < GRAD_TOL
    assert loss == pytest.approx(lref, rel=1e-5)


def test_gradient_is_deterministic(mlp):
    X, T, _ = _rand_inputs(4096, 3)
    g1, l1 = mlp.gradient(X, T)
    g2, l2 = mlp.gradient(X, T)
    assert np.array_equal(g1, g2) and l1 == l2


def test_adam_step_matches_formula():
    torch = pytest.importorskip("torch")
    from nbody6ppgpu_gb300.rsmlp import RSMLP
    m = RSMLP(seed=9)
    X, T, _ = _rand_inputs(512, 4)
    w0 = m.master.cpu().numpy().astype(np.float64)
    g, _ = m.gradient(X, T)
    lr, b1, b2, eps = 1e-3, 0.9, 0.999, 1e-8
    rc = m.lib.gpunb_rsmlp_adam(m.master.data_ptr(), m.m1.data_ptr(), m.m2.data_ptr(),
                                m.grad.data_ptr(), lr, b1, b2, eps, 1, m.wq.data_ptr(),
                                m.stream.cuda_stream)
    assert rc == 0
    m.stream.synchronize()
    g64 = g.astype(np.float64)
    mhat = (1 - b1) * g64 / (1 - b1)
    vhat = (1 - b2) * g64 * g64 / (1 - b2)
    ref = w0 - lr * mhat / (np.sqrt(vhat) + eps)
    wf, wq = m.params()
    assert np.max(np.abs(wf - ref)) < 1e-6
    # the BF16 copy is the rounded master
    assert np.array_equal(wq, torch.tensor(wf).to(torch.bfloat16).float().numpy())


def test_training_fits_a_smooth_map():
    pytest.importorskip("torch")
    from nbody6ppgpu_gb300.rsmlp import RSMLP
    rng = np.random.default_rng(11)
    X = rng.normal(size=(40000, 8))
    T = 0.3 * np.tanh(X[:, 0]) + 0.2 * X[:, 1] * X[:, 2] / (1.0 + X[:, 3] ** 2) - 0.1 * X[:, 7]
    m = RSMLP(seed=1)
    losses = m.train(X, T, epochs=12)
    assert losses[-1] < 0.15 * T.var()
    assert losses[-1] < 0.5 * losses[0]
    # the kernels train the same network the oracle evaluates (inference in
    # BF16: the tolerance of test_forward_matches_oracle)
    wf, wq = m.params()
    ref, _ = mlp_oracle.forward(wq, wf, m.normalise(X[:500]))
    e = np.abs(m.predict(X[:500]) - ref) / (1.0 + np.abs(ref))
    assert e.max() < FWD_TOL and np.sqrt(np.mean(e * e)) < FWD_RMS


def _irregular(c, idx, lst):
    """FP64 sums over the listed neighbours (self excluded): acc, jerk, pot
    -- the part of the force the host computes from the list."""
    acc = np.zeros((idx.size, 3)); jrk = np.zeros((idx.size, 3)); pot = np.zeros(idx.size)
    for q, i in enumerate(idx):
        js = lst[q, 1:1 + lst[q, 0]]
        js = js[js != i]
        dx = c.x[js] - c.x[i]
        dv = c.v[js] - c.v[i]
        r2 = np.einsum("ij,ij->i", dx, dx)
        rinv = 1.0 / np.sqrt(r2)
        mr3 = c.m[js] * rinv ** 3
        rv = np.einsum("ij,ij->i", dx, dv) / r2
        acc[q] = (mr3[:, None] * dx).sum(0)
        jrk[q] = (mr3[:, None] * (dv - 3.0 * rv[:, None] * dx)).sum(0)
        pot[q] = (c.m[js] * rinv).sum()
    return acc, jrk, pot


def test_total_force_is_independent_of_the_radius():
    """Whatever RS the predictor proposes, regular + irregular force (and jerk,
    potential) is the same: the radius only moves bodies between the two
    sums, so the predictor cannot change the dynamics."""
    from nbody6ppgpu_gb300 import ics
    from nbody6ppgpu_gb300.gpunb import GpuNb
    c = ics.plummer(4096, seed=21, masses="kroupa", nb_target=60.0)
    idx = np.arange(0, c.n, 4)
    rng = np.random.default_rng(0)
    nb = GpuNb(c.n)
    try:
        nb.send(c.m, c.x, c.v)
        tot = []
        for scale in (np.ones(idx.size), np.exp(rng.uniform(-0.3, 0.3, idx.size))):
            rs = c.rs[idx] * scale
            r = nb.regf(rs ** 2, c.dtr[idx], c.x[idx], c.v[idx], 1025, 1024)
            assert np.all(r.list[:, 0] >= 0)
            a, j, p = _irregular(c, idx, r.list)
            tot.append((r.acc + a, r.jrk + j, r.pot + p))
    finally:
        nb.close()
    for k, tol in ((0, 1e-6), (1, 2e-5), (2, 1e-6)):
        d = np.abs(tot[0][k] - tot[1][k]).reshape(idx.size, -1)
        s = np.abs(tot[0][k]).reshape(idx.size, -1)
        assert np.max(np.linalg.norm(d, axis=1) / np.linalg.norm(s, axis=1)) < tol, k


def test_predictor_cuts_overflow_recomputes():
    """A cold (virial ratio 0.1) Plummer cluster of 65536 bodies collapses, so
    local densities rise faster than the plain rule's 25%-per-step volume
    limit follows and lists overflow.  The predictor, trained on pairs
    harvested from two other seeds with the plain rule, is run on a third seed
    from the same state with the plain rule as fallback outside 0.5-1.5 x the
    target: it must need at least 5x fewer overflow recomputes at the same
    mean membership."""
    pytest.importorskip("scipy")
    from experiments.rs_experiment import run
    r = run(model="plummer", n=65536, ticks=256, nnbopt=100, nnbmax=200, levels=6, epochs=25,
            rounds=1, q=0.1, band=(0.5, 1.5))
    plain, pred = r["plain"], r["predictor"]
    assert plain["overflow_events"] >= 10000          # the regime does overflow
    assert pred["overflow_events"] * 5 <= plain["overflow_events"]   # measured 6.1x
    assert abs(pred["mean_count"] / plain["mean_count"] - 1.0) < 0.1
    assert pred["count_p99"] <= plain["count_p99"]
    assert pred["predictor_used"] > 0.9 * pred["active"]


def test_device_labels_equal_the_kdtree_labels():
    """The device labeller (the library's own rows at an enlarged radius, keys
    sorted per row on the GPU) gives the KD-tree labels of the host exactly,
    over targets from 5 to 200 members and radius hints off by up to 2x."""
    from nbody6ppgpu_gb300 import ics
    from nbody6ppgpu_gb300.gpunb import GpuNb
    from nbody6ppgpu_gb300.rsharness import label_log_radius, label_log_radius_gpu
    pytest.importorskip("scipy")
    c = ics.plummer(20000, seed=31, masses="kroupa", nb_target=60.0)
    idx = ics.active_set(c.n, 3000, seed=31)
    rng = np.random.default_rng(31)
    ks = rng.integers(5, 200, idx.size)
    hint = c.rs[idx] * np.cbrt((ks + 2.0) / 61.0) * np.exp(rng.uniform(-0.7, 0.7, idx.size))
    with GpuNb(c.n) as nb:
        nb.send(c.m, c.x, c.v)
        g = label_log_radius_gpu(nb, c.x, c.v, c.dtr, idx, ks, hint)
    h = label_log_radius(c.x, c.v, c.dtr, idx, ks)
    assert np.max(np.abs(g - h)) < 1e-12
