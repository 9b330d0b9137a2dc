import numpy as np

from nbody6ppgpu_gb300 import ics


def test_plummer_henon_units():
    c = ics.plummer(2048, seed=1, nb_target=50)
    assert abs(c.m.sum() - 1.0) < 1e-12
    w = ics.potential_energy(c.m, c.x)
    k = 0.5 * np.sum(c.m * np.einsum("ij,ij->i", c.v, c.v))
    assert abs(k + w + 0.25) < 1e-9 and abs(k / -w - 0.5) < 1e-9
    assert np.abs((c.m[:, None] * c.x).sum(0)).max() < 1e-12
    cnt = ics.neighbour_counts(c.x, c.rs, np.arange(c.n))
    assert abs(cnt.mean() - 50) < 1.0
    assert np.all(c.dtr <= ics.SMAX) and np.all(c.dtr > 0)


def test_seeded_reproducible():
    a = ics.plummer(256, seed=4)
    b = ics.plummer(256, seed=4)
    assert np.array_equal(a.x, b.x) and np.array_equal(a.rs, b.rs)


def test_kroupa_range_and_slopes():
    rng = np.random.default_rng(0)
    m = ics.kroupa_masses(200000, rng)
    assert m.min() >= 0.08 and m.max() <= 100.0
    lo = m[m < 0.5]
    hi = m[(m > 1.0) & (m < 10.0)]
    # MLE of the power-law slopes on each segment
    def slope(x, a, b):
        from scipy.optimize import brentq
        ln = np.log(x).mean()
        f = lambda al: ln - (np.log(a) + 1.0 / (al - 1) -
                             (np.log(b / a) * (b / a) ** (1 - al)) / (1 - (b / a) ** (1 - al)))
        return brentq(f, 1.01, 4.0)
    assert abs(slope(lo, 0.08, 0.5) - 1.3) < 0.05
    assert abs(slope(hi, 1.0, 10.0) - 2.3) < 0.1


def test_king_model():
    k = ics.king(4096, seed=2, w0=6.0, nb_target=40)
    w = ics.potential_energy(k.m, k.x)
    kin = 0.5 * np.sum(k.m * np.einsum("ij,ij->i", k.v, k.v))
    assert abs(kin + w + 0.25) < 1e-9
    assert k.meta["binaries"] == round(0.1 * 4096)
    cnt = ics.neighbour_counts(k.x, k.rs, np.arange(0, k.n, 4))
    assert abs(cnt.mean() - 40) < 2.0


def test_active_set():
    a = ics.active_set(1000, 32, seed=1)
    assert len(np.unique(a)) == 32 and a.max() < 1000
