"""The band check's count estimate for a predicted radius (rsharness.motion_count)
against a direct count: the members of each row moved on their relative
velocity by one regular step and tested as the kernel tests them then."""
import numpy as np
import pytest

from nbody6ppgpu_gb300.rsharness import motion_count


def _direct(x, v, i, members, dtr, rs_new, rs_old):
    n = 0
    for j in members:
        if j == i:
            continue
        dx = x[j] - x[i] + dtr * (v[j] - v[i])
        d2 = dx + dtr * (v[j] - v[i])
        if min(dx @ dx, d2 @ d2) < rs_new * rs_new:
            n += 1
    cnt = sum(1 for j in members if j != i)
    return n + cnt * max((rs_new / rs_old) ** 3 - 1.0, 0.0)


def test_motion_count_equals_the_direct_count():
    rng = np.random.default_rng(4)
    n, lmax = 3000, 60
    x = rng.normal(size=(n, 3))
    v = rng.normal(size=(n, 3))
    dtr = 2.0 ** -rng.integers(3, 8, n)
    idx = rng.choice(n, 1500, replace=False)          # more than one chunk of 1024
    rows = np.zeros((idx.size, lmax), dtype=np.int32)
    members = []
    for k, i in enumerate(idx):
        m = int(rng.integers(0, lmax - 1))
        ids = np.sort(rng.choice(n, m, replace=False))
        if k % 3 == 0 and i not in ids and m > 0:      # self in the row, as the library reports
            ids[0] = i
            ids = np.sort(ids)
        rows[k, 0] = len(ids)
        rows[k, 1:1 + len(ids)] = ids
        members.append(ids)
    rs_old = rng.uniform(0.5, 1.5, idx.size)
    rs_new = rs_old * np.exp(rng.normal(0.0, 0.4, idx.size))
    got = motion_count(x, v, idx, rows, dtr, rs_new, rs_old)
    want = [_direct(x, v, i, members[k], dtr[i], rs_new[k], rs_old[k]) for k, i in enumerate(idx)]
    np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-12)


def test_motion_count_follows_a_contraction():
    """Neighbours falling in: the static estimate (count at today's density)
    rejects a radius halved for the next step; the motion estimate keeps the
    count."""
    rng = np.random.default_rng(7)
    m = 100
    d = rng.normal(size=(m, 3))
    d *= (rng.uniform(0.0, 1.0, m) ** (1 / 3) / np.linalg.norm(d, axis=1))[:, None]
    x = np.vstack([np.zeros(3), d])                  # particle 0 and its 100 members in r < 1
    dtr = np.full(m + 1, 0.25)
    v = np.vstack([np.zeros(3), -d])                 # each member at 0.5 r at t + dtr, 0.25 r at t + 2 dtr
    rows = np.zeros((1, m + 2), dtype=np.int32)
    rows[0, 0] = m + 1
    rows[0, 1:m + 2] = np.arange(m + 1)
    rs_old, rs_new = np.array([1.0]), np.array([0.5])
    got = motion_count(x, v, np.array([0]), rows, dtr, rs_new, rs_old)[0]
    static = m * (rs_new[0] / rs_old[0]) ** 3
    assert got == m and static == m / 8


@pytest.mark.gpu
def test_motion_count_on_the_device_equals_the_host_count():
    torch = pytest.importorskip("torch")
    from nbody6ppgpu_gb300.rsharness import motion_count_device
    rng = np.random.default_rng(5)
    n, lmax = 5000, 80
    x = rng.normal(size=(n, 3))
    v = rng.normal(size=(n, 3))
    dtr = 2.0 ** -rng.integers(3, 8, n)
    idx = rng.choice(n, 3000, replace=False)
    rows = np.zeros((idx.size, lmax), dtype=np.int32)
    for k, i in enumerate(idx):
        ids = np.sort(np.append(rng.choice(n, int(rng.integers(0, lmax - 2)), replace=False), i))
        ids = np.unique(ids)
        rows[k, 0] = len(ids)
        rows[k, 1:1 + len(ids)] = ids
    rs_old = rng.uniform(0.5, 1.5, idx.size)
    rs_new = rs_old * np.exp(rng.normal(0.0, 0.4, idx.size))
    dev = torch.device("cuda", 0)
    got = motion_count_device(torch.tensor(x, device=dev), torch.tensor(v, device=dev), idx, rows,
                              dtr, rs_new, rs_old, chunk=1000)
    want = motion_count(x, v, idx, rows, dtr, rs_new, rs_old)
    np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-12)
