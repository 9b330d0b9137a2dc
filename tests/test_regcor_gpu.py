"""The regular corrector on the device (gpunb_regcor_device) against the host
restatement of REGCOR_GPU (oracle/regcor_oracle.py) on one active block of a
Plummer cluster whose lists and forces come from the library's own regular
force.  The block covers every branch: empty new lists, at most three
neighbours, empty old lists, gains and losses, old neighbours with steps below
SMIN kept inside 2 RS, c.m. bodies with KS binding energies, the tidal FIDOT
term, and the corrector suppression for large step ratios.  Lists must be
identical; FP64 state agrees to 1e-11 relative (the two sides differ only in
the order and contraction of FP64 operations)."""
import numpy as np
import pytest

from nbody6ppgpu_gb300 import ics
from oracle import regcor_oracle as R

pytestmark = pytest.mark.gpu

LMAX = 130
NNBMAX = 120


def _lists(nb, c, act, h2, lmax, nnbmax):
    """1-based LISTGP rows of the active bodies from the library, self removed"""
    r = nb.regf(h2, c.dtr[act], c.x[act], c.v[act], lmax, nnbmax)
    rows = np.zeros((act.size, lmax), dtype=np.int32)
    for k, i in enumerate(act):
        ids = r.neighbours(k)
        ids = ids[ids != i] + 1
        rows[k, 0] = len(ids)
        rows[k, 1:1 + len(ids)] = ids
    return r, rows


def test_device_corrector_matches_the_host_restatement():
    torch = pytest.importorskip("torch")
    from nbody6ppgpu_gb300.gpunb import GpuNb
    from nbody6ppgpu_gb300.regcor import regcor_device
    rng = np.random.default_rng(11)
    ntot = 3000
    n_cm = 40                                   # the last 40 bodies are KS c.m. bodies
    c = ics.plummer(ntot, seed=6, masses="kroupa", nb_target=25.0)
    act = ics.active_set(ntot, 700, seed=6)
    time = 1.0
    h2 = c.h2()
    h2_new = h2[act].copy()
    h2_new[::37] = 1e-12                        # empty new lists
    h2_new[5::23] *= 0.2                        # a few neighbours (~25 x 0.2^1.5)
    h2_old = h2.copy()
    h2_old[act] *= np.exp(rng.normal(0.0, 0.3, act.size))   # gains and losses
    with GpuNb(ntot) as nb:
        nb.send(c.m, c.x, c.v)
        r, nlist = _lists(nb, c, act, h2_new, LMAX, NNBMAX)
        _, old_rows = _lists(nb, c, np.arange(ntot), h2_old, LMAX, NNBMAX)
    assert np.all(nlist[:, 0] >= 0) and np.all(old_rows[:, 0] >= 0)
    old_rows[act[::29], :] = 0                  # empty old lists
    assert (nlist[:, 0] == 0).sum() >= 10 and ((nlist[:, 0] > 0) & (nlist[:, 0] <= 3)).sum() >= 3

    dtr = 2.0 ** -rng.integers(4, 8, ntot)
    s = {"x": c.x.copy(), "xdot": c.v.copy(), "body": c.m.copy(),
         "h": -np.abs(rng.normal(0.0, 2.0, n_cm)) - 0.05,
         "x0": c.x - c.v * dtr[:, None], "x0dot": c.v + 0.01 * rng.normal(0.0, 1.0, (ntot, 3)),
         "t0r": time - dtr, "stepr": dtr * 2.0 ** rng.integers(-1, 2, ntot),
         "step": dtr * 2.0 ** -rng.integers(0, 4, ntot), "timenw": np.zeros(ntot),
         "fi": rng.normal(0.0, 0.1, (ntot, 3)), "fidot": rng.normal(0.0, 0.1, (ntot, 3)),
         "rs": np.sqrt(h2), "list": np.zeros((ntot, LMAX), dtype=np.int32)}
    s["t0"] = time - s["step"]
    s["fr"] = np.zeros((ntot, 3))
    s["fr"][act] = r.acc * (1.0 + 1e-3 * rng.normal(0.0, 1.0, (act.size, 3)))
    s["frdot"] = np.zeros((ntot, 3))
    s["frdot"][act] = r.jrk * (1.0 + 1e-2 * rng.normal(0.0, 1.0, (act.size, 3)))
    for k in ("d0", "d0r", "d1r", "d2r", "d3r", "xn", "xndot"):
        s[k] = np.zeros((ntot, 3))
    s["list"][:, :] = old_rows
    smin = 1e-3
    s["step"][rng.choice(ntot, 300, replace=False)] = 2.0 ** -12   # below SMIN
    s["step"][act[3::53]] = 1e-7                                  # corrector suppressed
    p = dict(time=time, dtmin=1e-6, smin=smin, smax=0.125, etar=0.02, tidal4=0.3, kz14=1,
             m_flag=0, nnbmax=NNBMAX, n=ntot - n_cm, ntot=ntot, ifirst=1, lmax=LMAX,
             nnbopt=25, nb_flag=1, rscale=0.8, rc=0.3, rsfac=50.0, bodym=float(c.m.mean()),
             rdens=[0.01, -0.02, 0.005])
    iact = (act + 1).astype(np.int32)
    freg = r.acc.copy()
    fdr = r.jrk.copy()

    dev = torch.device("cuda", 0)
    T = {k: (torch.tensor(v, device=dev) if v is not None else None) for k, v in s.items()}
    counters = torch.zeros(4, dtype=torch.int32, device=dev)
    nl_d = torch.tensor(nlist, device=dev)
    regcor_device(torch.tensor(iact, device=dev), torch.tensor(freg, device=dev),
                  torch.tensor(fdr, device=dev), nl_d, p, T, counters=counters)
    torch.cuda.synchronize()
    got = {k: v.cpu().numpy() for k, v in T.items() if v is not None}

    want = {k: (v.copy() if v is not None else None) for k, v in s.items()}
    want_nl = nlist.copy()
    want_counters = R.regcor_block(iact, freg.copy(), fdr.copy(), want_nl, want, p)

    assert list(counters.cpu().numpy()) == want_counters
    assert want_counters[0] > 0 and want_counters[1] > 0 and want_counters[2] > 0
    nl_got = nl_d.cpu().numpy()
    for k in range(act.size):
        m = nl_got[k, 0]
        assert m == want_nl[k, 0] and np.array_equal(nl_got[k, 1:1 + m], want_nl[k, 1:1 + m]), k
    for i in act:
        m = want["list"][i, 0]
        assert got["list"][i, 0] == m and np.array_equal(got["list"][i, 1:1 + m],
                                                         want["list"][i, 1:1 + m]), i
    for key in ("rs", "t0r", "stepr", "step", "timenw", "fi", "fidot", "fr", "frdot", "d0", "d0r",
                "d1r", "d2r", "d3r", "xn", "xndot"):
        a, b = got[key][act], want[key][act]
        scale = np.maximum(np.abs(b), np.abs(b).max(axis=0) * 1e-6 if b.ndim == 2 else 0.0)
        err = np.abs(a - b) / np.maximum(scale, 1e-300)
        assert err.max() <= 1e-11, (key, float(err.max()))
    # bodies outside the block are untouched
    rest = np.setdiff1d(np.arange(ntot), act)
    for key in ("fi", "fr", "xn", "rs", "step", "list"):
        assert np.array_equal(got[key][rest], s[key][rest]), key
