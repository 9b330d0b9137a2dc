"""Generate the golden fixtures that pin the CPU oracle to the reference.

Runs, in this (x86_64) container, the reference's own CPU regular-force,
potential and irregular-force code (src/Main/reg.avx.cpp, pot.avx.cpp,
irr.avx.cpp, compiled from the reference sources by `make -C oracle ref` into
oracle/_ref) and the FP64 oracles on seeded inputs, and stores inputs and
both outputs in tests/golden/*.npz.  The tests then check the oracle against these files on
any host, without the reference present.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from nbody6ppgpu_gb300 import ics  # noqa: E402
from oracle import oracle as O  # noqa: E402

OUT = Path(__file__).resolve().parent


def pack_list(lst: np.ndarray):
    cnt = lst[:, 0].astype(np.int32)
    ids = np.concatenate([lst[i, 1:1 + c] for i, c in enumerate(cnt) if c > 0] or
                         [np.empty(0, np.int32)]).astype(np.int32)
    return cnt, ids


def regf_case(name, m, x, v, h2, dtr, ii, lmax, nnbmax, m_flag, ref):
    ref.send(m, x, v)
    ra, rj, rp, rl = ref.regf(h2[ii], dtr[ii], x[ii], v[ii], lmax, nnbmax, m_flag)
    oa, oj, op, ol, aa, ja = O.regf_fp64(m, x, v, h2[ii], dtr[ii], x[ii], v[ii], lmax, nnbmax,
                                         m_flag, with_abs=True)
    rc, rid = pack_list(rl)
    oc, oid = pack_list(ol)
    np.savez_compressed(OUT / f"{name}.npz", m=m, x=x, v=v, h2=h2[ii], dtr=dtr[ii], ii=ii,
                        lmax=lmax, nnbmax=nnbmax, m_flag=m_flag,
                        ref_acc=ra, ref_jrk=rj, ref_pot=rp, ref_cnt=rc, ref_ids=rid,
                        fp64_acc=oa, fp64_jrk=oj, fp64_pot=op, fp64_cnt=oc, fp64_ids=oid,
                        fp64_accabs=aa, fp64_jrkabs=ja)
    print(f"{name}: ni={len(ii)} nj={len(m)} rows identical ref/fp64:",
          int(np.sum(rc == oc)), "/", len(rc))


def main():
    # the reference's source tree: $NBODY6PP_REFERENCE, else /root/reference
    O.build(ref_dir=os.environ.get("NBODY6PP_REFERENCE", "/root/reference"))
    if not O.RefAVX.available():
        raise SystemExit("reference AVX library not available (needs x86_64 and the sources)")
    ref = O.RefAVX(1 << 16)

    # Plummer N=2048, equal masses, mean count 50, nbmax 256
    c = ics.plummer(2048, seed=1, nb_target=50.0)
    regf_case("plummer2048_equal", c.m, c.x, c.v, c.h2(), c.dtr, np.arange(c.n), 257, 256, 0, ref)

    # mass-weighted criterion (KZ(39) = 2, 3): Kroupa masses, h2 = RS^2 / BODYM
    k = ics.plummer(512, seed=5, masses="kroupa", nb_target=30.0)
    bodym = float(k.m.mean())
    regf_case("mflag_plummer512", k.m, k.x, k.v, k.h2(1, bodym), k.dtr,
              np.arange(0, k.n, 3), 257, 256, 1, ref)

    # overflow: inflate RS of every 7th body so that its count exceeds nnbmax
    o = ics.plummer(512, seed=9, nb_target=20.0)
    h2 = o.h2().copy()
    h2[::7] *= 16.0
    regf_case("overflow_plummer512", o.m, o.x, o.v, h2, o.dtr, np.arange(o.n), 41, 40, 0, ref)

    # ragged sizes: odd nj (the AVX code pads to even), ni not a multiple of 4
    r = ics.plummer(37, seed=3, nb_target=6.0)
    regf_case("ragged_n37", r.m, r.x, r.v, r.h2(), r.dtr, np.array([0, 5, 11, 36, 20]), 40, 36,
              0, ref)

    # gpupot_: all bodies, and an istart/ni sub-range
    pm, px = c.m, c.x
    np.savez_compressed(OUT / "pot_plummer2048.npz", m=pm, x=px,
                        ref_all=ref.pot(pm, px), fp64_all=O.pot_fp64(pm, px),
                        istart=100, ni=50,
                        ref_sub=ref.pot(pm, px, 100, 50), fp64_sub=O.pot_fp64(pm, px, 100, 50))
    ref.close()
    print("pot: written")

    # irregular force (irr.avx.cpp): neighbour lists of the regular path with
    # the particle itself removed, predictor state from the full force
    irr_case("irr_plummer2048", c, seed=21, ti=0.25, empty=())
    irr_case("irr_ragged_n37", r, seed=22, ti=1.5, empty=(0, 7, 30))


def irr_case(name, c, seed, ti, empty):
    n = c.n
    rng = np.random.default_rng(seed)
    lmax = 257
    _, _, _, lst = O.regf_fp64(c.m, c.x, c.v, c.h2(), c.dtr, c.x, c.v, lmax, lmax - 1)
    lists = np.zeros((n, lmax), dtype=np.int32)
    for i in range(n):
        ids = lst[i, 1:1 + max(lst[i, 0], 0)]
        ids = ids[ids != i]
        if i in empty:
            ids = ids[:0]
        lists[i, 0] = len(ids)
        lists[i, 1:1 + len(ids)] = ids
    acc, jrk, _, _ = O.regf_fp64(c.m, c.x, c.v, np.full(n, 1e-30), np.zeros(n), c.x, c.v,
                                 2, 1)
    f = 0.5 * acc
    fdot = jrk / 6.0
    t0 = ti - rng.uniform(0.0, 0.01, n)
    active = rng.permutation(n)[: max(1, (2 * n) // 3)]
    refi = O.RefIrrAVX(n, lmax)
    refi.set_jp(c.x, c.v, f, fdot, c.m, t0)
    refi.set_lists(lists)
    ra, rj, rn = refi.firr(ti, active)
    refi.close()
    oa, oj, on = O.irr_fp64(c.x, c.v, f, fdot, c.m, t0, lists, ti, active)
    np.savez_compressed(OUT / f"{name}.npz", x0=c.x, v0=c.v, f=f, fdot=fdot, m=c.m, t0=t0,
                        lists=lists, ti=ti, active=active, ref_acc=ra, ref_jrk=rj, ref_nnbid=rn,
                        fp64_acc=oa, fp64_jrk=oj, fp64_nnbid=on)
    print(f"{name}: ni={len(active)} n={n} nearest-neighbour ids identical ref/fp64:",
          int(np.sum(rn == on)), "/", len(rn))


if __name__ == "__main__":
    main()
