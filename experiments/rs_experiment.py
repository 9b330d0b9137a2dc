"""Neighbour-radius experiment: the plain RS rule against the learned
predictor with the plain rule as fallback.

    python -m experiments.rs_experiment --n 16384 --ticks 64 --model king

1. Harvest (features, label) pairs by running the regular-step harness with the
   plain rule on two seeded clusters (the pairs the integrator itself
   generates); train the MLP on the GPU kernels (Adam, FP32 master, BF16
   weights).
2. Optionally (rounds = 2) harvest again on the same seeds with the
   predictor in the loop, and refit on all pairs.
3. Run a third seeded cluster twice from the same state -- plain rule, and
   predictor + fallback -- and compare list-overflow recomputes after the
   first block (the first block is identical for both), the membership
   against the rule's own target, and the regular-call time.
Prints one JSON line.
"""
from __future__ import annotations

import argparse
import dataclasses
import json
import math
import time

import numpy as np

from nbody6ppgpu_gb300 import ics
from nbody6ppgpu_gb300.rsharness import GUARDS, PRED_BAND, Harness
from nbody6ppgpu_gb300.rsmlp import RSMLP


def make(model: str, n: int, seed: int, target: float, q: float = 0.5):
    """Seeded cluster; q < 1/2 scales the virial velocities to virial ratio q
    (a cold start that collapses)."""
    if model == "king":
        c = ics.king(n, seed=seed, nb_target=target)
    else:
        c = ics.plummer(n, seed=seed, masses="kroupa", nb_target=target, exact_energy_max=0)
    if q != 0.5:
        c = dataclasses.replace(c, v=c.v * math.sqrt(q / 0.5))
    return c


def band_diagnostics(diag, band):
    """How the band check's count estimates compare with the count the
    predicted radius actually had at the next regular step, k exp(3 (y - L))
    with L the label (log R_k / RS) and k the target: per group of rows
    (accepted, rejected below the band, above it), the medians of the true,
    motion and static counts over the target and the fraction whose true count
    lay inside the band."""
    if not diag:
        return {}
    a = np.array([(l, y, pm, ps, t, float(ok)) for l, y, pm, ps, t, ok in diag])
    lab, y, pm, ps, tgt, ok = a.T
    true = np.exp(3.0 * (y - lab))          # true count / target
    lo, hi = band
    groups = {"accepted": ok == 1, "rejected_low": (ok == 0) & (pm < lo * tgt),
              "rejected_high": (ok == 0) & (pm > hi * tgt)}
    out = {}
    for name, m in groups.items():
        if m.sum() == 0:
            out[name] = {"rows": 0}
            continue
        out[name] = {"rows": int(m.sum()),
                     "true_over_target_median": float(np.median(true[m])),
                     "true_in_band": float(np.mean((true[m] >= lo) & (true[m] <= hi))),
                     "motion_over_target_median": float(np.median(pm[m] / tgt[m])),
                     "static_over_target_median": float(np.median(ps[m] / tgt[m])),
                     "motion_over_true_median": float(np.median(pm[m] / (true[m] * tgt[m])))}
    return out


def run(model="king", n=16384, ticks=64, nnbopt=100, nnbmax=200, levels=6, epochs=25,
        train_seeds=(11, 12), eval_seed=13, q=0.5, rounds=1, band=PRED_BAND, guard="max",
        other_guards=(), diag=False, diag_dump=None):
    """rounds > 1: after the first fit, harvest again on the training seeds
    with the predictor in the loop (the states it leads to), add those pairs
    and refit -- the usual remedy for the shift between the plain rule's
    states and the predictor's.  The predictor is evaluated with the band
    check `guard` ("predictor") and with each of other_guards
    ("predictor_<guard>")."""
    t_harvest = t_train = 0.0
    X, Y = [], []
    mlp = None
    for rnd in range(rounds):
        t0 = time.perf_counter()
        for s in train_seeds:
            h = Harness(make(model, n, s, nnbopt, q), nnbopt, nnbmax, harvest=True, levels=levels,
                        band=band, guard=guard)
            h.run(ticks, predictor=mlp)
            x, y = h.dataset()
            h.close()
            X.append(x)
            Y.append(y)
        t_harvest += time.perf_counter() - t0
        t0 = time.perf_counter()
        mlp = RSMLP(seed=3)
        losses = mlp.train(np.concatenate(X), np.concatenate(Y), epochs=epochs)
        t_train += time.perf_counter() - t0
    X = np.concatenate(X)
    Y = np.concatenate(Y)
    c = make(model, n, eval_seed, nnbopt, q)
    out = {"model": model, "q": q, "n": n, "ticks": ticks, "rounds": rounds, "band": band,
           "guard": guard, "nnbopt": nnbopt,
           "nnbmax": nnbmax,
           "levels": levels, "train_pairs": int(len(X)), "label_variance": float(Y.var()),
           "train_mse_first_epoch": losses[0], "train_mse_last_epoch": losses[-1],
           "harvest_s": t_harvest, "train_s": t_train}
    legs = [("plain", None, guard), ("predictor", mlp, guard)]
    legs += [(f"predictor_{g}", mlp, g) for g in other_guards if g != guard]
    for name, pred, g in legs:
        h = Harness(c, nnbopt, nnbmax, levels=levels, band=band, guard=g,
                    harvest=diag and pred is not None)
        s = h.run(ticks, predictor=pred).as_dict()
        if diag and pred is not None:
            out[name + "_band_diagnostics"] = band_diagnostics(h.diag, band)
            if diag_dump:
                rows = np.array([(l, y, pm, ps, t, float(ok)) for l, y, pm, ps, t, ok in h.diag],
                                dtype=np.float32)
                keep = np.linspace(0, len(rows) - 1, min(len(rows), 300_000)).astype(int)
                np.save(f"{diag_dump}_{name}.npy", rows[keep])
        h.close()
        out[name] = {k: s[k] for k in ("first_call_overflows", "overflow_events",
                                       "overflow_after_predictor", "overflow_after_fallback",
                                       "active", "recompute_rate", "mean_count", "count_p99",
                                       "regf_seconds", "predict_seconds", "predictor_used",
                                       "predictor_fallback", "fallback_low", "fallback_high")}
    p = out["plain"]["overflow_events"]
    for name, _, _ in legs[1:]:
        q_ = out[name]["overflow_events"]
        key = "overflow_recompute_ratio_plain_over_" + name
        out[key] = (p / q_) if q_ else (None if p == 0 else float("inf"))
    return out


def pooled_king(ticks_harvest=48, ticks_eval=48, n_king=1 << 20, n_plummer=65536, nnbopt=100,
            nnbmax=200, levels=6, epochs=25, q=0.1, band=PRED_BAND, eval_seed=41,
            max_pairs=2_000_000, guard="max", harvest_every=1):
    """The learned-radius configuration: training pairs harvested with the
    plain rule on a Plummer/Kroupa cluster of n_plummer bodies (the bench's
    cluster type) and on a King W0 = 6 model of n_king bodies, pooled (at most
    max_pairs, drawn evenly), the MLP trained on the GPU kernels, then a
    further King model of n_king bodies run from the same state with the plain
    rule and with the predictor (plain-rule fallback outside the band):
    overflow recomputes after the first block, membership, regular-call time.
    q < 1/2 starts the clusters cold, so that they contract and lists
    overflow."""
    t0 = time.perf_counter()
    X, Y, sources = [], [], {}
    for name, model, n, seed in (("plummer", "plummer", n_plummer, 21),
                                 ("king", "king", n_king, 22)):
        h = Harness(make(model, n, seed, nnbopt, q), nnbopt, nnbmax, harvest=True, levels=levels,
                    band=band, harvest_every=harvest_every if n > n_plummer else 1)
        h.run(ticks_harvest)
        x, y = h.dataset()
        h.close()
        X.append(x)
        Y.append(y)
        sources[name] = {"n": n, "seed": seed, "pairs": int(len(x))}
    X = np.concatenate(X)
    Y = np.concatenate(Y)
    if len(X) > max_pairs:
        keep = np.linspace(0, len(X) - 1, max_pairs).astype(int)
        X, Y = X[keep], Y[keep]
    t_harvest = time.perf_counter() - t0
    t0 = time.perf_counter()
    mlp = RSMLP(seed=3)
    losses = mlp.train(X, Y, epochs=epochs)
    t_train = time.perf_counter() - t0
    c = make("king", n_king, eval_seed, nnbopt, q)
    out = {"config": "King W0=6 evaluation model, pairs pooled from Plummer/Kroupa and King runs",
           "n_eval": n_king, "q": q, "ticks_harvest": ticks_harvest, "ticks_eval": ticks_eval,
           "band": band, "guard": guard, "nnbopt": nnbopt, "nnbmax": nnbmax, "levels": levels,
           "harvest_every_king": harvest_every, "harvest_sources": sources, "train_pairs": int(len(X)),
           "label_variance": float(Y.var()), "train_mse_first_epoch": losses[0],
           "train_mse_last_epoch": losses[-1], "harvest_s": t_harvest, "train_s": t_train}
    for name, pred in (("plain", None), ("predictor", mlp)):
        t0 = time.perf_counter()
        h = Harness(c, nnbopt, nnbmax, levels=levels, band=band, guard=guard)
        s = h.run(ticks_eval, predictor=pred).as_dict()
        h.close()
        out[name] = {k: s[k] for k in ("first_call_overflows", "overflow_events",
                                       "overflow_after_predictor", "overflow_after_fallback",
                                       "active", "recompute_rate", "mean_count", "count_p99",
                                       "regf_seconds", "predict_seconds", "predictor_used",
                                       "predictor_fallback", "fallback_low", "fallback_high")}
        out[name]["wall_s"] = time.perf_counter() - t0
    p_, q_ = out["plain"]["overflow_events"], out["predictor"]["overflow_events"]
    out["overflow_recompute_ratio_plain_over_predictor"] = (p_ / q_) if q_ else (
        None if p_ == 0 else float("inf"))
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--pooled-king", action="store_true",
                    help="pairs pooled from a Plummer run of 65536 bodies and a King run of "
                         "--n bodies, evaluation on a further King model of --n bodies")
    ap.add_argument("--ticks-harvest", type=int, default=48)
    ap.add_argument("--harvest-every", type=int, default=1,
                    help="--pooled-king: label only the King bodies i %% k == 0")
    ap.add_argument("--eval-seed", type=int, default=41,
                    help="--pooled-king: seed of the King model the policies are evaluated on")
    ap.add_argument("--model", default="king", choices=["king", "plummer"])
    ap.add_argument("--n", type=int, default=16384)
    ap.add_argument("--ticks", type=int, default=64)
    ap.add_argument("--nnbopt", type=int, default=100)
    ap.add_argument("--nnbmax", type=int, default=200)
    ap.add_argument("--levels", type=int, default=6)
    ap.add_argument("--q", type=float, default=0.5, help="virial ratio of the start")
    ap.add_argument("--epochs", type=int, default=25)
    ap.add_argument("--rounds", type=int, default=1,
                    help="harvest rounds (later ones with the predictor in the loop)")
    ap.add_argument("--band", type=float, nargs=2, default=PRED_BAND,
                    help="accept a prediction whose count lies in [lo, hi] x target")
    ap.add_argument("--guard", default="max", choices=GUARDS,
                    help="how the count of a predicted radius is estimated")
    ap.add_argument("--other-guards", nargs="*", default=[], choices=GUARDS,
                    help="also evaluate the predictor with these band checks")
    ap.add_argument("--diag", action="store_true",
                    help="label the predictor legs too and compare the count estimates "
                         "with the counts the predicted radii had")
    ap.add_argument("--diag-dump", default=None,
                    help="with --diag: save a sample of the per-row diagnostics to "
                         "<prefix>_<leg>.npy (label, y, motion, static, target, accepted)")
    a = ap.parse_args()
    if a.pooled_king:
        print(json.dumps(pooled_king(a.ticks_harvest, a.ticks, n_king=a.n, nnbopt=a.nnbopt,
                                 nnbmax=a.nnbmax, levels=a.levels, epochs=a.epochs, q=a.q,
                                 band=tuple(a.band), guard=a.guard,
                                 harvest_every=a.harvest_every, eval_seed=a.eval_seed)),
              flush=True)
        return
    print(json.dumps(run(a.model, a.n, a.ticks, a.nnbopt, a.nnbmax, a.levels, epochs=a.epochs,
                         q=a.q, rounds=a.rounds, band=tuple(a.band), guard=a.guard,
                         other_guards=tuple(a.other_guards), diag=a.diag,
                         diag_dump=a.diag_dump)), flush=True)


if __name__ == "__main__":
    main()
