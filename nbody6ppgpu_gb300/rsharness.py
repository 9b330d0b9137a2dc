"""Regular-step harness for the neighbour-radius experiments.

Drives libgpunb.so the way NBODY6++'s regular section does (intgrt.F:912-944,
util_gpu.F:33-116): every tick the whole j-set is sent, the particles whose
regular step is due form the active block, `gpunb_regf_` returns their
regular force and neighbour lists, overflowed rows are repaired by the
overflow rule and the chunk is computed again (one recompute per overflowed
particle, as the GO TO 550 loop of util_gpu.F:98-101 does), and RS is then
updated -- by the plain rule (regcor_gpu.F:146-253) or by the learned
predictor with the plain rule as fallback.  The bodies move under the total
force (a second regf call with an empty neighbour sphere gives it), with a
kick-drift-kick leapfrog on the smallest regular step.

Training pairs: the features of a particle at one regular step, and as label
log(RS_k / RS), RS_k the radius that gives it exactly k neighbours at its next
regular step under the kernel's membership test (position or predicted
position inside RS; `label_log_radius_gpu` on the device from the library's
own rows, `label_log_radius` with KD-trees on the host), k the membership the plain rule aims
at for it (regcor_gpu.F:152-163: NNBOPT-stabilised, tapered outside the
half-mass radius).  The rule approaches that membership by at
most 25% in volume per step; the predictor proposes the radius for it
directly.
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass, field

import numpy as np

from . import ics, rsrule
from .gpunb import GpuNb
from .rsmlp import features

CHUNK = 1024            # maxthr of util_gpu.F:7


@dataclass
class HarnessStats:
    regular_calls: int = 0
    active: int = 0
    first_call_overflows: int = 0    # overflows of the first block (same for every policy)
    overflow_events: int = 0         # overflowed rows after it (one recompute each)
    overflow_after_predictor: int = 0  # ... of which the RS came from the predictor
    overflow_after_fallback: int = 0   # ... of which the plain rule replaced a prediction
    recompute_pairs: float = 0.0     # extra pair work of the recomputes
    pairs: float = 0.0               # pair work of the first evaluations
    predictor_used: int = 0
    predictor_fallback: int = 0
    fallback_low: int = 0            # ... count below the band
    fallback_high: int = 0           # ... count above it (the rest: no finite prediction)
    regf_seconds: float = 0.0
    predict_seconds: float = 0.0
    counts: list = field(default_factory=list)

    def as_dict(self):
        d = dict(self.__dict__)
        c = np.concatenate(self.counts) if self.counts else np.zeros(0)
        d.pop("counts")
        d["mean_count"] = float(c.mean()) if c.size else 0.0
        d["count_p99"] = float(np.percentile(c, 99)) if c.size else 0.0
        d["recompute_rate"] = self.overflow_events / max(self.active, 1)
        return d


def initial_rs(x: np.ndarray, nnbopt: int, n: int) -> np.ndarray:
    """fpoly0.F:50-52: RS = RS0 sqrt(1 + r^2); RS0 from the mean density
    (a common choice of the input parameter) -- deliberately not adapted to
    the local density, as at the start of a run."""
    rs0 = (3.0 * nnbopt / (4.0 * math.pi * n)) ** (1.0 / 3.0)
    r2 = np.einsum("ij,ij->i", x, x)
    return rs0 * np.sqrt(1.0 + r2)


def label_log_radius(x: np.ndarray, v: np.ndarray, dtr: np.ndarray, idx: np.ndarray,
                     ks: np.ndarray) -> np.ndarray:
    """log of the radius R at which particle i's neighbour list holds exactly
    k_i members besides itself, under the kernel's own membership test
    min(|dx|^2, |dx + dtr_i dv|^2) < R^2 (gpunb.velocity.cu:172-180): the
    geometric mean of the k-th and (k+1)-th smallest keys q_j =
    min(|dx|^2, |dx + dtr_i dv|^2).

    The k+2 smallest keys are all among the k+2 nearest bodies in position or
    the k+2 nearest in predicted position x + dtr_i v (q_j is at most either
    distance), so two k-nearest queries per step size give them exactly."""
    from scipy.spatial import cKDTree
    out = np.empty(idx.size)
    tree = cKDTree(x)
    d_all = dtr[idx]
    for d in np.unique(d_all):
        sel = np.nonzero(d_all == d)[0]
        ii = idx[sel]
        k = ks[sel]
        K = int(min(k.max() + 2, x.shape[0]))
        _, ja = tree.query(x[ii], k=K, workers=-1)
        xp = x + d * v
        _, jb = cKDTree(xp).query(xp[ii], k=K, workers=-1)
        J = np.sort(np.concatenate([ja, jb], axis=1), axis=1)
        dup = np.zeros(J.shape, dtype=bool)
        dup[:, 1:] = J[:, 1:] == J[:, :-1]
        dx = x[J] - x[ii][:, None, :]
        dp = dx + d * (v[J] - v[ii][:, None, :])
        q = np.minimum(np.einsum("abk,abk->ab", dx, dx), np.einsum("abk,abk->ab", dp, dp))
        q[dup] = np.inf
        q.sort(axis=1)                          # column 0: the body itself (q = 0)
        rows = np.arange(sel.size)
        lo = np.maximum(q[rows, k], 1e-300)
        hi = np.maximum(q[rows, k + 1], lo)
        out[sel] = 0.25 * (np.log(lo) + np.log(hi))
    return out


LABEL_ROW_MAX = 1024     # longest row the device labeller sorts (gpunb_rsmlp_label_device)


def label_log_radius_gpu(nb: GpuNb, x: np.ndarray, v: np.ndarray, dtr: np.ndarray,
                         idx: np.ndarray, ks: np.ndarray, r_hint: np.ndarray) -> np.ndarray:
    """The labels of `label_log_radius`, computed on the device from the
    library's own neighbour rows: the j-set must be the one last sent to `nb`
    (positions x, velocities v).  Each row is taken at a radius 1.3 r_hint
    (r_hint: an estimate of R_k, e.g. RS (k+2)^(1/3) / (count+1)^(1/3)),
    doubled for the rows that hold fewer than k + 2 members and shrunk for
    those above LABEL_ROW_MAX, until every row qualifies; the keys of a
    qualifying row are exact, so the labels equal the KD-tree ones."""
    import torch
    lib = nb.lib
    fn = lib.gpunb_rsmlp_label_device
    dev = torch.device("cuda", 0)
    xd = torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64, device=dev)
    vd = torch.as_tensor(np.ascontiguousarray(v), dtype=torch.float64, device=dev)
    out = np.full(idx.size, np.nan)
    todo = np.arange(idx.size)
    scale = np.full(idx.size, 1.3)
    nnbmax = LABEL_ROW_MAX
    for _ in range(40):
        if todo.size == 0:
            break
        ii = idx[todo]
        ni = ii.size
        r = scale[todo] * r_hint[todo]
        h2 = torch.as_tensor(r * r, dtype=torch.float64, device=dev)
        dt = torch.as_tensor(dtr[ii], dtype=torch.float64, device=dev)
        sel = torch.as_tensor(ii, device=dev)
        xi = xd[sel].contiguous()
        vi = vd[sel].contiguous()
        acc = torch.empty((ni, 3), dtype=torch.float64, device=dev)
        jrk = torch.empty_like(acc)
        pot = torch.empty(ni, dtype=torch.float64, device=dev)
        nnb = torch.empty(ni, dtype=torch.int32, device=dev)
        off = torch.empty(ni + 1, dtype=torch.int32, device=dev)
        lst = torch.empty(ni * nnbmax, dtype=torch.int32, device=dev)
        kd = torch.as_tensor(ks[todo].astype(np.int32), device=dev)
        logr = torch.empty(ni, dtype=torch.float64, device=dev)
        ok = torch.empty(ni, dtype=torch.int32, device=dev)
        torch.cuda.synchronize()
        rc = lib.gpunb_regf_device(ni, h2.data_ptr(), dt.data_ptr(), xi.data_ptr(),
                                   vi.data_ptr(), acc.data_ptr(), jrk.data_ptr(), pot.data_ptr(),
                                   nnb.data_ptr(), off.data_ptr(), lst.data_ptr(), ni * nnbmax,
                                   nnbmax, 0, None)
        if rc != 0:
            raise RuntimeError(f"gpunb_regf_device failed ({rc})")
        # the regf call ran on the library's own stream: wait for it (and read
        # its error word) before the labeller runs on the default stream
        if lib.gpunb_device_status(None) != 0:
            raise RuntimeError("device error in the regular-force pass of the labeller")
        rc = fn(ni, off.data_ptr(), lst.data_ptr(), nnb.data_ptr(), xd.data_ptr(), vd.data_ptr(),
                xi.data_ptr(), vi.data_ptr(), dt.data_ptr(), kd.data_ptr(), logr.data_ptr(),
                ok.data_ptr(), None)
        if rc != 0:
            raise RuntimeError(f"gpunb_rsmlp_label_device failed ({rc})")
        torch.cuda.synchronize()
        okh = ok.cpu().numpy()
        good = okh == 1
        out[todo[good]] = logr.cpu().numpy()[good]
        scale[todo[okh == 0]] *= 2.0
        scale[todo[okh == -1]] *= 0.8
        todo = todo[~good]
    if todo.size:
        raise RuntimeError(f"{todo.size} labels did not converge")
    return out


# accepted range of the count a predicted radius gives, as a multiple of the
# plain rule's target (the device update kernel takes the same bounds):
# 0.5-1.5 by default; WIDE_BAND lowers the floor
PRED_BAND = (0.5, 1.5)
WIDE_BAND = (0.25, 1.5)

# How the count of a predicted radius is estimated for the band check
# ("max" by default):
#   "motion": at the next regular step -- the members of the current list
#             moved on their relative velocities by one regular step and
#             tested as the kernel tests them then (position or predicted
#             position inside the radius), plus, for a growing radius, the
#             shell beyond the current radius at the current density;
#   "static": at the current density, count x (RS_new / RS)^3;
#   "max":    the larger of the two.
# In a contraction a correct prediction of a strong shrink implies a low count
# at today's density, so the static estimate rejects it and the lagging plain
# rule then overflows; the motion estimate follows the neighbours inwards.
# Over a long regular step the straight-line motion undercounts instead
# (orbits curve, the infall accelerates): measured against the counts the
# predicted radii had (Plummer 65536 collapse), the motion estimate reads
# about half the true count on the rows it rejects, which the static one gets
# right, so a prediction is taken as too small only when both say so.
GUARDS = ("motion", "static", "max")


def motion_count(x: np.ndarray, v: np.ndarray, idx: np.ndarray, rows: np.ndarray,
                 dtr: np.ndarray, rs_new: np.ndarray, rs_old: np.ndarray) -> np.ndarray:
    """Estimated count of radius rs_new at the next regular step of the
    particles idx: members j of their current rows (LISTGP layout, 0-based ids,
    self included and skipped here) with
    min(|dx'|^2, |dx' + dtr dv|^2) < rs_new^2, dx' = dx + dtr dv (the kernel's
    membership test one step later, separations moved on the current relative
    velocity), plus count x ((rs_new / rs_old)^3 - 1) when the radius grows."""
    out = np.zeros(idx.size)
    cnt = np.zeros(idx.size)
    for s in range(0, idx.size, CHUNK):
        ii = idx[s:s + CHUNK]
        r = rows[s:s + CHUNK]
        m = np.maximum(r[:, 0], 0)
        width = int(m.max()) if m.size else 0
        if width == 0:
            continue
        ids = r[:, 1:1 + width].astype(np.int64)
        valid = (np.arange(width)[None, :] < m[:, None]) & (ids != ii[:, None])
        j = np.where(valid, ids, ii[:, None])
        dt = dtr[ii][:, None, None]
        dv = v[j] - v[ii][:, None, :]
        d1 = x[j] - x[ii][:, None, :] + dt * dv
        d2 = d1 + dt * dv
        key = np.minimum((d1 * d1).sum(-1), (d2 * d2).sum(-1))
        out[s:s + CHUNK] = (valid & (key < (rs_new[s:s + CHUNK] ** 2)[:, None])).sum(1)
        cnt[s:s + CHUNK] = valid.sum(1)
    return out + cnt * np.maximum((rs_new / rs_old) ** 3 - 1.0, 0.0)


def motion_count_device(xd, vd, idx: np.ndarray, rows: np.ndarray, dtr: np.ndarray,
                        rs_new: np.ndarray, rs_old: np.ndarray, chunk: int = 16384) -> np.ndarray:
    """`motion_count` evaluated with torch on the device: xd, vd are device
    tensors of the whole set's positions and velocities; the rest as there."""
    import torch
    dev = xd.device
    out = np.zeros(idx.size)
    cnt = np.zeros(idx.size)
    for s in range(0, idx.size, chunk):
        r = rows[s:s + chunk]
        m = np.maximum(r[:, 0], 0)
        width = int(m.max()) if m.size else 0
        if width == 0:
            continue
        ii = torch.as_tensor(idx[s:s + chunk], device=dev)
        ids = torch.as_tensor(r[:, 1:1 + width].astype(np.int64), device=dev)
        mm = torch.as_tensor(m, device=dev)
        valid = (torch.arange(width, device=dev)[None, :] < mm[:, None]) & (ids != ii[:, None])
        j = torch.where(valid, ids, ii[:, None])
        dt = torch.as_tensor(dtr[idx[s:s + chunk]], dtype=torch.float64, device=dev)[:, None, None]
        dv = vd[j] - vd[ii][:, None, :]
        d1 = xd[j] - xd[ii][:, None, :] + dt * dv
        d2 = d1 + dt * dv
        key = torch.minimum((d1 * d1).sum(-1), (d2 * d2).sum(-1))
        rn = torch.as_tensor(rs_new[s:s + chunk], dtype=torch.float64, device=dev)
        out[s:s + chunk] = (valid & (key < (rn * rn)[:, None])).sum(1).cpu().numpy()
        cnt[s:s + chunk] = valid.sum(1).cpu().numpy()
    return out + cnt * np.maximum((rs_new / rs_old) ** 3 - 1.0, 0.0)


class Harness:
    def __init__(self, cluster: ics.Cluster, nnbopt: int, nnbmax: int, smax: float = 0.125,
                 levels: int = 4, params: rsrule.RSParams | None = None, rs=None,
                 harvest: bool = False, rs0_factor: float = 1.0,
                 band: tuple[float, float] = PRED_BAND, gpu_labels: bool = True,
                 guard: str = "max", harvest_every: int = 1):
        if guard not in GUARDS:
            raise ValueError(f"guard must be one of {GUARDS}")
        self.c = cluster
        self.gpu_labels = gpu_labels   # labels from the device labeller (else KD-tree)
        self.band = band
        self.guard = guard
        self.n = cluster.n
        self.nnbopt, self.nnbmax = nnbopt, nnbmax
        self.m = cluster.m.copy()
        self.x = cluster.x.copy()
        self.v = cluster.v.copy()
        self.rs = (rs0_factor * initial_rs(self.x, nnbopt, self.n) if rs is None
                   else rs.copy())
        # regular steps: fpoly0.F:55-56, quantised to SMAX / 2^k, k < levels
        st = ics.regular_step(self.x, smax)
        k = np.clip(np.ceil(np.log2(smax / st)), 0, levels - 1).astype(int)
        self.stepr = smax / 2.0 ** k
        self.dt = smax / 2.0 ** (levels - 1)
        self.tick = 0
        self.next_tick = (self.stepr / self.dt).round().astype(int)
        self.prev_nnb = np.full(self.n, nnbopt, dtype=np.int64)
        # RS source of each particle: 0 plain rule, 1 predictor, 2 plain rule
        # after a rejected prediction
        self.src = np.zeros(self.n, dtype=np.int64)
        self.p = params or rsrule.RSParams(nnbopt=nnbopt, nnbmax=nnbmax,
                                           bodym=float(self.m.mean()))
        self.nb = GpuNb(self.n)
        self.acc = self._total_force()
        self.harvest = harvest
        self.harvest_every = max(1, int(harvest_every))   # label the bodies i % k == 0
        self.pending = {}
        self.X, self.Y = [], []
        # with harvest and a predictor: per labelled row (label, y, motion
        # count, static count, target, accepted) for the band diagnostics
        self.diag = []
        self.stats = HarnessStats()

    def close(self):
        self.nb.close()

    # -- dynamics -------------------------------------------------------------
    def _total_force(self):
        self.nb.send(self.m, self.x, self.v)
        h2 = np.full(self.n, 1e-30)
        r = self.nb.regf(h2, np.zeros(self.n), self.x, self.v, 2, 1)
        return r.acc

    def _kdk(self):
        self.v += 0.5 * self.dt * self.acc
        self.x += self.dt * self.v
        self.acc = self._total_force()
        self.v += 0.5 * self.dt * self.acc
        self.tick += 1

    # -- the regular block ---------------------------------------------------------
    def _regf_with_recompute(self, idx):
        """gpunb_regf_ on the active block in chunks of CHUNK; overflowed rows
        are shrunk by the overflow rule and their chunk recomputed, one
        recompute per overflowed row (util_gpu.F:66-101)."""
        lmax = self.nnbmax + 1
        t0 = time.perf_counter()
        self.nb.send(self.m, self.x, self.v)
        accs, jrks, nnbs, lists = [], [], [], []
        for s in range(0, idx.size, CHUNK):
            ch = idx[s:s + CHUNK]
            res = self.nb.regf(self.rs[ch] ** 2, self.stepr[ch], self.x[ch], self.v[ch], lmax,
                               self.nnbmax)
            self.stats.pairs += ch.size * float(self.n)
            while True:
                over = res.list[:, 0] < 0
                nover = int(over.sum())
                if nover == 0:
                    break
                if self.stats.regular_calls == 0:
                    self.stats.first_call_overflows += nover
                else:
                    self.stats.overflow_events += nover
                    self.stats.overflow_after_predictor += int((self.src[ch[over]] == 1).sum())
                    self.stats.overflow_after_fallback += int((self.src[ch[over]] == 2).sum())
                    self.stats.recompute_pairs += nover * ch.size * float(self.n)
                self.rs[ch[over]] = rsrule.overflow_rs(self.rs[ch[over]], res.list[over, 0],
                                                       self.p)
                sub = ch[over]
                r2 = self.nb.regf(self.rs[sub] ** 2, self.stepr[sub], self.x[sub], self.v[sub],
                                  lmax, self.nnbmax)
                res.acc[over] = r2.acc
                res.jrk[over] = r2.jrk
                res.pot[over] = r2.pot
                res.list[over] = r2.list
            accs.append(res.acc); jrks.append(res.jrk)
            nnbs.append(res.list[:, 0].copy()); lists.append(res.list)
        self.stats.regf_seconds += time.perf_counter() - t0
        self.stats.regular_calls += 1
        return (np.concatenate(accs), np.concatenate(jrks), np.concatenate(nnbs),
                np.concatenate(lists))

    def step(self, predictor=None):
        """Advance one tick; returns the active block's size."""
        self._kdk()
        idx = np.nonzero(self.next_tick <= self.tick)[0]
        if idx.size == 0:
            return 0
        acc, jrk, nnb_raw, rows = self._regf_with_recompute(idx)
        nnb = np.maximum(nnb_raw - 1, 0)                 # self removed (util_gpu.F:102-111)
        self.stats.active += idx.size
        self.stats.counts.append(nnb)
        if self.harvest:
            self._harvest(idx)
        F = features(self.x[idx], self.v[idx], self.m[idx] * self.n, self.rs[idx], nnb, acc,
                     jrk, self.stepr[idx], self.nnbopt)
        rs_old = self.rs[idx].copy()
        plain, target = rsrule.regcor_rs(rs_old, nnb, self.prev_nnb[idx], self.x[idx],
                                         self.v[idx], self.stepr[idx], self.p,
                                         return_target=True)
        plain = np.where(nnb < 2, rsrule.few_nb_rs(rs_old), plain)
        new = plain
        self.src[idx] = 0
        if predictor is not None:
            t0 = time.perf_counter()
            y = predictor.predict(F)
            self.stats.predict_seconds += time.perf_counter() - t0
            # the count the predicted radius gives (GUARDS); outside band x
            # the rule's own target the plain rule is used
            static_count = (nnb + 1.0) * np.exp(3.0 * y) - 1.0
            if self.guard == "static":
                pred_count = static_count
            else:
                pred_count = self._motion_count(idx, rows, rs_old * np.exp(
                    np.where(np.isfinite(y), y, 0.0)), rs_old)
                if self.guard == "max":
                    pred_count = np.maximum(pred_count, static_count)
            lo, hi = self.band
            ok = (pred_count >= lo * target) & (pred_count <= hi * target) & np.isfinite(y)
            new = np.where(ok, rs_old * np.exp(y), plain)
            self.src[idx] = np.where(ok, 1, 2)
            self.stats.fallback_low += int((pred_count < lo * target).sum())
            self.stats.fallback_high += int((pred_count > hi * target).sum())
            self.stats.predictor_used += int(ok.sum())
            self.stats.predictor_fallback += int((~ok).sum())
        if self.harvest:
            if predictor is not None:   # the motion estimate, for the diagnostics
                mc = (pred_count if self.guard == "motion" else
                      self._motion_count(idx, rows, rs_old * np.exp(
                          np.where(np.isfinite(y), y, 0.0)), rs_old))
            for q, i in enumerate(idx):
                if int(i) % self.harvest_every:
                    continue
                d = None
                if predictor is not None:
                    d = (float(y[q]), float(mc[q]), float(static_count[q]), bool(ok[q]))
                self.pending[int(i)] = (F[q], rs_old[q], target[q], d)
        self.rs[idx] = new
        self.prev_nnb[idx] = nnb
        self.next_tick[idx] += (self.stepr[idx] / self.dt).round().astype(int)
        return idx.size

    def _motion_count(self, idx, rows, rs_new, rs_old):
        """motion_count on the device (the set's current positions copied over)."""
        import torch
        dev = torch.device("cuda", 0)
        xd = torch.as_tensor(self.x, dtype=torch.float64, device=dev)
        vd = torch.as_tensor(self.v, dtype=torch.float64, device=dev)
        return motion_count_device(xd, vd, idx, rows, self.stepr, rs_new, rs_old)

    def _harvest(self, idx):
        have = np.array([int(i) for i in idx if int(i) in self.pending], dtype=np.int64)
        if have.size == 0:
            return
        ks = np.array([int(min(max(round(self.pending[i][2]), 1), self.n - 3)) for i in have])
        if self.gpu_labels and ks.max() + 2 <= LABEL_ROW_MAX:
            cnt = np.maximum(self.prev_nnb[have], 0) + 1.0
            hint = self.rs[have] * np.cbrt((ks + 2.0) / cnt)
            logr = label_log_radius_gpu(self.nb, self.x, self.v, self.stepr, have, ks, hint)
        else:
            logr = label_log_radius(self.x, self.v, self.stepr, have, ks)
        for q, i in enumerate(have):
            f, rs_then, tgt, d = self.pending.pop(int(i))
            self.X.append(f)
            self.Y.append(logr[q] - math.log(rs_then))
            if d is not None:
                self.diag.append((self.Y[-1],) + d[:3] + (tgt, d[3]))

    def run(self, ticks: int, predictor=None):
        for _ in range(ticks):
            self.step(predictor)
        return self.stats

    def dataset(self):
        return np.array(self.X), np.array(self.Y)
