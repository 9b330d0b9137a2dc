"""Sharding the regular-force path over processes, one GPU per process.

The reference has two schemes; both are restated here over torch.distributed
(NCCL between GPUs, gloo between CPU processes):

* i-split (src/Main/intgrt.F:992-1031): every rank holds the whole j-set and
  computes a contiguous block of the active list -- NL/size rows each, the
  first NL mod size ranks one more -- and the rows are then exchanged so that
  every rank holds all of them (the MPI_SENDRECV ring of :1100-1131; here one
  all_gather).
* j-split (src/Main/gpunb.velocity.cu:643-645,703-729,822-878): rank r holds
  the j-slice [joff[r], joff[r+1]), joff[r] = r*nj // size, and computes
  partial sums and a partial list for every active particle; the partials are
  summed in FP64 in rank order and the lists concatenated with the slice
  offsets added, which keeps them ascending.

The per-rank computation is any callable with the signature of
`GpuNb.regf` (h2, dtr, xi, vi, lmax, nnbmax, m_flag) -> RegfResult, normally
the library on the rank's own GPU.  Results do not depend on the number of
ranks: the i-split returns exactly the single-process rows, the j-split the
same lists and sums that differ only by the FP64 rounding of the partial sums.
"""
from __future__ import annotations

from typing import Callable, Sequence

import numpy as np

from .gpunb import RegfResult

RegfFn = Callable[..., RegfResult]


def i_split(nl: int, size: int) -> tuple[np.ndarray, np.ndarray]:
    """(start, count) of every rank's block of an active list of length nl
    (intgrt.F:995-1008, 0-based starts)."""
    if nl < 0 or size < 1:
        raise ValueError("need nl >= 0 and size >= 1")
    inl, idiff = divmod(nl, size)
    count = np.full(size, inl, dtype=np.int64)
    count[:idiff] += 1
    start = np.concatenate([[0], np.cumsum(count)[:-1]])
    return start, count


def j_offsets(nj: int, size: int) -> np.ndarray:
    """Slice boundaries joff[0..size] of the j-split (gpunb.velocity.cu:715-717)."""
    if nj < 0 or size < 1:
        raise ValueError("need nj >= 0 and size >= 1")
    return np.array([(r * nj) // size for r in range(size + 1)], dtype=np.int64)


def merge_j_parts(parts: Sequence[RegfResult], joff: Sequence[int], nnbmax: int) -> RegfResult:
    """Merge the partial results of the ranks of a j-split, in rank order
    (gpunb.velocity.cu:822-878).  Partial ids are local to their slice.

    The merged count is the sum of the partial member counts; the row
    overflows (count reported as -count) when that sum exceeds nnbmax, which
    includes every row where a part already overflowed.  The reference adds
    a negative partial count into its sum; here the reported value is the
    true member count, as a single-process call reports it."""
    if not parts:
        raise ValueError("no parts")
    ni, lmax = parts[0].list.shape
    acc = np.zeros((ni, 3))
    jrk = np.zeros((ni, 3))
    pot = np.zeros(ni)
    for p in parts:                 # fixed order: deterministic FP64 sums
        acc += p.acc
        jrk += p.jrk
        pot += p.pot
    counts = np.stack([np.abs(p.list[:, 0]) for p in parts]).astype(np.int64)   # [size, ni]
    total = counts.sum(0)
    over = total > nnbmax
    out = np.zeros((ni, lmax), dtype=np.int32)
    out[:, 0] = np.where(over, -total, total)
    # rank r's members of row i go to columns 1 + (members of ranks < r) + k
    prefix = np.cumsum(counts, axis=0) - counts
    k = np.arange(lmax - 1)
    for r, p in enumerate(parts):
        rows, cols = np.nonzero((k[None, :] < counts[r][:, None]) & ~over[:, None])
        out[rows, 1 + prefix[r, rows] + cols] = p.list[rows, 1 + cols] + int(joff[r])
    return RegfResult(acc=acc, jrk=jrk, pot=pot, list=out)


class ShardedRegf:
    """Regular force of one active block, sharded over the ranks of a
    torch.distributed process group.  `regf` is this rank's computation (its
    j-set already sent: all bodies for the i-split, the rank's slice for the
    j-split); `device` is where the exchange buffers live ("cuda" for NCCL,
    "cpu" for gloo)."""

    def __init__(self, regf: RegfFn, group=None, device: str = "cpu"):
        import torch
        import torch.distributed as dist
        self.torch, self.dist = torch, dist
        self.regf_fn = regf
        self.group = group
        self.device = device
        self.size = dist.get_world_size(group)
        self.rank = dist.get_rank(group)

    def _all_gather(self, a: np.ndarray) -> list[np.ndarray]:
        t = self.torch.from_numpy(np.ascontiguousarray(a)).to(self.device)
        bufs = [self.torch.empty_like(t) for _ in range(self.size)]
        self.dist.all_gather(bufs, t, group=self.group)
        return [b.cpu().numpy() for b in bufs]

    def i_split(self, h2, dtr, xi, vi, lmax: int, nnbmax: int, m_flag: int = 0) -> RegfResult:
        """Every rank returns all ni rows; rank r computed rows
        [start[r], start[r] + count[r]).  The rows travel compact: the forces,
        the signed counts and the accepted members only (padded to the
        longest rank's), not lmax-wide rows."""
        ni = len(h2)
        start, count = i_split(ni, self.size)
        s, c = int(start[self.rank]), int(count[self.rank])
        cmax = int(count.max())
        f = np.zeros((cmax, 8))
        ids = np.zeros(0, dtype=np.int32)
        if c:
            r = self.regf_fn(h2[s:s + c], dtr[s:s + c], xi[s:s + c], vi[s:s + c], lmax, nnbmax,
                             m_flag)
            f[:c, 0:3], f[:c, 3:6], f[:c, 6] = r.acc, r.jrk, r.pot
            f[:c, 7] = r.list[:, 0]
            n_acc = np.maximum(r.list[:, 0], 0)
            rows, cols = np.nonzero(np.arange(lmax - 1)[None, :] < n_acc[:, None])
            ids = r.list[rows, 1 + cols].astype(np.int32)
        sizes = self._all_gather(np.array([ids.size], dtype=np.int64))
        width = int(max(int(z[0]) for z in sizes))
        pad = np.zeros(max(width, 1), dtype=np.int32)
        pad[:ids.size] = ids
        fs, idss = self._all_gather(f), self._all_gather(pad)
        F = np.concatenate([fs[q][:count[q]] for q in range(self.size)])
        nnb = F[:, 7].astype(np.int32)
        allids = np.concatenate([idss[q][:int(sizes[q][0])] for q in range(self.size)])
        L = np.zeros((ni, lmax), dtype=np.int32)
        L[:, 0] = nnb
        n_acc = np.maximum(nnb, 0)
        rows, cols = np.nonzero(np.arange(lmax - 1)[None, :] < n_acc[:, None])
        L[rows, 1 + cols] = allids
        return RegfResult(acc=F[:, 0:3].copy(), jrk=F[:, 3:6].copy(), pot=F[:, 6].copy(), list=L)

    def j_split(self, joff: Sequence[int], h2, dtr, xi, vi, lmax: int, nnbmax: int,
                m_flag: int = 0) -> RegfResult:
        """Every rank returns the merged rows of all ni particles; this rank's
        `regf` covers j-slice [joff[rank], joff[rank+1])."""
        r = self.regf_fn(h2, dtr, xi, vi, lmax, nnbmax, m_flag)
        f = np.concatenate([r.acc, r.jrk, r.pot[:, None]], axis=1)
        fs, ls = self._all_gather(f), self._all_gather(r.list)
        parts = [RegfResult(acc=fs[q][:, 0:3], jrk=fs[q][:, 3:6], pot=fs[q][:, 6], list=ls[q])
                 for q in range(self.size)]
        return merge_j_parts(parts, joff, nnbmax)
