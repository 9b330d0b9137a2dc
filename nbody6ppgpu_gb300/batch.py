"""Batched clusters on the device: many independent j-sets, each with its own
active block, computed by one persistent launch (gpunb_batch_send_device /
gpunb_batch_regf_device).  torch provides the device buffers and the stream;
all computation is in libgpunb.so."""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from .gpunb import GpunbError, _check, load


@dataclass
class BatchResult:
    acc: list          # per set: [ni_c, 3]
    jrk: list
    pot: list
    nnb: list          # per set: [ni_c] count or -count
    lists: list        # per set: list of id arrays (ids within the set)


class DeviceBatch:
    """Holds the concatenated device arrays of one batch of sets."""

    def __init__(self, sets, active, nnbmax: int, device=0, stream=None):
        """sets: list of (m, x, v) numpy arrays; active: list of index arrays
        into each set (the active block)."""
        import torch
        self.torch = torch
        self.lib = load()
        self.dev = torch.device("cuda", device)
        self.stream = stream or torch.cuda.Stream(self.dev)
        self.ncl = len(sets)
        self.nj = np.array([len(s[0]) for s in sets], dtype=np.int32)
        self.ni = np.array([len(a) for a in active], dtype=np.int32)
        self.nnbmax = int(nnbmax)
        T = lambda a: torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64).to(self.dev)
        self.m = T(np.concatenate([s[0] for s in sets]))
        self.x = T(np.concatenate([s[1] for s in sets]).reshape(-1, 3))
        self.v = T(np.concatenate([s[2] for s in sets]).reshape(-1, 3))
        self._active = active
        self._sets = sets
        tot = int(self.ni.sum())
        self.total_ni = tot
        self.h2 = torch.empty(tot, dtype=torch.float64, device=self.dev)
        self.dtr = torch.empty(tot, dtype=torch.float64, device=self.dev)
        self.xi = T(np.concatenate([s[1][a] for s, a in zip(sets, active)]).reshape(-1, 3))
        self.vi = T(np.concatenate([s[2][a] for s, a in zip(sets, active)]).reshape(-1, 3))
        self.acc = torch.empty((tot, 3), dtype=torch.float64, device=self.dev)
        self.jrk = torch.empty((tot, 3), dtype=torch.float64, device=self.dev)
        self.pot = torch.empty(tot, dtype=torch.float64, device=self.dev)
        self.nnb = torch.empty(tot, dtype=torch.int32, device=self.dev)
        self.off = torch.empty(tot + 1, dtype=torch.int32, device=self.dev)
        self.lst = torch.empty(max(tot * self.nnbmax, 1), dtype=torch.int32, device=self.dev)

    def set_radii(self, h2_list, dtr_list):
        self.h2.copy_(self.torch.as_tensor(np.concatenate(h2_list)))
        self.dtr.copy_(self.torch.as_tensor(np.concatenate(dtr_list)))

    def send(self):
        nj = (C.c_int * self.ncl)(*self.nj.tolist())
        rc = self.lib.gpunb_batch_send_device(self.ncl, nj, self.m.data_ptr(), self.x.data_ptr(),
                                              self.v.data_ptr(), self.stream.cuda_stream)
        if rc:
            _check(self.lib)
            raise GpunbError(rc, "batch send")

    def regf(self, m_flag: int = 0):
        ni = (C.c_int * self.ncl)(*self.ni.tolist())
        rc = self.lib.gpunb_batch_regf_device(
            self.ncl, ni, self.h2.data_ptr(), self.dtr.data_ptr(), self.xi.data_ptr(),
            self.vi.data_ptr(), self.acc.data_ptr(), self.jrk.data_ptr(), self.pot.data_ptr(),
            self.nnb.data_ptr(), self.off.data_ptr(), self.lst.data_ptr(),
            self.total_ni * self.nnbmax, self.nnbmax, int(m_flag), self.stream.cuda_stream)
        if rc:
            _check(self.lib)
            raise GpunbError(rc, "batch regf")

    def results(self) -> BatchResult:
        self.stream.synchronize()
        acc = self.acc.cpu().numpy(); jrk = self.jrk.cpu().numpy(); pot = self.pot.cpu().numpy()
        nnb = self.nnb.cpu().numpy(); off = self.off.cpu().numpy(); lst = self.lst.cpu().numpy()
        out = BatchResult([], [], [], [], [])
        o = 0
        for c in range(self.ncl):
            k = int(self.ni[c])
            out.acc.append(acc[o:o + k]); out.jrk.append(jrk[o:o + k]); out.pot.append(pot[o:o + k])
            out.nnb.append(nnb[o:o + k])
            out.lists.append([lst[off[i]:off[i + 1]] for i in range(o, o + k)])
            o += k
        return out

    def last_plan(self):
        v, n = C.c_int(), C.c_int()
        self.lib.gpunb_batch_last_plan(C.byref(v), C.byref(n))
        return v.value, n.value
