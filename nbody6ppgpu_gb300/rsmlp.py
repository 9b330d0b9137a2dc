"""Learned neighbour-radius predictor (8 -> 64 -> 64 -> 1 MLP, GELU, BF16
weights, FP32 accumulation), trained and evaluated by the hand-written kernels
of csrc/rsmlp.cu.  torch supplies device buffers and the stream only.

The model predicts y = log(RS_k / RS), RS_k the radius that holds k
neighbours at the particle's next regular step under the kernel's membership
test (position or predicted position inside RS), k the membership the plain
rule aims at (src/Main/regcor_gpu.F:152-163).  It never touches forces: its
output replaces the plain RS rule (regcor_gpu.F:146-253) only when the count
it implies stays within 0.5-1.5 x that target (the band is a parameter); otherwise, and after any list
overflow, the plain rules of `rsrule` apply.

Features (per active particle, before its RS is updated):
  0 log distance to the density centre     4 log |jerk|
  1 log local density from the neighbours   5 log regular step
  2 previous neighbour count / NNBOPT       6 log (mass x N)
  3 log |F_reg|                             7 log RS
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from .gpunb import load

NF = 8


def features(x, v, m_scaled, rs, nnb, acc, jrk, dtr, nnbopt, centre=(0.0, 0.0, 0.0)):
    """Feature matrix [n, 8] (float64) of the active particles."""
    r = np.linalg.norm(x - np.asarray(centre), axis=1)
    dens = (np.maximum(nnb, 0) + 1.0) / (4.0 / 3.0 * np.pi * rs ** 3)
    tiny = 1e-30
    return np.stack([
        np.log(r + 1e-6),
        np.log(dens),
        np.maximum(nnb, 0) / float(nnbopt),
        np.log(np.linalg.norm(acc, axis=1) + tiny),
        np.log(np.linalg.norm(jrk, axis=1) + tiny),
        np.log(np.maximum(dtr, 1e-12)),
        np.log(np.maximum(m_scaled, 1e-12)),
        np.log(rs),
    ], axis=1)


class RSMLP:
    """Parameters on the device: FP32 master copy, BF16 copy, Adam moments."""

    def __init__(self, seed: int = 0, device: int = 0):
        import torch
        self.torch = torch
        self.lib = load()
        for name, args, res in [
            ("gpunb_rsmlp_num_params", [], C.c_int),
            ("gpunb_rsmlp_to_bf16", [C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
            ("gpunb_rsmlp_forward", [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                     C.c_void_p], C.c_int),
            ("gpunb_rsmlp_backward", [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                      C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                      C.c_void_p], C.c_int),
            ("gpunb_rsmlp_adam", [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_float,
                                  C.c_float, C.c_float, C.c_float, C.c_int, C.c_void_p,
                                  C.c_void_p], C.c_int),
        ]:
            f = getattr(self.lib, name)
            f.argtypes = args
            f.restype = res
        self.P = self.lib.gpunb_rsmlp_num_params()
        self.dev = torch.device("cuda", device)
        self.stream = torch.cuda.Stream(self.dev)
        rng = np.random.default_rng(seed)
        w = np.zeros(self.P, dtype=np.float32)
        H, I = 64, NF
        o = 0
        w[o:o + H * I] = rng.normal(0, np.sqrt(2.0 / (I + H)), H * I); o += H * I + H
        w[o:o + H * H] = rng.normal(0, np.sqrt(2.0 / (H + H)), H * H); o += H * H + H
        w[o:o + H] = rng.normal(0, np.sqrt(2.0 / (H + 1)), H)
        self.master = torch.tensor(w, device=self.dev)
        self.m1 = torch.zeros_like(self.master)
        self.m2 = torch.zeros_like(self.master)
        self.wq = torch.empty(self.P, dtype=torch.bfloat16, device=self.dev)
        self.grad = torch.zeros_like(self.master)
        self.loss = torch.zeros(1, dtype=torch.float32, device=self.dev)
        self.step_count = 0
        self.mu = np.zeros(NF)
        self.sd = np.ones(NF)
        self._sync_bf16()

    # -- helpers -------------------------------------------------------------
    def _sync_bf16(self):
        rc = self.lib.gpunb_rsmlp_to_bf16(self.master.data_ptr(), self.wq.data_ptr(),
                                          self.stream.cuda_stream)
        assert rc == 0
        self.stream.synchronize()

    def _dev(self, a, dtype=None):
        t = self.torch.as_tensor(np.ascontiguousarray(a, dtype=np.float32))
        return t.to(self.dev)

    def set_normalisation(self, X: np.ndarray):
        self.mu = X.mean(0)
        self.sd = X.std(0) + 1e-6

    def normalise(self, X: np.ndarray) -> np.ndarray:
        return ((X - self.mu) / self.sd).astype(np.float32)

    # -- kernels ---------------------------------------------------------------
    def forward_normalised(self, Xn: np.ndarray) -> np.ndarray:
        B = Xn.shape[0]
        xd = self._dev(Xn)
        y = self.torch.empty(max(B, 1), dtype=self.torch.float32, device=self.dev)
        self.torch.cuda.synchronize()
        rc = self.lib.gpunb_rsmlp_forward(B, xd.data_ptr(), self.wq.data_ptr(),
                                          self.master.data_ptr(), y.data_ptr(),
                                          self.stream.cuda_stream)
        assert rc == 0
        self.stream.synchronize()
        return y.cpu().numpy()[:B]

    def predict(self, X: np.ndarray) -> np.ndarray:
        return self.forward_normalised(self.normalise(X))

    def gradient(self, Xn: np.ndarray, T: np.ndarray, W: np.ndarray | None = None):
        """Gradient (FP32, P) and loss of mean w (y - t)^2 on one batch."""
        B = Xn.shape[0]
        xd, td = self._dev(Xn), self._dev(T)
        wd = self._dev(W) if W is not None else None
        nb = (B + 127) // 128
        part = self.torch.empty(nb * self.P + nb, dtype=self.torch.float32, device=self.dev)
        self.torch.cuda.synchronize()
        rc = self.lib.gpunb_rsmlp_backward(B, xd.data_ptr(), td.data_ptr(),
                                           wd.data_ptr() if wd is not None else None,
                                           self.wq.data_ptr(), self.master.data_ptr(),
                                           self.grad.data_ptr(), self.loss.data_ptr(),
                                           part.data_ptr(), self.stream.cuda_stream)
        assert rc == 0
        self.stream.synchronize()
        return self.grad.cpu().numpy().copy(), float(self.loss.cpu().numpy()[0])

    def train(self, X: np.ndarray, T: np.ndarray, epochs: int = 20, batch: int = 4096,
              lr: float = 2e-3, lr_final: float = 1e-4, seed: int = 0,
              verbose: bool = False) -> list:
        """Adam on the GPU kernels, learning rate decayed geometrically from lr
        to lr_final over the run; returns the per-epoch mean loss."""
        torch = self.torch
        self.set_normalisation(X)
        Xn = self.normalise(X)
        T = T.astype(np.float32)
        rng = np.random.default_rng(seed)
        n = Xn.shape[0]
        losses = []
        xd_all, td_all = self._dev(Xn), self._dev(T)
        nb_max = (batch + 127) // 128
        part = torch.empty(nb_max * self.P + nb_max, dtype=torch.float32, device=self.dev)
        torch.cuda.synchronize()
        sp = self.stream.cuda_stream
        steps_total = epochs * ((n + batch - 1) // batch)
        decay = (lr_final / lr) ** (1.0 / max(steps_total - 1, 1))
        it = 0
        for ep in range(epochs):
            perm = rng.permutation(n)
            xd = xd_all[torch.as_tensor(perm, device=self.dev)]
            td = td_all[torch.as_tensor(perm, device=self.dev)]
            torch.cuda.synchronize()
            tot = 0.0
            nbat = 0
            for s in range(0, n, batch):
                B = min(batch, n - s)
                rc = self.lib.gpunb_rsmlp_backward(B, xd.data_ptr() + 4 * NF * s,
                                                   td.data_ptr() + 4 * s, None,
                                                   self.wq.data_ptr(), self.master.data_ptr(),
                                                   self.grad.data_ptr(), self.loss.data_ptr(),
                                                   part.data_ptr(), sp)
                assert rc == 0
                self.step_count += 1
                lr_it = lr * decay ** it
                it += 1
                rc = self.lib.gpunb_rsmlp_adam(self.master.data_ptr(), self.m1.data_ptr(),
                                               self.m2.data_ptr(), self.grad.data_ptr(), lr_it,
                                               0.9, 0.999, 1e-8, self.step_count,
                                               self.wq.data_ptr(), sp)
                assert rc == 0
                nbat += 1
            self.stream.synchronize()
            # epoch loss on the full set (forward kernel)
            y = self.forward_normalised(Xn)
            losses.append(float(np.mean((y - T) ** 2)))
            if verbose:
                print(f"epoch {ep}: mse {losses[-1]:.4g}")
        return losses

    def params(self):
        return self.master.cpu().numpy().copy(), self.wq.float().cpu().numpy().copy()


class RSParamsC(C.Structure):
    """gpunb_rs_params (include/gpunb.h)."""
    _fields_ = [("nnbopt", C.c_int), ("nnbmax", C.c_int), ("nb_flag", C.c_int),
                ("few_nb_rule", C.c_int), ("rscale", C.c_double), ("rc", C.c_double),
                ("rsfac", C.c_double), ("bodym", C.c_double), ("rdens", C.c_double * 3),
                ("band_lo", C.c_double), ("band_hi", C.c_double),
                ("list_off", C.c_void_p), ("list", C.c_void_p), ("xj", C.c_void_p),
                ("vj", C.c_void_p)]


def rs_update_device(p, x, v, m_scaled, rs, nnb, nnb0, acc, jrk, dtr, mlp: "RSMLP | None" = None,
                     few_nb_rule: bool = True, device: int = 0, band=(0.5, 1.5), rows=None):
    """gpunb_rs_update_device on host arrays (copied to the device and back):
    the plain RS rule of `rsrule.regcor_rs` (with the few-member rule when
    few_nb_rule) and, with `mlp`, the learned proposal and its fallback, in
    one kernel.  p: rsrule.RSParams; band: acceptance band of the proposal;
    rows: (off[ni + 1], ids, xj, vj), the block's neighbour rows in CSR form
    over the j-set (xj, vj), for the band check at the next regular step
    (None: at the current density).  Returns (rs_new, target, used)."""
    import torch
    lib = load()
    fn = lib.gpunb_rs_update_device
    fn.argtypes = [C.c_int, C.POINTER(RSParamsC)] + [C.c_void_p] * 15
    fn.restype = C.c_int
    dev = torch.device("cuda", device)
    ni = len(rs)

    def d(a, dt=torch.float64):
        return torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=dev)

    keep = []
    rp = [None] * 4
    if rows is not None:
        off, ids, xj, vj = rows
        keep = [d(off, torch.int32), d(ids, torch.int32), d(xj), d(vj)]
        rp = [t.data_ptr() for t in keep]
    cp = RSParamsC(int(p.nnbopt), int(p.nnbmax), int(p.nb_flag), int(few_nb_rule),
                   float(p.rscale), float(p.rc), float(p.rsfac), float(p.bodym),
                   (C.c_double * 3)(0.0, 0.0, 0.0), float(band[0]), float(band[1]), *rp)
    X, V, M, R = d(x), d(v), d(m_scaled), d(rs)
    NB, NB0 = d(nnb, torch.int32), d(nnb0, torch.int32)
    A, J, DT = d(acc), d(jrk), d(dtr)
    out = torch.empty(ni, dtype=torch.float64, device=dev)
    tgt = torch.empty_like(out)
    used = torch.empty(ni, dtype=torch.int32, device=dev)
    if mlp is not None:
        norm = d(np.concatenate([mlp.mu, mlp.sd]).astype(np.float32), torch.float32)
        wq, wf, nm = mlp.wq.data_ptr(), mlp.master.data_ptr(), norm.data_ptr()
    else:
        wq = wf = nm = None
    torch.cuda.synchronize()
    rc = fn(ni, C.byref(cp), X.data_ptr(), V.data_ptr(), M.data_ptr(), R.data_ptr(),
            NB.data_ptr(), NB0.data_ptr(), A.data_ptr(), J.data_ptr(), DT.data_ptr(), wq, wf, nm,
            out.data_ptr(), tgt.data_ptr(), used.data_ptr(), None)
    if rc != 0:
        raise RuntimeError(f"gpunb_rs_update_device failed ({rc})")
    torch.cuda.synchronize()
    return out.cpu().numpy(), tgt.cpu().numpy(), used.cpu().numpy()
