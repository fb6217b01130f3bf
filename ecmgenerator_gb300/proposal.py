"""Learned active-set proposal for the ORCA linear program (no reference
counterpart; the LP it short-cuts is ``ORCA::RandomizedLP``, ORCA.cpp:428-587).

``ProposalModel`` wraps ``ecmg_mlp``: a 96 -> 128 -> 128 -> 160 MLP whose
inference runs in BF16 on the tensor cores inside the tick and whose training
(FP32 forward/backward, softmax cross-entropy, Adam) runs in this library's own
CUDA kernels.  ``collect_traces`` runs a simulator in trace mode and gathers
(features, class of the plain LP result) rows on the device.

Class encoding (neighbour q is the q-th nearest, constraint index nObst + q):
``CLS_PREF`` no constraint moved the initial velocity; ``CLS_SINGLE + q`` the
projection onto q's line; ``CLS_PAIR + q_hi*(q_hi-1)/2 + q_lo`` q_hi's line
bounded by q_lo's line; ``CLS_CIRCLE + q`` q's line bounded by the speed
circle; ``CLS_OTHER`` anything else (never proposed).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import EcmgError

N_IN, N_HID, N_OUT = 96, 128, 160
N_NBRS = 16
CLS_PREF, CLS_SINGLE, CLS_PAIR, CLS_CIRCLE, CLS_OTHER = 0, 1, 17, 137, 153


def param_layout():
    """(name, shape) of the parameter blocks, in the order of the flat array."""
    return [("W1", (N_IN, N_HID)), ("b1", (N_HID,)), ("W2", (N_HID, N_HID)), ("b2", (N_HID,)),
            ("W3", (N_HID, N_OUT)), ("b3", (N_OUT,))]


def split_params(flat):
    out, o = {}, 0
    for name, shp in param_layout():
        n = int(np.prod(shp))
        out[name] = np.asarray(flat[o:o + n]).reshape(shp)
        o += n
    return out


def decode_class(c: int):
    """(kind, q, q_lo): kind in {'pref', 'single', 'pair', 'circle', 'other'}."""
    if c == CLS_PREF:
        return ("pref", -1, -1)
    if CLS_SINGLE <= c < CLS_PAIR:
        return ("single", c - CLS_SINGLE, -1)
    if CLS_PAIR <= c < CLS_CIRCLE:
        p = c - CLS_PAIR
        q = 1
        while (q + 1) * q // 2 <= p:
            q += 1
        return ("pair", q, p - q * (q - 1) // 2)
    if CLS_CIRCLE <= c < CLS_OTHER:
        return ("circle", c - CLS_CIRCLE, -1)
    return ("other", -1, -1)


def _dptr(t) -> int:
    """device pointer of a CUDA tensor (torch is used for device memory only)"""
    if not t.is_cuda or not t.is_contiguous():
        raise ValueError("expected a contiguous CUDA tensor")
    return t.data_ptr()


class ProposalModel:
    """ecmg_mlp: parameters live on the GPU in FP32; the tick uses BF16 copies."""

    def __init__(self, seed: int = 0):
        self.L = _lib.load()
        h = C.c_void_p()
        rc = self.L.ecmg_mlp_create(C.c_ulonglong(seed), C.byref(h))
        if rc:
            raise EcmgError(rc, "ecmg_mlp_create failed (is a CUDA device visible?)")
        self.h = h
        self.n_params = int(self.L.ecmg_mlp_param_count())

    def close(self):
        if getattr(self, "h", None):
            self.L.ecmg_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, rc, what):
        if rc:
            raise EcmgError(rc, what)

    def get_params(self) -> np.ndarray:
        out = np.zeros(self.n_params, np.float32)
        self._ck(self.L.ecmg_mlp_get_params(self.h, out.ctypes.data), "ecmg_mlp_get_params")
        return out

    def set_params(self, flat):
        flat = np.ascontiguousarray(flat, np.float32)
        if flat.size != self.n_params:
            raise ValueError(f"expected {self.n_params} parameters, got {flat.size}")
        self._ck(self.L.ecmg_mlp_set_params(self.h, flat.ctypes.data), "ecmg_mlp_set_params")

    def save(self, path):
        np.save(path, self.get_params())

    def load(self, path):
        self.set_params(np.load(path))

    def loss_grad(self, x, y):
        """mean cross-entropy and its gradient over all rows; x: CUDA bf16
        [n, 96], y: CUDA uint8 [n]"""
        n = int(x.shape[0])
        loss = C.c_float()
        g = np.zeros(self.n_params, np.float32)
        self._ck(self.L.ecmg_mlp_loss_grad(self.h, _dptr(x), _dptr(y), n, C.byref(loss), g.ctypes.data),
                 "ecmg_mlp_loss_grad")
        return float(loss.value), g

    def train(self, x, y, steps: int, batch: int = 65536, lr: float = 1e-3, seed: int = 1, log: bool = True):
        """Adam on minibatches drawn from the rows of (x, y); returns per-step
        loss and accuracy (host arrays) when log is set"""
        n = int(x.shape[0])
        loss = np.zeros(steps, np.float32) if log else None
        acc = np.zeros(steps, np.float32) if log else None
        self._ck(self.L.ecmg_mlp_train(self.h, _dptr(x), _dptr(y), n, int(steps), int(batch), float(lr),
                                       C.c_ulonglong(seed), loss.ctypes.data if log else None,
                                       acc.ctypes.data if log else None), "ecmg_mlp_train")
        return loss, acc

    def predict(self, x):
        import torch
        n = int(x.shape[0])
        out = torch.empty(n, dtype=torch.uint8, device=x.device)
        self._ck(self.L.ecmg_mlp_predict(self.h, _dptr(x), n, _dptr(out) if n else None), "ecmg_mlp_predict")
        return out


def collect_traces(sim, ticks: int, every: int = 1, max_rows: int | None = None):
    """Run `ticks` ticks of `sim` in trace mode and keep the rows of every
    `every`-th tick: returns CUDA tensors (features bf16 [n, 96], labels
    uint8 [n]).  Rows of agents removed during their tick (zero features,
    CLS_OTHER) are dropped."""
    import torch
    sim.set_trace(True)
    xs, ys = [], []
    total = 0
    try:
        for t in range(ticks):
            sim.update()
            if t % every:
                continue
            x, y, _ = sim.get_trace(device=True)
            keep = (x.view(torch.int16) != 0).any(dim=1) | (y != CLS_OTHER)
            x, y = x[keep], y[keep]
            xs.append(x)
            ys.append(y)
            total += int(x.shape[0])
            if max_rows is not None and total >= max_rows:
                break
    finally:
        sim.set_trace(False)
    x = torch.cat(xs) if xs else torch.empty((0, N_IN), dtype=torch.bfloat16, device="cuda")
    y = torch.cat(ys) if ys else torch.empty((0,), dtype=torch.uint8, device="cuda")
    if max_rows is not None:
        x, y = x[:max_rows].contiguous(), y[:max_rows].contiguous()
    return x, y


def class_histogram(y) -> dict:
    """share of each class kind in a label array (numpy or torch)"""
    y = np.asarray(y.cpu() if hasattr(y, "cpu") else y).astype(np.int64)
    n = max(1, y.size)
    kinds = {"pref": 0, "single": 0, "pair": 0, "circle": 0, "other": 0}
    kinds["pref"] = int((y == CLS_PREF).sum())
    kinds["single"] = int(((y >= CLS_SINGLE) & (y < CLS_PAIR)).sum())
    kinds["pair"] = int(((y >= CLS_PAIR) & (y < CLS_CIRCLE)).sum())
    kinds["circle"] = int(((y >= CLS_CIRCLE) & (y < CLS_OTHER)).sum())
    kinds["other"] = int((y >= CLS_OTHER).sum())
    return {k: v / n for k, v in kinds.items()}
