"""Learned column-line preconditioner: Python side of the C ABI.

The network and its kernels live in ``csrc/learned.cu``; this module holds
the parameter layout, a seeded initialiser, and a thin handle class around
``cathy_gb300_lp_*`` for training and evaluation on explicit graphs.  The
reference CATHY has no learned component; the preconditioner it augments is
the Picard linear solve (SYMSLV, solscal-extended.f:4669), which the GPU
engine runs as PCG with a column-line factor.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np

from . import _lib
from ._lib import check, f32p, f64p, i32p, u8p

NF, HID = 16, 64
NPARAMS = HID * NF + HID + HID * HID + HID + HID + 1
NPAIRS = 4
ORDER = (("W1", (HID, NF)), ("b1", (HID,)), ("W2", (HID, HID)), ("b2", (HID,)),
         ("w3", (HID,)), ("b3", (1,)))


def init_params(seed: int = 0, b3: float = 0.0) -> np.ndarray:
    """He-style seeded initialisation with a small output layer, so that
    omega = tanh(o) ~ 0: the untrained network reproduces the plain
    column-line preconditioner."""
    rng = np.random.default_rng(seed)
    W1 = np.zeros((HID, NF))
    W1[:, :8] = rng.standard_normal((HID, 8)) * np.sqrt(2.0 / 8)
    W2 = rng.standard_normal((HID, HID)) * np.sqrt(2.0 / HID)
    w3 = rng.standard_normal(HID) * 0.1 / np.sqrt(HID)
    parts = [W1, np.zeros(HID), W2, np.zeros(HID), w3, np.array([b3])]
    return np.concatenate([p.ravel() for p in parts]).astype(np.float32)


def split(vec) -> dict:
    out, o = {}, 0
    for k, shp in ORDER:
        sz = int(np.prod(shp))
        out[k] = np.asarray(vec[o:o + sz], np.float32).reshape(shp)
        o += sz
    return out


def _p(a, t):
    return a.ctypes.data_as(t)


class LearnedPreconditioner:
    """Device-resident model (fp32 master weights, Adam state, bf16 copies)."""

    def __init__(self, params: Optional[np.ndarray] = None, device: int = 0, lr: float = 1e-3):
        L = _lib.load()
        self._L = L
        self.h = C.c_void_p()
        p = None if params is None else np.ascontiguousarray(params, np.float32)
        if p is not None and p.size != NPARAMS:
            raise ValueError(f"expected {NPARAMS} parameters, got {p.size}")
        self._keep = p
        check(L.cathy_gb300_lp_create(None if p is None else _p(p, f32p), device,
                                      C.byref(self.h)), "cathy_gb300_lp_create")
        self.set_lr(lr)

    def close(self):
        if self.h:
            self._L.cathy_gb300_lp_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def handle(self):
        return self.h

    def params(self) -> np.ndarray:
        out = np.zeros(NPARAMS, np.float32)
        check(self._L.cathy_gb300_lp_params(self.h, _p(out, f32p), None, 0.0, None),
              "cathy_gb300_lp_params")
        return out

    def set_params(self, vec):
        v = np.ascontiguousarray(vec, np.float32)
        check(self._L.cathy_gb300_lp_params(self.h, None, _p(v, f32p), 0.0, None),
              "cathy_gb300_lp_params")

    def set_lr(self, lr: float):
        check(self._L.cathy_gb300_lp_params(self.h, None, None, float(lr), None),
              "cathy_gb300_lp_params")

    def steps(self) -> int:
        s = C.c_int64()
        check(self._L.cathy_gb300_lp_params(self.h, None, None, 0.0, C.byref(s)),
              "cathy_gb300_lp_params")
        return int(s.value)

    def eval(self, graph: dict, pairs=(), train_steps: int = 0):
        """Loss, network outputs and gradients on one graph.

        ``graph``: rowptr, cols (0-based full CSR), vals, dmask, nnod, ks,
        pnodi, et2, dt.  ``pairs``: up to 4 (p, q) Krylov pairs.
        Returns dict(loss, dprime, omega, grads)."""
        rp = np.ascontiguousarray(graph["rowptr"], np.int32)
        cl = np.ascontiguousarray(graph["cols"], np.int32)
        va = np.ascontiguousarray(graph["vals"], np.float32)
        dm = np.ascontiguousarray(graph["dmask"], np.uint8)
        ks = np.ascontiguousarray(graph["ks"], np.float32)
        pn = np.ascontiguousarray(graph["pnodi"], np.float32)
        e2 = np.ascontiguousarray(graph["et2"], np.float32)
        n = len(rp) - 1
        npairs = len(pairs)
        if npairs > NPAIRS:
            raise ValueError("at most 4 Krylov pairs")
        P = np.ascontiguousarray(np.array([p for p, _ in pairs], np.float32).reshape(npairs, n))
        Q = np.ascontiguousarray(np.array([q for _, q in pairs], np.float32).reshape(npairs, n))
        loss = C.c_double()
        dprime = np.zeros(n, np.float32)
        omega = np.zeros(len(cl), np.float32)
        grads = np.zeros(NPARAMS, np.float32)
        check(self._L.cathy_gb300_lp_eval(
            self.h, n, int(graph["nnod"]), _p(rp, i32p), _p(cl, i32p), _p(va, f32p),
            _p(dm, u8p), _p(ks, f32p), _p(pn, f32p), _p(e2, f32p), float(graph["dt"]), npairs,
            _p(P, f32p) if npairs else None, _p(Q, f32p) if npairs else None, int(train_steps),
            C.byref(loss), _p(dprime, f32p), _p(omega, f32p), _p(grads, f32p)),
            "cathy_gb300_lp_eval")
        return dict(loss=loss.value, dprime=dprime, omega=omega, grads=grads)
