"""Learned warm start: a 1D-conv network trained on converged fields that the
solver itself generates, then used to initialise new instances.

The network, its training and its inference are GPU kernels behind the C ABI
(scft_ws_*); this module orchestrates dataset generation, training, saving and
evaluation.  Every warm-started instance is still converged by the plain mixing
loop to the same tolerance.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _lib as L
from . import api
from ._lib import check

GRID = 256
FEATURES = 5
DEFAULT_WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights", "warmstart_w0.npz")


def _fp(a):
    assert a.dtype == np.float32 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_float))


class WarmStart:
    def __init__(self, bf16: bool = True, seed: int = 0):
        self.lib = L.load()
        h = C.c_void_p()
        check(self.lib.scft_ws_create(int(bf16), C.c_ulonglong(seed), C.byref(h)), "scft_ws_create")
        self.h = h
        self.nparam = check(self.lib.scft_ws_param_count(h), "scft_ws_param_count")

    # parameters
    def params(self) -> np.ndarray:
        p = np.empty(self.nparam, dtype=np.float32)
        check(self.lib.scft_ws_get_params(self.h, _fp(p)), "scft_ws_get_params")
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        if p.size != self.nparam:
            raise ValueError(f"expected {self.nparam} parameters, got {p.size}")
        check(self.lib.scft_ws_set_params(self.h, _fp(p)), "scft_ws_set_params")

    def save(self, path=DEFAULT_WEIGHTS, **meta):
        os.makedirs(os.path.dirname(path), exist_ok=True)
        np.savez(path, params=self.params(), **{k: np.asarray(v) for k, v in meta.items()})

    def load(self, path=DEFAULT_WEIGHTS):
        self.set_params(np.load(path)["params"])

    # raw network calls (host buffers)
    def forward(self, features: np.ndarray) -> np.ndarray:
        f = np.ascontiguousarray(features, dtype=np.float32)
        B = f.shape[0]
        out = np.empty((B, GRID), dtype=np.float32)
        check(self.lib.scft_ws_forward(self.h, _fp(f), B, _fp(out)), "scft_ws_forward")
        return out

    def loss_grad(self, features, targets):
        f = np.ascontiguousarray(features, dtype=np.float32)
        t = np.ascontiguousarray(targets, dtype=np.float32)
        g = np.empty(self.nparam, dtype=np.float32)
        loss = C.c_double()
        check(self.lib.scft_ws_loss_grad(self.h, _fp(f), _fp(t), f.shape[0], C.byref(loss), _fp(g)),
              "scft_ws_loss_grad")
        return loss.value, g

    # batches
    def add_dataset(self, batch: api.Batch, mask=None) -> int:
        m = None if mask is None else (C.c_int * batch.count)(*[int(bool(v)) for v in mask])
        return check(self.lib.scft_ws_dataset_from_batch(self.h, batch.h, m), "scft_ws_dataset_from_batch")

    def train(self, steps=3000, batch=256, lr=2e-3, seed=0) -> np.ndarray:
        losses = np.empty(steps, dtype=np.float32)
        check(self.lib.scft_ws_train(self.h, int(steps), int(batch), C.c_float(lr), C.c_ulonglong(seed),
                                     _fp(losses)), "scft_ws_train")
        return losses

    def set_tensor_cores(self, on: bool) -> bool:
        """BF16 networks: the 64 -> 64 layers on the tensor cores (default) or on
        the CUDA cores; returns the previous setting."""
        return bool(check(self.lib.scft_ws_set_tensor_cores(self.h, int(bool(on))), "scft_ws_set_tensor_cores"))

    def tensor_core_status(self) -> int:
        """0, or the code of a bounded wait of the tensor-core layers that ran out."""
        return check(self.lib.scft_ws_tensor_core_status(self.h), "scft_ws_tensor_core_status")

    def predict(self, batch: api.Batch):
        check(self.lib.scft_ws_predict(self.h, batch.h), "scft_ws_predict")

    def close(self):
        if getattr(self, "h", None):
            self.lib.scft_ws_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def batch_features(batch: api.Batch, with_targets=True):
    lib = L.load()
    f = np.empty((batch.count, FEATURES, GRID), dtype=np.float32)
    t = np.empty((batch.count, GRID), dtype=np.float32) if with_targets else None
    check(lib.scft_ws_batch_features(batch.h, _fp(f), None if t is None else _fp(t)), "scft_ws_batch_features")
    return f, t


def generate_and_train(train_instances, steps=3000, batch=256, lr=2e-3, seed=0, tol=1e-6, bf16=True,
                       chunk=4096, log=None):
    """Solve the training instances (cold start, FP32 propagator, FP64 mixing),
    keep the converged fields as targets, and train a network on them."""
    ws = WarmStart(bf16=bf16, seed=seed)
    stats = {"solved": 0, "total": 0}
    for i0 in range(0, len(train_instances), chunk):
        part = train_instances[i0:i0 + chunk]
        with api.Batch(part) as b:
            r = b.solve(precision=L.F32, tol=tol)
            ok = (r["status"] & L.ST_CONVERGED) != 0
            stats["solved"] += int(ok.sum())
            stats["total"] += len(part)
            ws.add_dataset(b, ok)
        if log:
            log(f"training fields: {stats['solved']}/{stats['total']} converged")
    losses = ws.train(steps=steps, batch=batch, lr=lr, seed=seed)
    stats["final_loss"] = float(np.mean(losses[-50:]))
    return ws, losses, stats
