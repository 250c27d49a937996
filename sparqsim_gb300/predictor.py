"""The learned output-size model of the split operators (csrc/predictor.cu).

Typical use: log sizes while running representative circuits, train on the
GPU, then enable predictions. Results of every operator are identical with
the model on or off; only which sizing path runs changes.

    from sparqsim_gb300 import predictor
    predictor.log(True)
    ... run circuits ...
    x, t = predictor.read_log()
    predictor.reset(seed=1)
    loss = predictor.train(x, t, epochs=200)
    predictor.enable(True)
"""
from __future__ import annotations

from ctypes import byref, c_float, c_uint64, c_void_p

import numpy as np

from ._native import call

FEATURES = 48
HIDDEN = 64
OUTPUTS = 2
PARAMS = FEATURES * HIDDEN + HIDDEN + HIDDEN * HIDDEN + HIDDEN + HIDDEN * OUTPUTS + OUTPUTS


def _f32(a, cols):
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float32))
    if a.ndim != 2 or a.shape[1] != cols:
        raise ValueError(f"expected an array of shape (n, {cols})")
    return a


def reset(seed: int = 0) -> None:
    """He-initialised weights, zero biases, fresh Adam state; predictions off until trained."""
    call("sq_predictor_reset", int(seed))


def get_params() -> np.ndarray:
    out = np.zeros(PARAMS, dtype=np.float32)
    call("sq_predictor_get_params", out.ctypes.data_as(c_void_p), PARAMS)
    return out


def set_params(p) -> None:
    p = np.ascontiguousarray(np.asarray(p, dtype=np.float32).reshape(-1))
    call("sq_predictor_set_params", p.ctypes.data_as(c_void_p), p.size)


def gradient(x, t):
    """(mean squared error, gradient) over rows (x, t); parameters unchanged."""
    x, t = _f32(x, FEATURES), _f32(t, OUTPUTS)
    g = np.zeros(PARAMS, dtype=np.float32)
    loss = c_float()
    call("sq_predictor_gradient", x.ctypes.data_as(c_void_p), t.ctypes.data_as(c_void_p), x.shape[0],
         g.ctypes.data_as(c_void_p), byref(loss))
    return float(loss.value), g


def predict(x) -> np.ndarray:
    x = _f32(x, FEATURES)
    y = np.zeros((x.shape[0], OUTPUTS), dtype=np.float32)
    call("sq_predictor_predict", x.ctypes.data_as(c_void_p), x.shape[0], y.ctypes.data_as(c_void_p))
    return y


def train(x, t, epochs: int = 100, batch: int = 256, lr: float = 1e-3, seed: int = 0) -> float:
    """Adam on the GPU; returns the loss of the last minibatch."""
    x, t = _f32(x, FEATURES), _f32(t, OUTPUTS)
    loss = c_float()
    call("sq_predictor_train", x.ctypes.data_as(c_void_p), t.ctypes.data_as(c_void_p), x.shape[0], int(epochs),
         int(batch), float(lr), int(seed), byref(loss))
    return float(loss.value)


def enable(on: bool = True) -> None:
    call("sq_predictor_enable", 1 if on else 0)


def log(on: bool = True) -> None:
    call("sq_predictor_log_enable", 1 if on else 0)


def read_log():
    n = c_uint64()
    call("sq_predictor_log_size", byref(n))
    x = np.zeros((n.value, FEATURES), dtype=np.float32)
    t = np.zeros((n.value, OUTPUTS), dtype=np.float32)
    got = c_uint64()
    call("sq_predictor_log_read", x.ctypes.data_as(c_void_p), t.ctypes.data_as(c_void_p), n.value, byref(got))
    return x[: got.value], t[: got.value]


def clear_log() -> None:
    call("sq_predictor_log_clear")


def stats() -> dict:
    p, o = c_uint64(), c_uint64()
    call("sq_predictor_stats", byref(p), byref(o))
    return {"predictions": p.value, "single_pass_overflows": o.value}


def set_hash_groups_hint(groups: int) -> None:
    """Groups the hash table is sized for when no prediction is made (0: default 2^20)."""
    call("sq_set_hash_groups_hint", int(groups))


def set_single_pass_limit(entries: int) -> None:
    """Output entries a single-pass split may allocate by its fully populated
    bound; 0 restores the default max(4 N, 2^27)."""
    call("sq_set_single_pass_limit", int(entries))
