"""Learned IAS15 warm start: pair logging, training and inference of the
network on the device (no counterpart in the reference).

A typical cycle: log (features, target) pairs from a plain run
(``collect``), train the network with the device's own forward, backward
and Adam kernels (``train``), then integrate with ``options(warm_start=1)``.
IAS15's convergence test and error estimate still judge every step; a
particle whose learned starts converge slower falls back to the plain
predictor.
"""
from __future__ import annotations

from ctypes import byref, c_double, c_void_p

import numpy as np

from ._lib import clib, last_error
from .batch import _ptr, integrate_batch_device, options

N_IN, N_OUT = 32, 21


def _check(rc: int, what: str):
    if rc != 0:
        raise RuntimeError("%s failed (%d): %s" % (what, rc, last_error()))


def n_params() -> int:
    return clib.assist_gb300_warm_n_params()


def init(seed: int = 0):
    _check(clib.assist_gb300_warm_init(seed), "assist_gb300_warm_init")


def set_params(p) -> None:
    p = np.ascontiguousarray(p, np.float32)
    _check(clib.assist_gb300_warm_set_params(p.ctypes.data_as(c_void_p), p.size), "assist_gb300_warm_set_params")


def get_params() -> np.ndarray:
    p = np.zeros(n_params(), np.float32)
    _check(clib.assist_gb300_warm_get_params(p.ctypes.data_as(c_void_p), p.size), "assist_gb300_warm_get_params")
    return p


def grad(X, T):
    """(loss, gradient) of the current network on device float32 tensors X [n,32], T [n,21]."""
    g = np.zeros(n_params(), np.float32)
    loss = c_double()
    _check(clib.assist_gb300_warm_grad(_ptr(X), _ptr(T), X.shape[0], g.ctypes.data_as(c_void_p), byref(loss)),
           "assist_gb300_warm_grad")
    return loss.value, g


def adam_step(g, lr: float):
    g = np.ascontiguousarray(g, np.float32)
    _check(clib.assist_gb300_warm_adam_step(g.ctypes.data_as(c_void_p), lr), "assist_gb300_warm_adam_step")


def train(X, T, steps: int, batch: int = 4096, lr: float = 1e-3, seed: int = 0) -> float:
    """Adam steps on random minibatches of consecutive rows (shuffle X, T first)."""
    loss = c_double()
    _check(clib.assist_gb300_warm_train(_ptr(X), _ptr(T), X.shape[0], steps, batch, lr, seed, byref(loss)),
           "assist_gb300_warm_train")
    return loss.value


def infer(X):
    """BF16 tensor-core inference (the kernel the batched IAS15 uses)."""
    import torch
    Y = torch.empty((X.shape[0], N_OUT), dtype=torch.float32, device=X.device)
    _check(clib.assist_gb300_warm_infer(_ptr(X), X.shape[0], _ptr(Y)), "assist_gb300_warm_infer")
    return Y


def collect(ephem, t0, t_end, state, params=None, capacity: int = 1 << 20, every: int = 1, opts=None):
    """Integrate once with the plain predictor and return the logged
    (features, targets) of every `every`-th accepted step (device tensors),
    plus the batch statistics."""
    import torch
    dev = state.device
    X = torch.empty((capacity, N_IN), dtype=torch.float32, device=dev)
    T = torch.empty((capacity, N_OUT), dtype=torch.float32, device=dev)
    if clib.assist_gb300_warm_n_params() <= 0:
        raise RuntimeError("warm-start network unavailable")
    _check(clib.assist_gb300_warm_set_log(_ptr(X), _ptr(T), capacity, every), "assist_gb300_warm_set_log")
    try:
        o = opts or options(group_steps=2, warm_start=0)
        st = state.clone()
        stats = integrate_batch_device(ephem, t0, t_end, st, params=params, opts=o)
        torch.cuda.synchronize()
        n = clib.assist_gb300_warm_log_count()
    finally:
        clib.assist_gb300_warm_set_log(None, None, 0, 1)
    return X[:n], T[:n], stats
