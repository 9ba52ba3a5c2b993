"""CPU restatement of the warm-start network (test infrastructure only).

The network that gives IAS15 its learned warm start maps 32 features of a
particle's step to 21 corrections of the predicted b coefficients:

    Z1 = X W1^T + b1,  A1 = gelu(Z1)          (32 -> 256)
    Z2 = A1 W2^T + b2, A2 = gelu(Z2)          (256 -> 256)
    Y  = A2 W3^T + b3                         (256 -> 21)

gelu is the tanh form 0.5 z (1 + tanh(sqrt(2/pi) (z + 0.044715 z^3))).
The loss of a batch of B pairs is L = 1/(2B) sum_b sum_o (Y - T)^2, and
training uses Adam (beta1 0.9, beta2 0.999, eps 1e-8, bias-corrected).
Weights are stored [out][in], as the device kernels keep them.

The device kernels (forward, backward, Adam, BF16 tensor-core inference)
are checked against these functions; this module is never on the product
path.  The network has no counterpart in the reference (ASSIST uses only
IAS15's own predictor); its gradients are pinned by finite differences
(tests/test_mlp_oracle.py).
"""
from __future__ import annotations

import numpy as np

N_IN, N_HID, N_OUT = 32, 256, 21
C_GELU = np.sqrt(2.0 / np.pi)


def gelu(z):
    return 0.5 * z * (1.0 + np.tanh(C_GELU * (z + 0.044715 * z ** 3)))


def gelu_grad(z):
    u = C_GELU * (z + 0.044715 * z ** 3)
    th = np.tanh(u)
    return 0.5 * (1.0 + th) + 0.5 * z * (1.0 - th * th) * C_GELU * (1.0 + 3 * 0.044715 * z * z)


PARAM_SHAPES = [("W1", (N_HID, N_IN)), ("b1", (N_HID,)), ("W2", (N_HID, N_HID)), ("b2", (N_HID,)),
                ("W3", (N_OUT, N_HID)), ("b3", (N_OUT,))]


def n_params() -> int:
    return sum(int(np.prod(s)) for _, s in PARAM_SHAPES)


def unpack(flat):
    """Flat parameter vector (the device layout: W1, b1, W2, b2, W3, b3) -> dict."""
    out, o = {}, 0
    for name, shape in PARAM_SHAPES:
        k = int(np.prod(shape))
        out[name] = np.asarray(flat[o:o + k]).reshape(shape)
        o += k
    return out


def pack(p) -> np.ndarray:
    return np.concatenate([np.asarray(p[name]).ravel() for name, _ in PARAM_SHAPES])


def init(seed: int) -> np.ndarray:
    """He-style initial weights, zero biases, the last layer scaled down."""
    rng = np.random.default_rng(seed)
    p = {"W1": rng.standard_normal((N_HID, N_IN)) * np.sqrt(2.0 / N_IN), "b1": np.zeros(N_HID),
         "W2": rng.standard_normal((N_HID, N_HID)) * np.sqrt(2.0 / N_HID), "b2": np.zeros(N_HID),
         "W3": rng.standard_normal((N_OUT, N_HID)) * 0.1 * np.sqrt(1.0 / N_HID), "b3": np.zeros(N_OUT)}
    return pack(p)


def forward(flat, X):
    p = unpack(flat)
    Z1 = X @ p["W1"].T + p["b1"]
    A1 = gelu(Z1)
    Z2 = A1 @ p["W2"].T + p["b2"]
    A2 = gelu(Z2)
    Y = A2 @ p["W3"].T + p["b3"]
    return Y, (Z1, A1, Z2, A2)


def loss_and_grad(flat, X, T):
    """Loss 1/(2B) sum (Y - T)^2 and its gradient (flat, device layout)."""
    p = unpack(flat)
    B = X.shape[0]
    Y, (Z1, A1, Z2, A2) = forward(flat, X)
    R = Y - T
    L = 0.5 * float((R * R).sum()) / B
    dY = R / B
    g = {"W3": dY.T @ A2, "b3": dY.sum(0)}
    dZ2 = (dY @ p["W3"]) * gelu_grad(Z2)
    g["W2"] = dZ2.T @ A1
    g["b2"] = dZ2.sum(0)
    dZ1 = (dZ2 @ p["W2"]) * gelu_grad(Z1)
    g["W1"] = dZ1.T @ X
    g["b1"] = dZ1.sum(0)
    return L, pack(g)


def adam_step(flat, grad, m, v, step, lr, beta1=0.9, beta2=0.999, eps=1e-8):
    """One Adam update (step counts from 1); returns new (params, m, v)."""
    m = beta1 * m + (1 - beta1) * grad
    v = beta2 * v + (1 - beta2) * grad * grad
    mh = m / (1 - beta1 ** step)
    vh = v / (1 - beta2 ** step)
    return flat - lr * mh / (np.sqrt(vh) + eps), m, v
