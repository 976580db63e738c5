"""FP64 NumPy restatement of the selector network (TEST INFRASTRUCTURE ONLY).

Same parameter layout as morpheus_gb300/csrc/selector.cu: W1[64][12], b1[64],
W2[64][64], b2[64], W3[6][64], b3[6]; inputs standardised as (x - mu)/sigma;
ReLU hidden layers; softmax over the feasible outputs; mean cross-entropy.
Used to check the GPU forward pass and gradients.
"""
from __future__ import annotations

import numpy as np

LAYOUT = [("W1", (64, 12)), ("b1", (64,)), ("W2", (64, 64)), ("b2", (64,)), ("W3", (6, 64)), ("b3", (6,))]


def unpack(p: np.ndarray) -> dict:
    out, o = {}, 0
    for name, shape in LAYOUT:
        n = int(np.prod(shape))
        out[name] = p[o:o + n].reshape(shape).astype(np.float64)
        o += n
    return out


def forward(p, mu, sigma, X, feasible=None):
    P = unpack(np.asarray(p, np.float64))
    xn = (X.astype(np.float64) - mu) / sigma
    z1 = xn @ P["W1"].T + P["b1"]
    h1 = np.maximum(z1, 0)
    z2 = h1 @ P["W2"].T + P["b2"]
    h2 = np.maximum(z2, 0)
    z3 = h2 @ P["W3"].T + P["b3"]
    if feasible is not None:
        z3 = np.where(feasible > 0, z3, -np.inf)
    zmax = z3.max(axis=1, keepdims=True)
    e = np.exp(z3 - zmax)
    prob = e / e.sum(axis=1, keepdims=True)
    return {"xn": xn, "z1": z1, "h1": h1, "z2": z2, "h2": h2, "p": prob}


def grad(p, mu, sigma, X, labels, feasible=None):
    """(mean gradient in the flat layout, mean loss)."""
    P = unpack(np.asarray(p, np.float64))
    a = forward(p, mu, sigma, X, feasible)
    n = X.shape[0]
    loss = -np.mean(np.log(np.maximum(a["p"][np.arange(n), labels], 1e-300)))
    dz3 = a["p"].copy()
    dz3[np.arange(n), labels] -= 1.0
    g = {"W3": dz3.T @ a["h2"], "b3": dz3.sum(0)}
    dz2 = (dz3 @ P["W3"]) * (a["z2"] > 0)
    g["W2"], g["b2"] = dz2.T @ a["h1"], dz2.sum(0)
    dz1 = (dz2 @ P["W2"]) * (a["z1"] > 0)
    g["W1"], g["b1"] = dz1.T @ a["xn"], dz1.sum(0)
    flat = np.concatenate([g[name].ravel() for name, _ in LAYOUT]) / n
    return flat, loss
