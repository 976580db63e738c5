"""Learned format selector: 12 GPU-computed sparsity features -> MLP
(12 -> 64 -> 64 -> 6, FP32) -> the format a DynamicMatrix switches to.

Forward, backward and Adam run in the project's own kernels (selector.cu);
this module holds the host loop, the rule-based baseline used for the
ablation, the evaluation metrics and the versioned weights blob.

    fmt = select_format(A)                  # formats_e value for matrix A
    convert(dyn, AUTO_FORMAT)               # in-place switch to that format
"""
from __future__ import annotations

import ctypes as C
import os
import struct

import numpy as np
import torch

from . import _lib
from .analytics import NFEATURES, features

NPARAMS = 5382
NOUT = 6
AUTO_FORMAT = -1
MAGIC = b"MGBSEL01"
DEFAULT_WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "selector_weights.bin")
_LAYOUT = [("W1", (64, 12)), ("b1", (64,)), ("W2", (64, 64)), ("b2", (64,)), ("W3", (6, 64)), ("b3", (6,))]


def _vp(t: torch.Tensor | None):
    return C.c_void_p(t.data_ptr() if t is not None else 0)


def read_weights(path: str = DEFAULT_WEIGHTS) -> tuple[np.ndarray, np.ndarray, np.ndarray, dict]:
    """(params, mu, sigma, metadata) of a weights file: MAGIC, u32 version,
    u32 parameter count, u32 metadata length, mu[12], sigma[12],
    params[5382] (little-endian float32), metadata (JSON)."""
    import json
    with open(path, "rb") as f:
        if f.read(8) != MAGIC:
            raise ValueError(f"{path}: not a selector weights file")
        version, n, mlen = struct.unpack("<III", f.read(12))
        if version != 1 or n != NPARAMS:
            raise ValueError(f"{path}: unsupported version {version} / {n} parameters")
        mu = np.frombuffer(f.read(4 * NFEATURES), "<f4").copy()
        sigma = np.frombuffer(f.read(4 * NFEATURES), "<f4").copy()
        params = np.frombuffer(f.read(4 * NPARAMS), "<f4").copy()
        meta = json.loads(f.read(mlen).decode() or "{}")
    return params, mu, sigma, meta


class Selector:
    def __init__(self, params: np.ndarray, mu: np.ndarray, sigma: np.ndarray, device="cuda"):
        assert params.size == NPARAMS and mu.size == NFEATURES and sigma.size == NFEATURES
        self.device = torch.device(device)
        self.params = torch.from_numpy(np.ascontiguousarray(params, np.float32)).to(self.device)
        self.mu = torch.from_numpy(np.ascontiguousarray(mu, np.float32)).to(self.device)
        self.sigma = torch.from_numpy(np.ascontiguousarray(np.maximum(sigma, 1e-6), np.float32)).to(self.device)

    # -- construction / persistence -------------------------------------
    @classmethod
    def random(cls, mu, sigma, seed: int = 0, device="cuda") -> "Selector":
        rng = np.random.default_rng(seed)
        parts = []
        for name, shape in _LAYOUT:
            if name.startswith("W"):
                parts.append(rng.normal(0.0, np.sqrt(2.0 / shape[1]), size=shape).astype(np.float32).ravel())
            else:
                parts.append(np.zeros(shape, np.float32).ravel())
        return cls(np.concatenate(parts), mu, sigma, device)

    def save(self, path: str, meta: dict | None = None) -> None:
        import json
        m = json.dumps(meta or {}).encode()
        with open(path, "wb") as f:
            f.write(MAGIC)
            f.write(struct.pack("<III", 1, NPARAMS, len(m)))
            f.write(self.mu.cpu().numpy().astype("<f4").tobytes())
            f.write(self.sigma.cpu().numpy().astype("<f4").tobytes())
            f.write(self.params.cpu().numpy().astype("<f4").tobytes())
            f.write(m)

    @classmethod
    def load(cls, path: str = DEFAULT_WEIGHTS, device="cuda") -> "Selector":
        params, mu, sigma, _ = read_weights(path)
        return cls(params, mu, sigma, device)

    # -- network ----------------------------------------------------------
    def logp(self, X: np.ndarray, feasible: np.ndarray | None = None) -> np.ndarray:
        Xt = torch.from_numpy(np.ascontiguousarray(X, np.float32)).to(self.device)
        Ft = None if feasible is None else torch.from_numpy(np.ascontiguousarray(feasible, np.uint8)).to(self.device)
        out = torch.empty((X.shape[0], NOUT), dtype=torch.float32, device=self.device)
        _lib.call("mgb_mlp_forward_f32", _vp(self.params), _vp(self.mu), _vp(self.sigma), _vp(Xt), _vp(Ft),
                  X.shape[0], _vp(out), None)
        torch.cuda.synchronize(self.device)
        return out.cpu().numpy()

    def predict(self, X: np.ndarray, feasible: np.ndarray | None = None) -> np.ndarray:
        return np.argmax(self.logp(X, feasible), axis=1)

    def grad(self, X, labels, feasible=None):
        """Mean cross-entropy gradient and loss (device kernels)."""
        Xt = torch.from_numpy(np.ascontiguousarray(X, np.float32)).to(self.device)
        Lt = torch.from_numpy(np.ascontiguousarray(labels, np.int32)).to(self.device)
        Ft = None if feasible is None else torch.from_numpy(np.ascontiguousarray(feasible, np.uint8)).to(self.device)
        g = torch.empty(NPARAMS, dtype=torch.float32, device=self.device)
        loss = torch.empty(1, dtype=torch.float32, device=self.device)
        _lib.call("mgb_mlp_grad_f32", _vp(self.params), _vp(self.mu), _vp(self.sigma), _vp(Xt), _vp(Lt), _vp(Ft),
                  X.shape[0], _vp(g), _vp(loss), None)
        torch.cuda.synchronize(self.device)
        return g.cpu().numpy(), float(loss.item())

    def train(self, X, labels, feasible=None, epochs: int = 400, lr: float = 3e-3, batch: int = 256,
              seed: int = 0) -> list[float]:
        """Adam on mini-batches, every step on the GPU (grad + adam kernels)."""
        n = X.shape[0]
        Xd = torch.from_numpy(np.ascontiguousarray(X, np.float32)).to(self.device)
        Ld = torch.from_numpy(np.ascontiguousarray(labels, np.int32)).to(self.device)
        Fd = None if feasible is None else torch.from_numpy(np.ascontiguousarray(feasible, np.uint8)).to(self.device)
        g = torch.empty(NPARAMS, dtype=torch.float32, device=self.device)
        m = torch.zeros_like(g)
        v = torch.zeros_like(g)
        loss = torch.empty(1, dtype=torch.float32, device=self.device)
        rng = np.random.default_rng(seed)
        hist = []
        step = 0
        for _ in range(epochs):
            perm = torch.from_numpy(rng.permutation(n)).to(self.device)
            Xp, Lp = Xd[perm].contiguous(), Ld[perm].contiguous()
            Fp = None if Fd is None else Fd[perm].contiguous()
            total = 0.0
            for b0 in range(0, n, batch):
                nb = min(batch, n - b0)
                step += 1
                _lib.call("mgb_mlp_grad_f32", _vp(self.params), _vp(self.mu), _vp(self.sigma),
                          C.c_void_p(Xp.data_ptr() + 4 * 12 * b0), C.c_void_p(Lp.data_ptr() + 4 * b0),
                          C.c_void_p(Fp.data_ptr() + 6 * b0) if Fp is not None else None, nb, _vp(g),
                          _vp(loss), None)
                _lib.call("mgb_mlp_adam_f32", _vp(self.params), _vp(g), _vp(m), _vp(v), NPARAMS, lr, 0.9, 0.999,
                          1e-8, step, None)
                total += float(loss.item()) * nb
            hist.append(total / n)
        return hist


# -- rule-based baseline (the method without the network) -----------------

RULE_GRID = {
    "dia_fill_max": [0.0, 1.0, 1.1, 1.25, 1.5, 2.0, 3.0, 5.0],
    "hdc_share_min": [0.5, 0.6, 0.7, 0.8, 0.9, 0.95, 0.99, 2.0],
    "ell_fill_max": [0.0, 1.0, 1.05, 1.1, 1.25, 1.5, 2.0, 3.0],
}


def rule_select(X: np.ndarray, feasible: np.ndarray, dia_fill_max: float, hdc_share_min: float,
                ell_fill_max: float) -> np.ndarray:
    """The non-learned selector over the same GPU features: DIA if its fill
    ratio <= dia_fill_max; else HDC if the true-diagonal share of the
    nonzeros >= hdc_share_min; else ELL if its fill ratio <= ell_fill_max;
    else CSR.  Infeasible formats are never chosen."""
    dia_fill = 2.0 ** X[:, 7]
    share = X[:, 8]
    ell_fill = 2.0 ** X[:, 9]
    out = np.full(X.shape[0], 1)
    ell_ok = (ell_fill <= ell_fill_max) & (feasible[:, 3] > 0)
    out[ell_ok] = 3
    hdc_ok = (share >= hdc_share_min) & (feasible[:, 5] > 0)
    out[hdc_ok] = 5
    dia_ok = (dia_fill <= dia_fill_max) & (feasible[:, 2] > 0)
    out[dia_ok] = 2
    return out


def tune_rule(X, feasible, times) -> dict:
    """Grid-search the three thresholds for the lowest mean regret on the
    training corpus (the rule's counterpart of training)."""
    best, best_r = None, np.inf
    for t in RULE_GRID["dia_fill_max"]:
        for h in RULE_GRID["hdc_share_min"]:
            for p in RULE_GRID["ell_fill_max"]:
                r = regret(times, rule_select(X, feasible, t, h, p)).mean()
                if r < best_r:
                    best, best_r = {"dia_fill_max": t, "hdc_share_min": h, "ell_fill_max": p}, r
    return best


def regret(times: np.ndarray, choice: np.ndarray) -> np.ndarray:
    tb = times.min(axis=1)
    return times[np.arange(len(choice)), choice] / tb - 1.0


def evaluate(times: np.ndarray, choice: np.ndarray) -> dict:
    r = regret(times, choice)
    csr = times[:, 1]
    sel = times[np.arange(len(choice)), choice]
    best = times.min(axis=1)
    return {"mean_regret": float(np.mean(r)), "median_regret": float(np.median(r)),
            "p90_regret": float(np.percentile(r, 90)),
            "accuracy": float(np.mean(choice == np.argmin(times, axis=1))),
            "geomean_speedup_vs_csr": float(np.exp(np.mean(np.log(csr / sel)))),
            "total_time_speedup_vs_csr": float(csr.sum() / sel.sum()),
            "oracle_geomean_speedup_vs_csr": float(np.exp(np.mean(np.log(csr / best))))}


# -- library entry points ---------------------------------------------------

_DEFAULT = None


def default_selector() -> Selector:
    global _DEFAULT
    if _DEFAULT is None:
        _DEFAULT = Selector.load(DEFAULT_WEIGHTS)
    return _DEFAULT


def select_format(A, selector: Selector | None = None) -> int:
    """The formats_e value the selector picks for matrix A (GPU features + MLP)."""
    f, feas = features(A)
    sel = selector or default_selector()
    return int(sel.predict(f[None, :], feas[None, :])[0])
