"""FP64 restatement of the device conjugate-gradient recurrence (TEST
INFRASTRUCTURE ONLY).  Same sequence of operations as
morpheus_gb300/csrc/solver.cu: r = b - A x, p = r; per iteration
alpha = r.r / p.Ap, x += alpha p, r -= alpha Ap, beta = r.r_new / r.r,
p = r + beta p; stop when r.r <= rtol^2 b.b or after max_iters.  A*p is the
oracle's Serial multiply (restating the reference,
core/src/impl/Csr/Serial/Morpheus_Multiply_Impl.hpp:38-58)."""
from __future__ import annotations

import numpy as np

from . import oracle as O


def cg(hm: dict, b: np.ndarray, x0: np.ndarray, max_iters: int, rtol: float):
    A = O.OracleMatrix.from_host(hm)
    x = x0.astype(np.float64).copy()
    r = b - A.multiply(x)
    p = r.copy()
    rr = float(r @ r)
    bb = float(b @ b)
    it = 0
    while it < max_iters and rr > rtol * rtol * bb:
        ap = A.multiply(p)
        pap = float(p @ ap)
        if not pap > 0:
            raise ArithmeticError("p.Ap <= 0: matrix is not SPD")
        alpha = rr / pap
        x += alpha * p
        r -= alpha * ap
        rr_new = float(r @ r)
        beta = rr_new / rr
        rr = rr_new
        p = r + beta * p
        it += 1
    return x, it, float(np.sqrt(rr / bb)) if bb > 0 else float(np.sqrt(rr))
