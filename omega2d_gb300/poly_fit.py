"""Coefficients of the polynomial arctangent used by the panel kernels (csrc/panels.cu).

atan(r) on [0, 1] is written r * P(r^2) with P of degree 8.  P is fitted to atan(r)/r for
minimum maximum RELATIVE error (so that small angles -- distant panels -- keep full relative
accuracy) by Lawson's iteratively reweighted least squares on 20,001 Chebyshev-spaced nodes,
then rounded to FP32.  Run ``python -m omega2d_gb300.poly_fit`` to reproduce the table and its
error in FP32 Horner evaluation (fused multiply-adds emulated in FP64 and rounded per step).
"""
from __future__ import annotations

import numpy as np


def fit_atan(degree: int = 8, iters: int = 300) -> tuple[np.ndarray, float]:
    K = degree + 1
    t = (1.0 - np.cos(np.linspace(0.0, np.pi, 20001))) / 2.0
    r = np.sqrt(t)
    f = np.ones_like(t)
    f[1:] = np.arctan(r[1:]) / r[1:]
    V = np.vander(t, K, increasing=True)
    w = np.ones_like(t)
    for _ in range(iters):
        sw = np.sqrt(w)
        c, *_ = np.linalg.lstsq(V * sw[:, None], f * sw, rcond=None)
        e = np.abs(V @ c - f) / f
        w = w * (e + 1e-30)
        w /= w.sum()
    return c.astype(np.float32), float(np.max(np.abs(V @ c - f) / f))


def fp32_error(c32: np.ndarray, n: int = 2_000_001) -> float:
    r = np.linspace(0.0, 1.0, n).astype(np.float32)
    t = (r * r).astype(np.float32)
    p = np.full_like(t, c32[-1])
    for k in range(len(c32) - 2, -1, -1):
        p = (p.astype(np.float64) * t.astype(np.float64) + np.float64(c32[k])).astype(np.float32)
    val = (r * p).astype(np.float64)
    ref = np.arctan(r.astype(np.float64))
    return float(np.max(np.abs(val[1:] - ref[1:]) / ref[1:]))


if __name__ == "__main__":
    c, e = fit_atan()
    print("coefficients (t^0 .. t^8):", ", ".join(f"{float(x):.9e}f" for x in c))
    print(f"fit relative error {e:.3g}; FP32 evaluation relative error {fp32_error(c):.3g}")
