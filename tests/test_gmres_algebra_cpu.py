"""The algebra of the fused GMRES cycle (omega2d_gb300/csrc/gmres.cu, gmres_cycle_kernel),
restated in FP64 numpy and checked against the textbook steps it replaces (the Krylov method of
src/BEM.h:169-234).  CPU only: these pin the formulas; the GPU tests pin the kernel against
FP64 solves.

* Second Gram-Schmidt pass from the basis' Gram matrix G = V^T V: with c = V^T w, the two
  classical passes give h = c + V^T (w - V c) = 2 c - G c, and ||w - V h||^2 = w.w - 2 h.c +
  h^T G h holds for any h.
* Givens rotations of a Hessenberg column as the affine recurrence x_{k+1} = -s_k x_k +
  c_k h_{k+1} (x_0 = h_0), scanned over a warp of 32 lanes holding two rotations each."""
import numpy as np
import pytest


def perturbed_basis(rng, n, k, eps):
    q, _ = np.linalg.qr(rng.normal(size=(n, k)))
    return q + eps * rng.normal(size=(n, k))


@pytest.mark.parametrize("eps", [0.0, 1e-9, 1e-6])
def test_gram_second_pass_matches_two_classical_passes(eps):
    """Exact for an orthonormal basis; for a basis that lost orthogonality by eps, the Gram
    form's coefficients differ from the two explicit passes by O(eps^2) of |c|, and the norm
    identity is exact for any h."""
    rng = np.random.default_rng(5)
    n, k = 4096, 36
    V = perturbed_basis(rng, n, k, eps)
    w = rng.normal(size=n)
    # two classical Gram-Schmidt passes, as the per-step kernels do them
    c1 = V.T @ w
    w1 = w - V @ c1
    c2 = V.T @ w1
    h_cgs2 = c1 + c2
    # the cycle kernel: one reduction gives c and the Gram column, then h = 2c - Gc
    G = V.T @ V
    c = V.T @ w
    h = 2.0 * c - G @ c
    assert np.max(np.abs(h - h_cgs2)) <= 1e-13 * np.max(np.abs(c)) + 50.0 * eps ** 2 * np.max(np.abs(c)) * k
    nrm2_direct = float(np.dot(w - V @ h, w - V @ h))
    nrm2_gram = float(np.dot(w, w) - 2.0 * np.dot(h, c) + h @ G @ h)
    assert abs(nrm2_gram - nrm2_direct) <= 1e-10 * np.dot(w, w)


def rotations_sequential(h, cs, sn):
    """The earlier rotations applied one after another (the per-step givens_kernel)."""
    h = h.copy()
    for k in range(len(cs)):
        t = cs[k] * h[k] + sn[k] * h[k + 1]
        h[k + 1] = -sn[k] * h[k] + cs[k] * h[k + 1]
        h[k] = t
    return h


def rotations_warp_scan(h, cs, sn):
    """The cycle kernel's form: lane l holds rotations 2l and 2l+1 as affine maps
    f_k(x) = -s_k x + c_k h_{k+1}; an inclusive Hillis-Steele scan of their composition over
    the 32 lanes, the exclusive prefix applied to x_0 = h_0, then h_k = c_k x_k + s_k h_{k+1}."""
    K = len(cs)
    lanes = 32
    c = np.ones(2 * lanes)
    s = np.zeros(2 * lanes)
    hp = np.zeros(2 * lanes)
    c[:K], s[:K], hp[:K] = cs, sn, h[1:K + 1]
    a, b = -s, c * hp
    a0, b0, a1, b1 = a[0::2], b[0::2], a[1::2], b[1::2]
    Ac, Bc = a1 * a0, a1 * b0 + b1                      # f_{2l+1} o f_{2l}
    o = 1
    while o < lanes:
        Ap, Bp = np.roll(Ac, o), np.roll(Bc, o)
        m = np.arange(lanes) >= o
        Bc = np.where(m, Ac * Bp + Bc, Bc)
        Ac = np.where(m, Ac * Ap, Ac)
        o *= 2
    Ae, Be = np.roll(Ac, 1), np.roll(Bc, 1)
    Ae[0], Be[0] = 1.0, 0.0
    x = np.empty(2 * lanes + 1)
    x[0::2][:lanes] = Ae * h[0] + Be                   # x_{2l}
    x[1::2][:lanes] = a0 * x[0::2][:lanes] + b0        # x_{2l+1}
    x[2 * lanes] = a1[-1] * x[2 * lanes - 1] + b1[-1]
    out = h.copy()
    out[:K] = c[:K] * x[:K] + s[:K] * hp[:K]
    out[K] = x[K]
    return out


@pytest.mark.parametrize("K", [0, 1, 2, 7, 31, 32, 33, 63, 64])
def test_givens_warp_scan_matches_sequential_rotations(K):
    rng = np.random.default_rng(100 + K)
    h = rng.normal(size=K + 2)
    th = rng.uniform(0, 2 * np.pi, K)
    cs, sn = np.cos(th), np.sin(th)
    ref = rotations_sequential(h, cs, sn)
    got = rotations_warp_scan(h, cs, sn)
    assert np.max(np.abs(got[:K + 1] - ref[:K + 1])) <= 1e-12 * np.max(np.abs(h))
