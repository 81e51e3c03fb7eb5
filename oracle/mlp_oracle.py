"""ORACLE (test infrastructure only): numpy FP64 restatement of the surrogate
network's forward pass, input gradient and the parameter gradient of the
value + input-gradient loss, used to check the library's training kernels.

The network and loss are defined in gala_gb300/csrc/gx_mlp.cuh and
gx_mlp_train.cu.  This restatement derives the parameter gradient by reverse
mode through both the forward pass and the input-gradient pass; it is itself
pinned by central finite differences of the loss (tests/test_mlp_oracle.py).
"""
from __future__ import annotations

import numpy as np

H = 256


def unpack(p, h=H):
    p = np.asarray(p, dtype=np.float64)
    o = 0
    W1 = p[o:o + 3 * h].reshape(h, 3); o += 3 * h
    b1 = p[o:o + h]; o += h
    Ws, bs = [W1], [b1]
    for _ in range(3):
        Ws.append(p[o:o + h * h].reshape(h, h)); o += h * h
        bs.append(p[o:o + h]); o += h
    w5 = p[o:o + h]; o += h
    b5 = p[o]; o += 1
    return Ws, bs, w5, b5


def silu3(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return z * s, s * (1 + z * (1 - s)), s * (1 - s) * (2 + z * (1 - 2 * s))


def forward(p, X, h=H):
    """y (B,), G = dy/dxh (B, 3) and the intermediates."""
    Ws, bs, w5, b5 = unpack(p, h)
    A, S, T = [X], [None], [None]
    for l in range(4):
        z = A[-1] @ Ws[l].T + bs[l]
        a, s1, s2 = silu3(z)
        A.append(a)
        S.append(s1)
        T.append(s2)
    y = A[4] @ w5 + b5
    D = [None] * 5
    U = [None] * 4
    D[4] = w5 * S[4]
    for l in (3, 2, 1):
        U[l] = D[l + 1] @ Ws[l]        # Ws[l] is W_{l+1} (0-based list)
        D[l] = U[l] * S[l]
    G = D[1] @ Ws[0]
    return y, G, dict(A=A, S=S, T=T, D=D, U=U, Ws=Ws, w5=w5)


def loss_and_grad(p, X, ys, Gs, alpha=1.0, beta=1.0, h=H):
    """L = alpha mean (y - y*)^2 + beta mean |G - G*|^2 and dL/dp (flat, gx_mlp.cuh order)."""
    B = X.shape[0]
    y, G, c = forward(p, X, h)
    A, S, T, D, U, Ws, w5 = c["A"], c["S"], c["T"], c["D"], c["U"], c["Ws"], c["w5"]
    L = alpha * np.mean((y - ys) ** 2) + beta * np.mean(np.sum((G - Gs) ** 2, axis=1))
    e = 2 * alpha * (y - ys) / B
    E = 2 * beta * (G - Gs) / B
    gW = [np.zeros_like(W) for W in Ws]
    gb = [np.zeros(h) for _ in range(4)]
    Zb = [None] * 5
    # adjoint of the input-gradient pass
    gW[0] += D[1].T @ E
    Dbar = E @ Ws[0].T
    for l in (1, 2, 3):
        Ubar = Dbar * S[l]
        Zb[l] = Dbar * U[l] * T[l]
        gW[l] += D[l + 1].T @ Ubar
        Dbar = Ubar @ Ws[l].T
    gw5 = np.sum(Dbar * S[4], axis=0) + A[4].T @ e
    gb5 = np.sum(e)
    Zb[4] = w5 * (Dbar * T[4] + e[:, None] * S[4])
    # ordinary backprop of the forward pass
    for l in (4, 3, 2):
        gW[l - 1] += Zb[l].T @ A[l - 1]
        gb[l - 1] += Zb[l].sum(axis=0)
        Abar = Zb[l] @ Ws[l - 1]
        Zb[l - 1] += Abar * S[l - 1]
    gW[0] += Zb[1].T @ A[0]
    gb[0] += Zb[1].sum(axis=0)
    flat = [gW[0].ravel(), gb[0]]
    for l in (1, 2, 3):
        flat += [gW[l].ravel(), gb[l]]
    flat += [gw5, np.array([gb5])]
    return L, np.concatenate(flat)
