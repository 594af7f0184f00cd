"""CPU restatement of the learned preconditioner's network, loss and gradient (TEST INFRASTRUCTURE ONLY).

The reference has no learned component (its sparse solves run in an external SLEPc process,
src/fem_problem/linalg/slepc_solve.rs:14-68), so this is the checker for the device training kernels
of fem_2d_gb300/csrc/precond.cu, written independently in FP64 numpy:

  H1 = tanh(X W1 + b1), H2 = tanh(H1 W2 + b2), Z = H2 W3 + b3         (rows = basis functions)
  per Elem patch E and sample s:  c = (Z_E^T Z_E + lam I)^-1 Z_E^T e_E
      loss_Es = (||e_E||^2 - c^T Z_E^T e_E) / ||e_E||^2
  loss = mean over patches and samples;  dloss/dZ_E = -2 (e_E - Z_E c) c^T / ||e_E||^2 / (P S)

Only tests/ may import this module.
"""
from __future__ import annotations

import numpy as np


def unpack(params, nin, hidden, k):
    p = np.asarray(params, dtype=np.float64)
    o = 0
    W1 = p[o:o + nin * hidden].reshape(nin, hidden); o += nin * hidden
    b1 = p[o:o + hidden]; o += hidden
    W2 = p[o:o + hidden * hidden].reshape(hidden, hidden); o += hidden * hidden
    b2 = p[o:o + hidden]; o += hidden
    W3 = p[o:o + hidden * k].reshape(hidden, k); o += hidden * k
    b3 = p[o:o + k]; o += k
    assert o == p.size
    return W1, b1, W2, b2, W3, b3


def forward(params, X, hidden, k):
    W1, b1, W2, b2, W3, b3 = unpack(params, X.shape[1], hidden, k)
    H1 = np.tanh(X @ W1 + b1)
    H2 = np.tanh(H1 @ W2 + b2)
    return H1, H2, H2 @ W3 + b3


def loss_grad(params, X, ptr, dof, E, hidden, k, lam=1e-6):
    """Mean projection loss and its gradient (flat, like params). E: S x ndofs."""
    X = np.asarray(X, dtype=np.float64)
    H1, H2, Z = forward(params, X, hidden, k)
    P, S = len(ptr) - 1, E.shape[0]
    scale = 1.0 / (P * S)
    dZ = np.zeros_like(Z)
    loss = 0.0
    for p in range(P):
        r0, r1 = ptr[p], ptr[p + 1]
        Zp = Z[r0:r1]
        Ep = E[:, dof[r0:r1]]                       # S x np
        G = Zp.T @ Zp + lam * np.eye(k)
        B = Ep @ Zp                                  # S x k (rows: Z^T e_s)
        C = np.linalg.solve(G, B.T).T                # S x k
        ee = np.sum(Ep * Ep, axis=1)
        ok = ee > 0
        loss += np.sum((ee[ok] - np.sum(C[ok] * B[ok], axis=1)) / ee[ok])
        R = Ep - C @ Zp.T                            # S x np
        w = np.where(ok, -2.0 / np.where(ok, ee, 1.0), 0.0) * scale
        dZ[r0:r1] = (R * w[:, None]).T @ C
    W1, b1, W2, b2, W3, b3 = unpack(params, X.shape[1], hidden, k)
    gW3 = H2.T @ dZ
    gb3 = dZ.sum(0)
    dH2 = (dZ @ W3.T) * (1 - H2 ** 2)
    gW2 = H1.T @ dH2
    gb2 = dH2.sum(0)
    dH1 = (dH2 @ W2.T) * (1 - H1 ** 2)
    gW1 = X.T @ dH1
    gb1 = dH1.sum(0)
    grad = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3])
    return loss * scale, grad


def loss_only(params, X, ptr, dof, E, hidden, k, lam=1e-6):
    return loss_grad(params, X, ptr, dof, E, hidden, k, lam)[0]
