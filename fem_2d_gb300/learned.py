"""Inner PCG solver of the shifted pencil and its learned per-Elem-patch preconditioner.

The reference solves its sparse eigenproblem in an external SLEPc process whose inner KSP solves are
configured there (src/fem_problem/linalg/slepc_solve.rs:14-68); it has no preconditioner of its own.
This module is the device inner solver for SPD shifts K = c_a A + c_b B:

* ``PCG(gep, c_a, c_b)``: conjugate gradients with the plain preconditioner, additive Schwarz over Elem
  patches (exact inverses of each Elem's diagonal block of K);
* ``PCG(gep, c_a, c_b, net)``: the same plus a two-level coarse correction whose coarse basis the
  ``PatchNet`` produces: for every basis function of an Elem, an MLP (16 -> hidden -> hidden -> k, tanh,
  FP32) maps geometric/polynomial features to k coefficients, giving k coarse vectors per Elem.

``PatchNet.train`` fits the network on the GPU with the library's own forward, backward and Adam kernels
to error vectors that the plain solver produces (``harvest_errors``): the loss is the mean over Elems
and samples of ||e_E - Z_E c*||^2 / ||e_E||^2, the relative distance of each Elem's restriction of the
error from the span of its k vectors.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import Context, Fem2dError, _check, _ptr, lib

_FP = ctypes.POINTER(ctypes.c_float)
_DP = ctypes.POINTER(ctypes.c_double)


class PatchNet:
    """The per-Elem-patch coarse-basis network (parameters live on the host between calls)."""

    def __init__(self, k=16, hidden=192, seed=0):
        h = ctypes.c_void_p()
        _check(lib().fem2d_patchnet_create(int(k), int(hidden), int(seed), ctypes.byref(h)))
        self._h = h
        self.k, self.hidden = k, hidden

    def __del__(self):
        try:
            from . import _lib
        except ImportError:   # interpreter shutdown: the library goes away with the process
            return
        if getattr(self, "_h", None) and _lib is not None:
            _lib.fem2d_patchnet_free(self._h)
            self._h = None

    @property
    def num_params(self):
        return lib().fem2d_patchnet_num_params(self._h)

    def get_params(self):
        out = np.zeros(self.num_params, np.float32)
        _check(lib().fem2d_patchnet_get_params(self._h, out.ctypes.data_as(_FP)))
        return out

    def set_params(self, params):
        p = np.ascontiguousarray(params, dtype=np.float32)
        if p.size != self.num_params:
            raise Fem2dError(1, "parameter count mismatch")
        _check(lib().fem2d_patchnet_set_params(self._h, p.ctypes.data_as(_FP)))

    def loss_grad(self, gep, shift, samples, ctx=None):
        """Mean projection loss on one GEP for samples (S x ndofs) and its parameter gradient (GPU)."""
        ctx = ctx or gep.ctx
        E = np.ascontiguousarray(samples, dtype=np.float64)
        loss = ctypes.c_double()
        grad = np.zeros(self.num_params, np.float32)
        _check(lib().fem2d_patchnet_loss_grad(ctx._h, self._h, gep._h, float(shift), _ptr(E, ctypes.c_double),
                                              E.shape[0], ctypes.byref(loss), grad.ctypes.data_as(_FP)))
        return loss.value, grad

    def train(self, geps, shift, samples, epochs=200, lr=1e-3, ctx=None):
        """Adam on the GPU over several GEPs; samples[i] is (S x ndofs_i), the same S for every GEP."""
        ctx = ctx or geps[0].ctx
        Es = [np.ascontiguousarray(s, dtype=np.float64) for s in samples]
        S = Es[0].shape[0]
        if any(e.shape[0] != S for e in Es):
            raise Fem2dError(1, "every GEP needs the same number of samples")
        gh = (ctypes.c_void_p * len(geps))(*[g._h.value for g in geps])
        eh = (_DP * len(Es))(*[e.ctypes.data_as(_DP) for e in Es])
        hist = np.zeros(epochs)
        _check(lib().fem2d_patchnet_train(ctx._h, self._h, gh, len(geps), float(shift), eh, S, int(epochs), float(lr),
                                          _ptr(hist, ctypes.c_double)))
        return hist


def patch_features(domain, shift):
    """The network's inputs on a Domain: (patch_ptr, dof, feat [rows x 16], weight)."""
    sz = np.zeros(2, np.int64)
    L = lib()
    _check(L.fem2d_patchnet_features(domain._h, float(shift), _ptr(sz, ctypes.c_int64), None, None, None, None))
    P, R = int(sz[0]), int(sz[1])
    ptr = np.zeros(P + 1, np.int64)
    dof = np.zeros(R, np.int32)
    feat = np.zeros((R, 16), np.float32)
    w = np.zeros(R, np.float32)
    _check(L.fem2d_patchnet_features(domain._h, float(shift), _ptr(sz, ctypes.c_int64), _ptr(ptr, ctypes.c_int64),
                                     _ptr(dof, ctypes.c_int32), feat.ctypes.data_as(_FP), w.ctypes.data_as(_FP)))
    return ptr, dof, feat, w


class PCG:
    """Device PCG for K = c_a A + c_b B (SPD), plain (net=None) or learned preconditioner."""

    def __init__(self, gep, c_a, c_b, net=None, ctx=None, basis=None):
        """basis (rows x k, rows in patch_features order): a caller-given coarse basis instead of the network's."""
        self.ctx = ctx or gep.ctx
        self.gep = gep   # keeps the GEP alive while the solver references its device arrays
        self.n = gep.dimension
        h = ctypes.c_void_p()
        if basis is not None:
            Zb = np.ascontiguousarray(basis, dtype=np.float32)
            _check(lib().fem2d_pcg_create_with_basis(self.ctx._h, gep._h, float(c_a), float(c_b), Zb.shape[1],
                                                     Zb.ctypes.data_as(_FP), ctypes.byref(h)))
        else:
            _check(lib().fem2d_pcg_create(self.ctx._h, gep._h, float(c_a), float(c_b), net._h if net else None,
                                          ctypes.byref(h)))
        self._h = h

    def __del__(self):
        try:
            from . import _lib
        except ImportError:   # interpreter shutdown
            return
        if getattr(self, "_h", None) and _lib is not None:
            _lib.fem2d_pcg_free(self._h)
            self._h = None

    def solve(self, rhs, tol=1e-10, max_iter=5000):
        """x = K^-1 rhs (ndofs or ndofs x nrhs); returns (x, stats dict)."""
        r = np.ascontiguousarray(np.asarray(rhs, dtype=np.float64))
        one = r.ndim == 1
        r2 = r.reshape(self.n, -1)
        x = np.zeros_like(r2)
        st = np.zeros(5)
        rc = lib().fem2d_pcg_solve(self._h, r2.shape[1], _ptr(r2, ctypes.c_double), _ptr(x, ctypes.c_double),
                                   float(tol), int(max_iter), _ptr(st, ctypes.c_double))
        stats = {"iters": int(st[0]), "relres": float(st[1]), "ms": float(st[2]), "setup_ms": float(st[3]),
                 "coarse_dim": int(st[4]), "converged": rc == 0}
        if rc not in (0, 11):
            _check(rc)
        return (x[:, 0] if one else x), stats


def harvest_errors(gep, c_a, c_b, nrhs=8, every=10, max_samples=256, tol=1e-10, max_iter=5000, seed=0, ctx=None,
                   first=0):
    """Error vectors of the plain solver (S x ndofs): the exact solutions of nrhs random systems come from
    the multifrontal solve, the PCG iterates are recorded every `every` iterations from iteration `first` on
    (late iterates hold the slowly converging components the coarse space must capture)."""
    ctx = ctx or gep.ctx
    n = gep.dimension
    rhs = np.random.default_rng(seed).standard_normal((n, nrhs))
    xstar = gep.shifted_solve(c_a, c_b, rhs, spd=True)
    solver = PCG(gep, c_a, c_b, None, ctx=ctx)
    out = np.zeros((max_samples, n))
    ns = ctypes.c_int()
    _check(lib().fem2d_pcg_harvest(solver._h, nrhs, _ptr(np.ascontiguousarray(rhs), ctypes.c_double),
                                   _ptr(np.ascontiguousarray(xstar), ctypes.c_double), float(tol), int(max_iter),
                                   int(first), int(every), int(max_samples), _ptr(out, ctypes.c_double),
                                   ctypes.byref(ns)))
    return out[: ns.value]
