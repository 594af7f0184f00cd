"""Python face of the fem2d oracle (TEST INFRASTRUCTURE ONLY).

The oracle is the checker for the GPU product: only tests/, ``__graft_entry__.smoke()`` and
``bench.py``'s CPU-baseline leg may import this module. It wraps ``liboracle.so`` (a literal C++
restatement of the reference's mesh, DoF enumeration, GLQ, basis spaces, 2-D quadrature integrals
and galerkin assembly, see fem2d_oracle.cpp) and adds the FP64 eigen-solves the reference relies on:

* ``reference_dense_solve``: restates ``nalgebra_solve_gep`` (src/fem_problem/linalg/nalgebra_solve.rs:14-50):
  Cholesky inverse of B, the product B^-1 A, a symmetric eigen-decomposition that reads only the lower
  triangle of that product (nalgebra 0.30.1 ``SymmetricEigen`` tridiagonalises from the lower triangle),
  then the eigenvalue nearest the target.
* ``gep_exact_dense``: LAPACK ``sygv`` on (A, B) through ``scipy.linalg.eigh`` (the "GEP-exact" solve).
* ``sparse_shift_invert``: ARPACK shift-invert ``scipy.sparse.linalg.eigsh(A, k, M=B, sigma)``, the FP64
  stand-in for the external SLEPc ``solve_gep`` (src/fem_problem/linalg/slepc_solve.rs:14-68).
"""
from __future__ import annotations

import ctypes
import json
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

HREF_T, HREF_U, HREF_V = 0, 1, 2
HIERPOLY, KOLEG = 0, 1


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "liboracle.so")
        if not os.path.exists(path):
            from . import build as _b  # noqa: F401  (lazy build for a fresh checkout)
            _b.build_oracle()
        L = ctypes.CDLL(path)
        P = ctypes.c_void_p
        i64p = ctypes.POINTER(ctypes.c_int64)
        f64p = ctypes.POINTER(ctypes.c_double)
        i32p = ctypes.POINTER(ctypes.c_int32)
        L.oracle_last_error.restype = ctypes.c_char_p
        L.oracle_mesh_new.restype = P
        L.oracle_mesh_new.argtypes = [ctypes.c_int64, f64p, ctypes.c_int64, i64p, f64p]
        L.oracle_free.argtypes = [P]
        L.oracle_mesh_unit.restype = P
        for name in ("oracle_set_orders", "oracle_p_refine", "oracle_h_refine"):
            getattr(L, name).argtypes = [P, i64p, ctypes.c_int64, ctypes.c_int, ctypes.c_int]
        for name in ("oracle_num_elems", "oracle_num_edges", "oracle_num_nodes", "oracle_num_specs"):
            getattr(L, name).restype = ctypes.c_int64
            getattr(L, name).argtypes = [P]
        L.oracle_elem_info.argtypes = [P, i64p]
        L.oracle_execute_h.argtypes = [P, i64p, i32p, ctypes.c_int64]
        L.oracle_domain.argtypes = [P, i64p]
        L.oracle_specs.argtypes = [P, i64p]
        L.oracle_galerkin.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, i64p]
        L.oracle_gep_export.argtypes = [P, i32p, i32p, f64p, f64p]
        L.oracle_galerkin_by_parts.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_int, i64p]
        L.oracle_by_parts_export.argtypes = [P, i32p, i32p, f64p]
        L.oracle_quad_doc.argtypes = [ctypes.c_int, f64p]
        L.oracle_glq.argtypes = [ctypes.c_int, f64p, f64p]
        L.oracle_shapes.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, f64p, f64p]
        L.oracle_default_ngq.argtypes = [ctypes.c_int]
        L.oracle_num_leaves.argtypes = [P]
        L.oracle_elem_bounds.argtypes = [P, f64p]
        L.oracle_xy_fields.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_int, f64p, ctypes.c_int64, f64p, f64p]
        _LIB = L
    return _LIB


def _p(a, ct):
    return a.ctypes.data_as(ctypes.POINTER(ct))


def _check(rc):
    if rc != 0:
        raise RuntimeError(lib().oracle_last_error().decode())


def mesh_arrays_from_json(obj):
    """Mesh JSON (the reference's format, src/fem_domain/domain/mesh.rs:100-141) to flat arrays."""
    if isinstance(obj, str):
        obj = json.loads(obj)
    nodes = np.asarray(obj["Nodes"], dtype=np.float64).reshape(-1, 2)
    els = obj["Elements"]
    ids = np.asarray([e["node_ids"] for e in els], dtype=np.int64).reshape(-1, 4)
    mats = np.asarray([e["materials"] for e in els], dtype=np.float64).reshape(-1, 4)
    return nodes, ids, mats


class OracleMesh:
    """Restated ``Mesh`` + ``Domain`` + ``galerkin_sample_gep_hcurl`` (CPU, FP64)."""

    def __init__(self, mesh_json=None):
        if mesh_json is None:   # Mesh::unit()
            self.h = lib().oracle_mesh_unit()
            self.ndofs = None
            return
        nodes, ids, mats = mesh_arrays_from_json(mesh_json)
        nodes = np.ascontiguousarray(nodes)
        ids = np.ascontiguousarray(ids)
        mats = np.ascontiguousarray(mats)
        h = lib().oracle_mesh_new(len(nodes), _p(nodes, ctypes.c_double), len(ids), _p(ids, ctypes.c_int64),
                                  _p(mats, ctypes.c_double))
        if not h:
            raise RuntimeError(lib().oracle_last_error().decode())
        self.h = h
        self.ndofs = None

    def __del__(self):
        if getattr(self, "h", None):
            lib().oracle_free(self.h)
            self.h = None

    def _ids(self, ids):
        if ids is None:
            return None, 0
        a = np.ascontiguousarray(np.asarray(ids, dtype=np.int64))
        self._keep = a
        return _p(a, ctypes.c_int64), len(a)

    def set_orders(self, i, j, ids=None):
        p, n = self._ids(ids)
        _check(lib().oracle_set_orders(self.h, p, n, i, j))

    def p_refine(self, di, dj, ids=None):
        p, n = self._ids(ids)
        _check(lib().oracle_p_refine(self.h, p, n, di, dj))

    def h_refine(self, kind, ids=None, ext=-1):
        p, n = self._ids(ids)
        _check(lib().oracle_h_refine(self.h, p, n, kind, ext))

    def execute_h(self, ids, kinds):
        a = np.ascontiguousarray(np.asarray(ids, dtype=np.int64))
        k = np.ascontiguousarray(np.asarray(kinds, dtype=np.int32))
        _check(lib().oracle_execute_h(self.h, _p(a, ctypes.c_int64), _p(k, ctypes.c_int32), len(a)))

    def apply_ops(self, ops):
        """Replay a refinement script (the op format of fem_2d_gb300.configs)."""
        for op in ops:
            if op[0] == "orders":
                self.set_orders(op[1], op[2], op[3])
            elif op[0] == "pref":
                self.p_refine(op[1], op[2], op[3])
            elif op[0] == "href":
                self.h_refine(op[1], op[2], op[3])
            elif op[0] == "hmix":
                self.execute_h(op[1], op[2])
            elif op[0] == "ordersmap":
                for (i, j), ids in op[1]:
                    self.set_orders(i, j, ids)
            else:
                raise ValueError(op[0])

    def num_elems(self):
        return lib().oracle_num_elems(self.h)

    def elem_info(self):
        n = self.num_elems()
        out = np.zeros((n, 14), dtype=np.int64)
        _check(lib().oracle_elem_info(self.h, _p(out, ctypes.c_int64)))
        return out

    def elem_bounds(self):
        """Per Elem (x0, y0, x1, y1)."""
        out = np.zeros((self.num_elems(), 4), dtype=np.float64)
        _check(lib().oracle_elem_bounds(self.h, _p(out, ctypes.c_double)))
        return out

    def domain(self):
        nd = ctypes.c_int64(0)
        _check(lib().oracle_domain(self.h, ctypes.byref(nd)))
        self.ndofs = nd.value
        return self.ndofs

    def specs(self):
        n = lib().oracle_num_specs(self.h)
        out = np.zeros((n, 6), dtype=np.int64)
        _check(lib().oracle_specs(self.h, _p(out, ctypes.c_int64)))
        return out

    def xy_fields(self, solution, d0, d1, basis=HIERPOLY):
        """UniformFieldSpace::xy_fields restated (fields.rs:63-122): (x, y), each (leaves, d0, d1)."""
        if self.ndofs is None:
            self.domain()
        nl = lib().oracle_num_leaves(self.h)
        sol = np.ascontiguousarray(solution, dtype=np.float64)
        x = np.zeros((nl, d0, d1))
        y = np.zeros((nl, d0, d1))
        _check(lib().oracle_xy_fields(self.h, basis, d0, d1, _p(sol, ctypes.c_double), len(sol),
                                      _p(x, ctypes.c_double), _p(y, ctypes.c_double)))
        return x, y

    def galerkin_by_parts(self, basis=HIERPOLY, nu=0, nv=0):
        """The Galerkin visit set evaluated with integrate_by_parts (integrals.rs:94-237, 356-418) on
        samplers with second derivatives (GLQ points plus the endpoints): (rows, cols, vals), vals[:, 0]
        the CurlCurl face term, vals[:, 1:5] its edge terms, vals[:, 5] the L2Inner value, summed per
        upper-triangle key in elem order."""
        nnz = ctypes.c_int64(0)
        _check(lib().oracle_galerkin_by_parts(self.h, basis, nu, nv, ctypes.byref(nnz)))
        n = nnz.value
        r = np.zeros(n, np.int32)
        c = np.zeros(n, np.int32)
        v = np.zeros((n, 6), np.float64)
        _check(lib().oracle_by_parts_export(self.h, _p(r, ctypes.c_int32), _p(c, ctypes.c_int32),
                                            _p(v, ctypes.c_double)))
        return r, c, v

    def galerkin(self, basis=HIERPOLY, nu=0, nv=0, threads=1):
        """Upper-triangle COO (rows, cols, a, b), sorted by (row, col) like the reference's BTreeMap."""
        nnz = ctypes.c_int64(0)
        _check(lib().oracle_galerkin(self.h, basis, nu, nv, threads, ctypes.byref(nnz)))
        n = nnz.value
        r = np.zeros(n, np.int32)
        c = np.zeros(n, np.int32)
        a = np.zeros(n, np.float64)
        b = np.zeros(n, np.float64)
        _check(lib().oracle_gep_export(self.h, _p(r, ctypes.c_int32), _p(c, ctypes.c_int32),
                                       _p(a, ctypes.c_double), _p(b, ctypes.c_double)))
        return r, c, a, b


class OracleReplay:
    """The oracle mesh as a ``replay`` class of fem_2d_gb300.configs: workload scripts built on it are
    the same as on the product's Mesh, and loading it loads no product library."""

    def __init__(self, mesh_json):
        self.mesh = OracleMesh(mesh_json)

    def apply(self, ops):
        self.mesh.apply_ops(ops)

    def elem_info(self):
        return self.mesh.elem_info()


def quad_doc(n):
    """[inner, edge 0..3] of u^2 v^2 by the by-parts quadratures (glq.rs:36-52, 79-100 doc examples)."""
    out = np.zeros(5)
    _check(lib().oracle_quad_doc(n, _p(out, ctypes.c_double)))
    return out


def glq(n):
    p = np.zeros(n)
    w = np.zeros(n)
    _check(lib().oracle_glq(n, _p(p, ctypes.c_double), _p(w, ctypes.c_double)))
    return p, w


def shapes(basis, nmax, x):
    x = np.ascontiguousarray(np.asarray(x, dtype=np.float64))
    out = np.zeros((4, nmax + 1, len(x)))
    _check(lib().oracle_shapes(basis, nmax, len(x), _p(x, ctypes.c_double), _p(out, ctypes.c_double)))
    return out


def full_sym(n, rows, cols, vals):
    """Mirror an upper-triangle COO into a full symmetric scipy CSR matrix."""
    import scipy.sparse as sp

    off = rows != cols
    r = np.concatenate([rows, cols[off]])
    c = np.concatenate([cols, rows[off]])
    v = np.concatenate([vals, vals[off]])
    return sp.csr_matrix((v, (r, c)), shape=(n, n))


def reference_dense_solve(A, B, target):
    """nalgebra_solve_gep restated (src/fem_problem/linalg/nalgebra_solve.rs:14-50)."""
    import scipy.linalg as sl

    A = np.asarray(A.todense() if hasattr(A, "todense") else A)
    B = np.asarray(B.todense() if hasattr(B, "todense") else B)
    L = np.linalg.cholesky(B)
    Linv = sl.solve_triangular(L, np.eye(len(B)), lower=True)
    Binv = Linv.T @ Linv
    ba = Binv @ A
    low = np.tril(ba)
    sym = low + np.tril(ba, -1).T
    w, v = np.linalg.eigh(sym)
    if np.all(np.abs(w) < 1e-12):
        raise RuntimeError("SpuriouslyConverged")
    k = int(np.argmin(np.abs(w - target)))
    return w[k], v[:, k]


def gep_exact_dense(A, B, target, k=1):
    """Generalized symmetric-definite solve by LAPACK (scipy.linalg.eigh), k pairs nearest target."""
    import scipy.linalg as sl

    A = np.asarray(A.todense() if hasattr(A, "todense") else A)
    B = np.asarray(B.todense() if hasattr(B, "todense") else B)
    w, v = sl.eigh(A, B)
    order = np.argsort(np.abs(w - target), kind="stable")[:k]
    return w[order], v[:, order]


def sparse_shift_invert(A, B, target, k):
    """k eigenpairs nearest target by ARPACK shift-invert (FP64, sparse LU of A - target*B)."""
    import scipy.sparse.linalg as sla

    w, v = sla.eigsh(A.tocsc(), k=k, M=B.tocsc(), sigma=target, which="LM", tol=1e-14)
    order = np.argsort(np.abs(w - target), kind="stable")
    return w[order], v[:, order]


def _borth_block(W, V, B, drop=1e-8):
    """B-orthogonalise W against B-orthonormal V (two passes) and orthonormalise W itself."""
    for _ in range(2):
        if V is not None:
            W = W - V @ (V.T @ (B @ W))
    for it in range(2):
        G = W.T @ (B @ W)
        w, U = np.linalg.eigh((G + G.T) / 2)
        keep = w > (w.max() * drop if it == 0 else 0.0)
        W = W @ (U[:, keep] / np.sqrt(w[keep]))
        if V is not None:
            W = W - V @ (V.T @ (B @ W))
    return W


def sparse_nearest_physical(A, B, sigma, k, block=None, steps=3, tol=1e-11, max_cycles=40, spurious=1e-6, perm=None):
    """FP64 oracle for gpu_solve_gep: the k eigenpairs nearest sigma excluding the curl null space.

    Search space from T = (A - sigma B)^-1 A (A + c B)^-1 B, c = 0.05 |sigma|, with sparse LU solves (SuperLU),
    block Krylov cycles with CGS2 B-orthogonalisation, Rayleigh-Ritz on (A, B), Ritz pairs with relative
    residual >= 1 or |theta| <= spurious*|sigma| not selected. Pinned against LAPACK dense solves on
    small meshes (tests/test_oracle_sparse.py).
    """
    import scipy.sparse.linalg as sla

    n = A.shape[0]
    b = block or min(n, k + max(8, k))
    if perm is None:
        luM = sla.splu((A - sigma * B).tocsc(), permc_spec="MMD_AT_PLUS_A")
        luP = sla.splu((A + 0.05 * abs(sigma) * B).tocsc(), permc_spec="MMD_AT_PLUS_A")
    else:
        luM = NDLU((A - sigma * B).tocsc(), perm)
        luP = NDLU((A + 0.05 * abs(sigma) * B).tocsc(), perm)

    def T(X):
        return luM.solve(A @ luP.solve(B @ X))

    X = T(np.random.default_rng(1).standard_normal((n, b)))
    for _ in range(max_cycles):
        V = _borth_block(X, None, B)
        last = V
        for _s in range(steps):
            W = _borth_block(T(last), V, B)
            if W.shape[1] == 0:
                break
            V = np.hstack([V, W])
            last = W
        AV = A @ V
        BV = B @ V
        GA = V.T @ AV
        th, Y = np.linalg.eigh((GA + GA.T) / 2)
        R = AV @ Y - (BV @ Y) * th
        rel = np.linalg.norm(R, axis=0) / (np.abs(th) * np.linalg.norm(BV @ Y, axis=0) + 1e-300)
        ok = (np.abs(th) > spurious * abs(sigma)) & (rel < 1.0)
        idx = np.nonzero(ok)[0]
        idx = idx[np.argsort(np.abs(th[idx] - sigma), kind="stable")][:b]
        X = V @ Y[:, idx]
        if len(idx) >= k and rel[idx[:k]].max() < tol:
            break
    return th[idx[:k]], X[:, :k], rel[idx[:k]]


def dense_nearest_physical(A, B, sigma, k, spurious=1e-6):
    """LAPACK (scipy.linalg.eigh) reference for small problems: k nearest sigma with |lambda| > spurious*|sigma|."""
    import scipy.linalg as sl

    A = np.asarray(A.todense() if hasattr(A, "todense") else A)
    B = np.asarray(B.todense() if hasattr(B, "todense") else B)
    w, v = sl.eigh(A, B)
    ok = np.nonzero(np.abs(w) > spurious * abs(sigma))[0]
    ok = ok[np.argsort(np.abs(w[ok] - sigma), kind="stable")][:k]
    return w[ok], v[:, ok]


def tangential_jumps(bounds, ex, ey):
    """Largest jump of the tangential field across the interior lines shared by two leaf Elems.

    ``bounds`` holds per leaf (x0, y0, x3, y3); ``ex``/``ey`` are (leaves, d0, d1) grids with m along x.
    On a vertical line the tangential component is E_y, on a horizontal line E_x. Grid points are
    matched where both leaves sample the same coordinate strictly inside the common segment (hanging
    edges included). An H(curl)-conforming discrete space gives zero jumps for every coefficient vector.
    Returns (max |jump| / max |E|, number of matched points).
    """
    nl, d0, d1 = ex.shape
    gu = np.linspace(0.0, 1.0, d0)
    gv = np.linspace(0.0, 1.0, d1)
    scale = max(np.max(np.abs(ex)), np.max(np.abs(ey)), 1e-300)
    worst, count = 0.0, 0
    tol = 1e-12
    key = lambda v: round(float(v), 9)   # noqa: E731
    starts_x, starts_y = {}, {}
    for b in range(nl):
        starts_x.setdefault(key(bounds[b][0]), []).append(b)
        starts_y.setdefault(key(bounds[b][1]), []).append(b)
    for a in range(nl):
        A = bounds[a]
        for b in starts_x.get(key(A[2]), []):   # b to the right of a
            B = bounds[b]
            lo, hi = max(A[1], B[1]), min(A[3], B[3])
            if b == a or hi - lo <= tol:
                continue
            ya = A[1] + gv * (A[3] - A[1])
            yb = B[1] + gv * (B[3] - B[1])
            for i, yy in enumerate(ya):
                if lo + tol < yy < hi - tol:
                    for j in np.nonzero(np.abs(yb - yy) < tol)[0]:
                        worst = max(worst, abs(ey[a, d0 - 1, i] - ey[b, 0, j]))
                        count += 1
        for b in starts_y.get(key(A[3]), []):   # b above a
            B = bounds[b]
            lo, hi = max(A[0], B[0]), min(A[2], B[2])
            if b == a or hi - lo <= tol:
                continue
            xa = A[0] + gu * (A[2] - A[0])
            xb = B[0] + gu * (B[2] - B[0])
            for i, xx in enumerate(xa):
                if lo + tol < xx < hi - tol:
                    for j in np.nonzero(np.abs(xb - xx) < tol)[0]:
                        worst = max(worst, abs(ex[a, i, d1 - 1] - ex[b, j, 0]))
                        count += 1
    return worst / scale, count


class OracleSparseMatrix:
    """SparseMatrix restated (sparse_matrix.rs:12-127): upper-triangle map, r <= c keys, += on collision."""

    def __init__(self, dimension):
        self.dimension = int(dimension)
        self.entries = {}

    def insert(self, rc, value):
        r, c = int(rc[0]), int(rc[1])
        assert r < self.dimension and c < self.dimension
        key = (r, c) if r <= c else (c, r)
        if key in self.entries:
            self.entries[key] += value
        else:
            self.entries[key] = value

    def aij_bytes(self):
        """From<SparseMatrix> for AIJMatrixBinary + print_to_petsc_binary_file (sparse_matrix.rs:184-265)."""
        import struct

        n = self.dimension
        row_counts = [0] * n
        for (r, c) in self.entries:
            row_counts[r] += 1
            if r != c:
                row_counts[c] += 1
        full = {(c, r): v for (r, c), v in self.entries.items()}
        full.update(self.entries)
        keys = sorted(full)
        out = bytearray(b"\0{P")
        out += struct.pack(">III", n, n, len(keys))
        out += struct.pack(">%dI" % n, *row_counts)
        out += struct.pack(">%dI" % len(keys), *[c for (_, c) in keys])
        out += struct.pack(">%dd" % len(keys), *[full[k] for k in keys])
        return bytes(out)


def petsc_vec_bytes(values):
    """The PETSc Vec binary retrieve_eigenvector reads (slepc_solve.rs:114-135)."""
    import struct

    return struct.pack(">ii", 1211214, len(values)) + struct.pack(">%dd" % len(values), *values)


def dof_boxes(om):
    """Support box (x0, y0, x1, y1) of every DoF: the union of the boxes of the Elems whose basis
    specs carry it (one Elem for an Elem-type DoF, the Elems on both sides for an edge-type DoF)."""
    if om.ndofs is None:
        om.domain()
    eb = om.elem_bounds()
    sp = om.specs()
    ids = sp[:, 5]
    box = np.empty((om.ndofs, 4))
    box[:, :2] = np.inf
    box[:, 2:] = -np.inf
    e = eb[sp[:, 0]]
    np.minimum.at(box[:, 0], ids, e[:, 0])
    np.minimum.at(box[:, 1], ids, e[:, 1])
    np.maximum.at(box[:, 2], ids, e[:, 2])
    np.maximum.at(box[:, 3], ids, e[:, 3])
    return box


def nd_order(box, leaf=256):
    """Geometric nested dissection of the DoFs by their support boxes: the oracle's own fill-reducing
    ordering for its sparse LU (an ordering changes no value, only the fill and the rounding order).

    Two DoFs couple only if their supports overlap with positive area (an Elem pairs with itself and
    its descendants, and an edge DoF's support spans both sides of its edge), so a line x = s splits
    the DoFs into those wholly left of it, those wholly right of it, and a separator of the DoFs whose
    boxes straddle it. Each level tries both axes and, between the 30% and 70% quantiles of the box
    centres, the cut with the fewest straddling DoFs; the order is left part, right part, separator,
    recursively, down to parts of ``leaf`` DoFs.
    """
    import sys

    out = []

    def cut(idx):
        best = None
        for ax in (0, 1):
            lo, hi = box[idx, ax], box[idx, ax + 2]
            c = np.sort(0.5 * (lo + hi))
            q0, q1 = c[int(0.3 * (len(c) - 1))], c[int(0.7 * (len(c) - 1))]
            cand = np.unique(np.concatenate([lo, hi]))
            cand = cand[(cand >= q0) & (cand <= q1)]
            if len(cand) == 0:
                continue
            slo, shi = np.sort(lo), np.sort(hi)
            left = np.searchsorted(shi, cand, side="right")             # hi <= s
            right = len(idx) - np.searchsorted(slo, cand, side="left")   # lo >= s
            score = (len(idx) - left - right) * len(idx) + np.abs(left - right)
            k = int(np.argmin(score))
            if best is None or score[k] < best[0]:
                best = (score[k], ax, cand[k])
        return best

    def rec(idx):
        if len(idx) <= leaf:
            out.append(idx)
            return
        b = cut(idx)
        if b is None:
            out.append(idx)
            return
        _, ax, s = b
        lo, hi = box[idx, ax], box[idx, ax + 2]
        L, R = idx[hi <= s], idx[lo >= s]
        if len(L) == 0 or len(R) == 0:
            out.append(idx)
            return
        rec(L)
        rec(R)
        out.append(idx[(lo < s) & (hi > s)])

    sys.setrecursionlimit(max(10000, sys.getrecursionlimit()))
    rec(np.arange(len(box)))
    return np.concatenate(out)


class NDLU:
    """SuperLU factorization of a sparse matrix under a given symmetric ordering (``nd_order``) with
    diagonal-preferring threshold pivoting; ``solve`` works in the original numbering."""

    def __init__(self, K, perm, pivot=0.1):
        import scipy.sparse.linalg as sla

        self.perm = perm
        self.inv = np.empty_like(perm)
        self.inv[perm] = np.arange(len(perm))
        Kp = K.tocsr()[perm][:, perm].tocsc()
        self.lu = sla.splu(Kp, permc_spec="NATURAL", diag_pivot_thresh=pivot, options={"SymmetricMode": True})

    def solve(self, X):
        return self.lu.solve(np.ascontiguousarray(X[self.perm]))[self.inv]


def _cluster_bounds(th_sel, rb, th_all, rel_tol=1e-6):
    """Quadratic (Kato-Temple type) eigenvalue error bounds for Ritz values th_sel with B^-1-norm
    residuals rb. Ritz values within rel_tol of each other form a cluster C (degenerate modes of the
    rectangle come in such pairs); with r_C = sqrt(sum_{j in C} rb_j^2) and g the distance from the
    cluster to the nearest Ritz value outside it, the bound is r_C^2 / (g - r_C) when g > 2 r_C, else
    r_C (some eigenvalue always lies within rb of a Ritz value). The gap is taken to the other computed
    Ritz values, which assumes no eigenvalue of the pencil is missing near the cluster."""
    out = np.empty(len(th_sel))
    for i, t in enumerate(th_sel):
        inc = np.abs(th_sel - t) <= rel_tol * abs(t)
        rc = float(np.sqrt(np.sum(rb[inc] ** 2)))
        others = th_all[np.abs(th_all - t) > rel_tol * abs(t)]
        g = float(np.min(np.abs(others - t))) if len(others) else np.inf
        out[i] = rc * rc / (g - rc) if g > 2 * rc else rc
    return out


def arpack_nearest_physical(A, B, sigma, k, perm, c=None, extra=None, spurious=1e-6, tol=1e-13, seed=0,
                            refine=2, reject=1e-2, pivot=0.1, schur=None):
    """Second, independent FP64 sparse oracle for large pencils: ARPACK (implicitly restarted Lanczos
    in the B inner product, through scipy ``eigsh``) on T = (A - sigma B)^-1 A (A + c B)^-1 B.

    T's eigenvalues mu = lambda / ((lambda - sigma)(lambda + c)) vanish on the curl null space and grow
    without bound as lambda nears sigma, so the largest |mu| are the physical modes near sigma. The
    solves are SuperLU factorizations under ``perm`` (threshold ``pivot`` for row pivoting: a smaller one
    keeps more diagonal pivots and less fill), or ``SchurLU`` substructuring when ``schur`` = (box, parts,
    sep) is given. The k + extra Lanczos vectors X are then refined
    ``refine`` times by one Rayleigh-Ritz step on (A, B) over span[X, T X] in FP64, and the k Ritz
    values nearest sigma with |lambda| > spurious |sigma| and relative residual below ``reject`` are
    returned with:

    * ``rel_residual`` ||A x - lambda B x|| / (|lambda| ||B x||) and ``backward_error``
      ||A x - lambda B x|| / ((||A||_1 + |lambda| ||B||_1) ||x||);
    * ``resid_binv`` = ||r||_{B^-1} for B-normalised x (some eigenvalue of the pencil lies within it of
      the Ritz value) and ``err_bound`` from ``_cluster_bounds``;
    * ``mu_min``: the smallest |mu| ARPACK returned. ``extra`` pairs beyond k (default k) are asked for
      because the order by |mu| is not the order by |lambda - sigma| below sigma; an eigenvalue missed
      has |mu| below ``mu_min``.
    """
    import scipy.sparse.linalg as sla

    n = A.shape[0]
    c = abs(sigma) if c is None else c
    extra = k if extra is None else extra
    if schur is None:
        luM = NDLU((A - sigma * B).tocsc(), perm, pivot)
        luP = NDLU((A + c * B).tocsc(), perm, pivot)
        luB = NDLU(B.tocsc(), perm, pivot)
    else:   # (box, parts, sep): two-level substructuring for very large pencils
        box, parts, sep = schur
        luM = SchurLU(A - sigma * B, box, parts, sep, pivot)
        luP = SchurLU(A + c * B, box, parts, sep, pivot)
        luB = SchurLU(B, box, parts, sep, pivot)
    Ac, Bc = A.tocsr(), B.tocsr()
    count = [0]

    def T(X):
        count[0] += 1 if X.ndim == 1 else X.shape[1]
        return luM.solve(Ac @ luP.solve(Bc @ X))

    m = k + extra
    Aop = sla.LinearOperator((n, n), matvec=lambda x: Bc @ T(x), dtype=np.float64)
    Mi = sla.LinearOperator((n, n), matvec=luB.solve, dtype=np.float64)
    v0 = np.random.default_rng(seed).standard_normal(n)
    mu, V = sla.eigsh(Aop, k=m, M=Bc, Minv=Mi, which="LM", tol=tol, v0=v0, ncv=min(n - 1, max(2 * m + 1, m + 32)))
    mu_min = float(np.min(np.abs(mu)))

    def rayleigh_ritz(V):
        BV = Bc @ V
        G = V.T @ BV
        w, U = np.linalg.eigh((G + G.T) / 2)
        keep = w > w.max() * 1e-14
        W = V @ (U[:, keep] / np.sqrt(w[keep]))
        AW, BW = Ac @ W, Bc @ W
        H = W.T @ AW
        th, Y = np.linalg.eigh((H + H.T) / 2)
        return th, W @ Y, AW @ Y, BW @ Y

    def residuals(th, X, AX, BX):
        R = AX - BX * th
        rn = np.linalg.norm(R, axis=0)
        rel = rn / (np.abs(th) * np.linalg.norm(BX, axis=0) + 1e-300)
        # Rayleigh-Ritz on (A, B) over a space that holds T-application error can return Ritz values
        # that are mixtures of null-space and high-frequency directions; their residuals are O(1) or
        # larger, so they are not selected
        ok = np.nonzero((np.abs(th) > spurious * abs(sigma)) & (rel < reject))[0]
        return R, rn, rel, ok[np.argsort(np.abs(th[ok] - sigma), kind="stable")]

    th, X, AX, BX = rayleigh_ritz(V)
    for _ in range(refine):
        _, _, _, order = residuals(th, X, AX, BX)
        Xs = X[:, order[:m]]
        th, X, AX, BX = rayleigh_ritz(np.hstack([Xs, T(Xs)]))
    R, rn, rel, order = residuals(th, X, AX, BX)
    nA, nB = sla.norm(Ac, 1), sla.norm(Bc, 1)
    bwd = rn / ((nA + np.abs(th) * nB) * np.linalg.norm(X, axis=0))
    idx = order[:k]
    ok = order
    Rs = R[:, idx]
    Z = luB.solve(Rs)
    rb = np.sqrt(np.abs(np.einsum("ij,ij->j", Rs, Z)))
    phys = th[ok]
    # the eigenvalues from ARPACK's converged mu directly: mu (lambda - sigma)(lambda + c) = lambda, the
    # root of the sign of lambda's side of sigma. Relative conditioning |d lambda / lambda| / |d mu / mu|
    # = |(lambda - sigma)(lambda + c)| / (lambda^2 + sigma c) <= 1, and rounding noise in the solves (high-
    # frequency directions, where T's eigenvalues are ~0) barely moves the wanted mu, whereas a Rayleigh-
    # Ritz step on (A, B) can turn that noise into spurious or inaccurate Ritz pairs on ill-conditioned
    # (monomial) pencils
    qa, qb, qc = mu, mu * (c - sigma) - 1.0, -mu * sigma * c
    disc = np.sqrt(qb * qb - 4.0 * qa * qc)
    r1 = (-qb + disc) / (2.0 * qa)
    r2 = (-qb - disc) / (2.0 * qa)
    lam_mu = np.where(mu > 0, np.maximum(r1, r2), np.where((r1 > 0) & (r1 < sigma), r1, r2))
    okm = np.nonzero(np.abs(lam_mu) > spurious * abs(sigma))[0]
    sel = okm[np.argsort(np.abs(lam_mu[okm] - sigma), kind="stable")][:k]
    return {"values": th[idx], "vectors": X[:, idx], "rel_residual": rel[idx], "backward_error": bwd[idx],
            "resid_binv": rb, "err_bound": _cluster_bounds(th[idx], rb, phys), "mu_min": mu_min,
            "applications": count[0], "values_from_mu": lam_mu[sel], "mu": mu[sel]}


def nd_parts(box, levels=4):
    """The top `levels` levels of ``nd_order``'s geometric dissection: returns (parts, sep), the 2^levels
    subdomains (index arrays) and the union of their separators (index array)."""
    parts, seps = [], []

    def cut(idx):
        best = None
        for ax in (0, 1):
            lo, hi = box[idx, ax], box[idx, ax + 2]
            c = np.sort(0.5 * (lo + hi))
            q0, q1 = c[int(0.3 * (len(c) - 1))], c[int(0.7 * (len(c) - 1))]
            cand = np.unique(np.concatenate([lo, hi]))
            cand = cand[(cand >= q0) & (cand <= q1)]
            if len(cand) == 0:
                continue
            slo, shi = np.sort(lo), np.sort(hi)
            left = np.searchsorted(shi, cand, side="right")
            right = len(idx) - np.searchsorted(slo, cand, side="left")
            score = (len(idx) - left - right) * len(idx) + np.abs(left - right)
            k = int(np.argmin(score))
            if best is None or score[k] < best[0]:
                best = (score[k], ax, cand[k])
        return best

    def rec(idx, level):
        b = cut(idx) if level < levels else None
        if b is None:
            parts.append(idx)
            return
        _, ax, s = b
        lo, hi = box[idx, ax], box[idx, ax + 2]
        rec(idx[hi <= s], level + 1)
        rec(idx[lo >= s], level + 1)
        seps.append(idx[(lo < s) & (hi > s)])

    rec(np.arange(len(box)), 0)
    return [p for p in parts if len(p)], (np.concatenate(seps) if seps else np.zeros(0, np.int64))


class SchurLU:
    """K x = b by two-level substructuring, for matrices beyond SuperLU's 32-bit size limits (its first
    fill estimate, about 20 x nnz, overflows near 1e8 nonzeros): each subdomain block K_ii (``nd_parts``)
    is factored by SuperLU under its own nested-dissection ordering; the separator unknowns are solved
    through the dense Schur complement S = K_SS - sum_i K_Si K_ii^-1 K_iS (LAPACK LU with partial
    pivoting). Subdomains of about a quarter of the waveguide's width keep their blocks of A - 10 B far
    from singular (their own PEC eigenvalues start near 39)."""

    def __init__(self, K, box, parts, sep, pivot=0.1):
        import scipy.linalg as sl
        import scipy.sparse.linalg as sla

        K = K.tocsr()
        self.n = K.shape[0]
        self.parts, self.sep = parts, sep
        self.lus, self.KiS, self.KSi = [], [], []
        KS = K[sep]
        S = KS[:, sep].toarray()
        for idx in parts:
            perm = nd_order(box[idx])
            inv = np.empty_like(perm)
            inv[perm] = np.arange(len(perm))
            Kii = K[idx][:, idx]
            lu = sla.splu(Kii[perm][:, perm].tocsc(), permc_spec="NATURAL", diag_pivot_thresh=pivot,
                          options={"SymmetricMode": True})
            KiS = K[idx][:, sep].tocsc()
            KSi = KS[:, idx].tocsr()
            nzc = np.nonzero(np.diff(KiS.indptr))[0]   # the separator columns this subdomain touches
            if len(nzc):
                rhs = KiS[:, nzc].toarray()[perm]
                Y = np.empty_like(rhs)
                for c0 in range(0, len(nzc), 512):
                    Y[:, c0:c0 + 512] = lu.solve(np.ascontiguousarray(rhs[:, c0:c0 + 512]))
                Y = Y[inv]
                S[:, nzc] -= KSi @ Y
            self.lus.append((lu, perm, inv))
            self.KiS.append(KiS.tocsr())
            self.KSi.append(KSi)
        self.Slu = sl.lu_factor(S) if len(sep) else None

    def _part_solve(self, i, b):
        lu, perm, inv = self.lus[i]
        return lu.solve(np.ascontiguousarray(b[perm]))[inv]

    def solve(self, b):
        import scipy.linalg as sl

        x = np.zeros_like(b)
        rS = b[self.sep].copy()
        for i, idx in enumerate(self.parts):
            rS -= self.KSi[i] @ self._part_solve(i, b[idx])
        xS = sl.lu_solve(self.Slu, rS) if self.Slu is not None else rS
        x[self.sep] = xS
        for i, idx in enumerate(self.parts):
            x[idx] = self._part_solve(i, b[idx] - self.KiS[i] @ xS)
        return x
