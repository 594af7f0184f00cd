"""Pin the FP64 sparse oracle (shift-invert block Krylov, LU solves) against LAPACK dense solves."""
import numpy as np

from fem_2d_gb300 import configs


def test_sparse_oracle_matches_lapack(oracle_lib):
    ref = oracle_lib
    w = configs.precision(seed=1, nx=4, ny=2)
    om = ref.OracleMesh(w.mesh_json)
    om.apply_ops(w.ops)
    n = om.domain()
    r, c, a, b = om.galerkin(w.basis, 10, 10)
    A = ref.full_sym(n, r, c, a)
    B = ref.full_sym(n, r, c, b)
    wd, _ = ref.dense_nearest_physical(A, B, 10.0, 6)
    ws, xs, rs = ref.sparse_nearest_physical(A, B, 10.0, 6)
    assert np.max(np.abs(ws - wd) / np.abs(wd)) < 1e-10
    assert np.max(rs) < 1e-9


def test_kat_slepc_eigenvalue_from_sparse_oracle(oracle_lib, kat):
    ref = oracle_lib
    m = ref.OracleMesh(kat["mesh_b"])
    m.apply_ops([("pref", 3, 3, None), ("href", 0, None, -1), ("href", 0, [6, 9, 12], -1)])
    n = m.domain()
    r, c, a, b = m.galerkin(0, 8, 8)
    A = ref.full_sym(n, r, c, a)
    B = ref.full_sym(n, r, c, b)
    ws, _, _ = ref.sparse_nearest_physical(A, B, 1.475, 1)
    assert abs(ws[0] - kat["slepc_eval"]) < 1e-11


def _small_full_form(ref):
    w = configs.full_scale(seed=3, nx=8, ny=4, rounds=2, fraction=0.44, replay=ref.OracleReplay)
    om = ref.OracleMesh(w.mesh_json)
    om.apply_ops(w.ops)
    n = om.domain()
    r, c, a, b = om.galerkin(0, 10, 10)
    return om, n, ref.full_sym(n, r, c, a), ref.full_sym(n, r, c, b)


def test_nested_dissection_is_a_permutation(oracle_lib):
    ref = oracle_lib
    om, n, A, B = _small_full_form(ref)
    box = ref.dof_boxes(om)
    perm = ref.nd_order(box, leaf=64)
    assert np.array_equal(np.sort(perm), np.arange(n))
    parts, sep = ref.nd_parts(box, 2)
    allv = np.concatenate(parts + [sep])
    assert np.array_equal(np.sort(allv), np.arange(n))
    # no coupling between different subdomains: every path between them crosses the separator
    K = (abs(A) + abs(B)).tocsr()
    lab = np.full(n, -1)
    for i, p in enumerate(parts):
        lab[p] = i
    rows, cols = K.nonzero()
    both = (lab[rows] >= 0) & (lab[cols] >= 0)
    assert np.all(lab[rows][both] == lab[cols][both])


def test_substructured_solver_and_arpack_oracle(oracle_lib):
    """SchurLU (SuperLU subdomains + dense Schur complement) solves A - 10 B backward-stably, and the
    ARPACK oracle on it gives LAPACK's eigenvalues."""
    import scipy.sparse.linalg as sla

    ref = oracle_lib
    om, n, A, B = _small_full_form(ref)
    box = ref.dof_boxes(om)
    parts, sep = ref.nd_parts(box, 2)
    K = A - 10.0 * B
    S = ref.SchurLU(K, box, parts, sep)
    x = np.random.default_rng(0).standard_normal((n, 2))
    y = S.solve(x)
    res = K @ y - x
    bwd = np.max(np.abs(res)) / (sla.norm(K, 1) * np.max(np.abs(y)) + np.max(np.abs(x)))
    assert bwd < 1e-15
    # (LAPACK smears the monomial basis's null space to |lambda| ~ 2e-5 here: a wider spurious cut)
    wd, _ = ref.dense_nearest_physical(A, B, 10.0, 8, spurious=1e-2)
    out = ref.arpack_nearest_physical(A, B, 10.0, 8, None, refine=0, schur=(box, parts, sep))
    assert np.max(np.abs(np.sort(out["values"]) - np.sort(wd)) / np.abs(np.sort(wd))) < 1e-10
    out2 = ref.arpack_nearest_physical(A, B, 10.0, 8, ref.nd_order(box), refine=0)
    assert np.max(np.abs(np.sort(out2["values"]) - np.sort(wd)) / np.abs(np.sort(wd))) < 1e-10
