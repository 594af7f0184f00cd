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
