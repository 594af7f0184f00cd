"""Pin the CPU oracle against the reference's own known answers (no GPU).

* src/lib.rs:46-81   nalg_problem: mesh_a, PRef(2,2), GLQ [8,8], nalgebra dense solve nearest 2.64 -> 2.6479657 (1e-6)
* src/lib.rs:83-120  slepc_problem: mesh_b, PRef(3,3), T, T on [6,9,12], GLQ [8,8], nearest 1.475
                     -> 1.4745880937 (1e-9); test_input/test_eval.dat, test_input/test_evec.dat (624 entries)
* src/fem_problem/integration/glq.rs:255-375  20-point GLQ tables (1e-9) and scaling to [0.25, 0.5]
* src/fem_domain/domain.rs:239-338 doc-tests  basis-spec counts
"""
import numpy as np
import pytest


def _kat_mesh_b(ref, kat):
    m = ref.OracleMesh(kat["mesh_b"])
    m.p_refine(3, 3)
    m.h_refine(ref.HREF_T)
    m.h_refine(ref.HREF_T, ids=[6, 9, 12])
    return m


def test_glq_tables(oracle_lib, kat):
    ref = oracle_lib
    x, w = ref.glq(20)
    assert np.max(np.abs(x - np.asarray(kat["glq_x20"]))) < 1e-9
    assert np.max(np.abs(w - np.asarray(kat["glq_w20"]))) < 1e-9
    # scale_gauss_quad_points to (0.25, 0.5): glq.rs:238-249
    scale = (0.5 - 0.25) / 2.0
    off = (0.5 + 0.25) / 2.0
    assert abs(scale - 0.125) < 1e-14
    assert np.max(np.abs(x * scale + off - np.asarray(kat["glq_x20_scaled_025_05"]))) < 1e-9
    # glq.rs doc-test: 10 points integrate u^2 v^2 exactly (4/9) and the points sum to 0
    x10, w10 = ref.glq(10)
    assert abs(np.sum(x10)) < 1e-12
    assert abs((w10 @ x10 ** 2) ** 2 - 4.0 / 9.0) < 1e-12


def test_default_ngq(oracle_lib):
    L = oracle_lib.lib()
    # basis.rs:172-177: 4*max_order rounded up to a power of two
    assert [L.oracle_default_ngq(k) for k in (1, 2, 3, 4, 5, 8)] == [4, 8, 16, 16, 32, 32]


def test_slepc_problem_known_answer(oracle_lib, kat):
    ref = oracle_lib
    k = kat["kat_slepc_problem"]
    m = _kat_mesh_b(ref, kat)
    n = m.domain()
    assert n == k["ndofs"] == 624
    r, c, a, b = m.galerkin(ref.HIERPOLY, 8, 8)
    A = ref.full_sym(n, r, c, a)
    B = ref.full_sym(n, r, c, b)
    w, v = ref.gep_exact_dense(A, B, k["target"], k=1)
    assert abs(w[0] - k["value"]) < k["tol"]
    assert abs(w[0] - kat["slepc_eval"]) < 1e-11
    ws, _ = ref.sparse_shift_invert(A, B, k["target"], 1)
    assert abs(ws[0] - kat["slepc_eval"]) < 1e-11
    # the golden eigenvector is B-normalised and pins DoF ordering up to sign
    g = np.asarray(kat["slepc_evec"])
    assert abs(g @ (B @ g) - 1.0) < 1e-10
    x = v[:, 0] / np.sqrt(v[:, 0] @ (B @ v[:, 0]))
    x *= np.sign(x @ (B @ g))
    assert np.max(np.abs(x - g)) < 1e-9


def test_nalg_problem_known_answer(oracle_lib, kat):
    ref = oracle_lib
    k = kat["kat_nalg_problem"]
    m = ref.OracleMesh(kat["mesh_a"])
    m.p_refine(2, 2)
    n = m.domain()
    r, c, a, b = m.galerkin(ref.HIERPOLY, 8, 8)
    A = ref.full_sym(n, r, c, a)
    B = ref.full_sym(n, r, c, b)
    val, vec = ref.reference_dense_solve(A, B, k["target"])
    assert abs(val - k["value"]) < k["tol"]
    assert len(vec) == n


def test_domain_spec_counts_doctests(oracle_lib):
    ref = oracle_lib
    # domain.rs:239-252: unit mesh at orders (2,2) -> 4 local basis specs on Elem 0
    m = ref.OracleMesh()
    m.set_orders(2, 2)
    m.domain()
    s = m.specs()
    assert np.sum(s[:, 0] == 0) == 4
    # domain.rs:269-290: after a T refinement, Elem 0 has 4 descendants with 8 specs each
    m = ref.OracleMesh()
    m.set_orders(2, 2)
    m.h_refine(ref.HREF_T)
    m.domain()
    s = m.specs()
    assert np.sum(s[:, 0] == 0) == 0
    for d in (1, 2, 3, 4):
        assert np.sum(s[:, 0] == d) == 8
    # domain.rs:313-338: T then T on Elem 1; Elem 0 empty, Elem 1 holds 4 specs
    m = ref.OracleMesh()
    m.set_orders(2, 2)
    m.h_refine(ref.HREF_T)
    m.h_refine(ref.HREF_T, ids=[1])
    m.domain()
    s = m.specs()
    assert np.sum(s[:, 0] == 0) == 0
    assert np.sum(s[:, 0] == 1) == 4
    info = m.elem_info()
    assert info[5, 3] == 1 and info[1, 3] == 0


def test_refinement_errors(oracle_lib, kat):
    ref = oracle_lib
    m = ref.OracleMesh(kat["mesh_a"])
    with pytest.raises(RuntimeError, match="DuplicateElemIds"):
        m.h_refine(ref.HREF_T, ids=[0, 0])
    m.h_refine(ref.HREF_T, ids=[0])
    with pytest.raises(RuntimeError, match="ElemNotRefineable"):
        m.h_refine(ref.HREF_U, ids=[0])
    with pytest.raises(RuntimeError, match="InvalidExpansionOrders"):
        m.set_orders(0, 3)


def test_threaded_assembly_matches_serial(oracle_lib, kat):
    ref = oracle_lib
    m = _kat_mesh_b(ref, kat)
    m.domain()
    r1, c1, a1, b1 = m.galerkin(ref.HIERPOLY, 8, 8, threads=1)
    r2, c2, a2, b2 = m.galerkin(ref.HIERPOLY, 8, 8, threads=4)
    assert np.array_equal(r1, r2) and np.array_equal(c1, c2)
    assert np.array_equal(a1, a2) and np.array_equal(b1, b2)
