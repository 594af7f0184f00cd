"""Device assembly parity: galerkin_sample_gep_hcurl on the GPU against the oracle's literal 2-D sums.

The pattern must be identical (integer, bit-exact); values agree entrywise within
    |A_gpu - A_oracle| <= 1e-12 * max|A|   (same for B)
which is the FP64 rounding gap between the reference's 2-D Gauss-Legendre sum and the separable
product the kernels evaluate.
"""
import numpy as np
import pytest

import fem_2d_gb300 as fg
from fem_2d_gb300 import configs

pytestmark = pytest.mark.gpu
TOL = 1e-12


@pytest.fixture(scope="module")
def ctx():
    from fem_2d_gb300 import build

    build.build()
    return fg.Context(0)


def _assemble_both(ref, mesh_json, ops, basis, glq, ctx):
    om = ref.OracleMesh(mesh_json)
    om.apply_ops(ops)
    n = om.domain()
    r, c, a, b = om.galerkin(basis, glq[0], glq[1])
    pm = fg.Mesh.from_json(mesh_json)
    configs.apply_ops(pm, ops)
    dom = fg.Domain.from_mesh(pm)
    bs = fg.KOLeg if basis == 1 else fg.HierPoly
    gep = fg.galerkin_sample_gep_hcurl(bs, fg.CurlCurl, fg.L2Inner, dom, list(glq), ctx=ctx)
    return n, (r, c, a, b), gep


def _check(ref_coo, gep):
    r, c, a, b = ref_coo
    gr, gc, ga, gb = gep.upper_coo()
    assert np.array_equal(r, gr) and np.array_equal(c, gc)
    ea = np.max(np.abs(ga - a)) / np.max(np.abs(a))
    eb = np.max(np.abs(gb - b)) / np.max(np.abs(b))
    assert ea <= TOL, ea
    assert eb <= TOL, eb
    return ea, eb


def test_kat_slepc_mesh(oracle_lib, kat, ctx):
    ref = oracle_lib
    ops = [("pref", 3, 3, None), ("href", 0, None, -1), ("href", 0, [6, 9, 12], -1)]
    n, coo, gep = _assemble_both(ref, kat["mesh_b"], ops, 0, (8, 8), ctx)
    assert n == 624
    _check(coo, gep)
    # the GPU-assembled pencil reproduces the known answer (checked with an FP64 LAPACK solve)
    A, B = gep.scipy()
    w, v = ref.gep_exact_dense(A, B, 1.475, k=1)
    assert abs(w[0] - kat["slepc_eval"]) < 1e-10
    assert gep.num_visits > 0
    assert ctx.kernel_launches >= 2


def test_kat_nalg_mesh(oracle_lib, kat, ctx):
    ref = oracle_lib
    n, coo, gep = _assemble_both(ref, kat["mesh_a"], [("pref", 2, 2, None)], 0, (8, 8), ctx)
    _check(coo, gep)
    A, B = gep.scipy()
    val, _ = ref.reference_dense_solve(A, B, 2.64)
    assert abs(val - 2.6479657) < 1e-6


def test_waveguide_small(oracle_lib, ctx):
    w = configs.waveguide_small()
    n, coo, gep = _assemble_both(oracle_lib, w.mesh_json, w.ops, w.basis, w.glq, ctx)
    _check(coo, gep)


@pytest.mark.parametrize("seed", [0, 1])
def test_precision_family_koleg(oracle_lib, ctx, seed):
    w = configs.precision(seed=seed, nx=6, ny=3)
    n, coo, gep = _assemble_both(oracle_lib, w.mesh_json, w.ops, w.basis, w.glq, ctx)
    _check(coo, gep)


def test_full_scale_family_small(oracle_lib, ctx):
    w = configs.full_scale(seed=1, nx=8, ny=4, rounds=3)
    n, coo, gep = _assemble_both(oracle_lib, w.mesh_json, w.ops, w.basis, w.glq, ctx)
    _check(coo, gep)


@pytest.mark.parametrize("seed", [0, 5])
def test_batch_family(oracle_lib, ctx, seed):
    w = configs.batch_member(seed)
    n, coo, gep = _assemble_both(oracle_lib, w.mesh_json, w.ops, w.basis, w.glq, ctx)
    _check(coo, gep)


def test_default_glq_and_mixed_materials(oracle_lib, kat, ctx):
    # glq_grid_dim = None -> default_ngq (basis.rs:172-177); mesh_a mixes eps and mu per Elem
    ref = oracle_lib
    ops = [("orders", 3, 2, None), ("href", 0, [1, 2], -1), ("href", 1, [5], -1)]
    om = ref.OracleMesh(kat["mesh_a"])
    om.apply_ops(ops)
    om.domain()
    coo = om.galerkin(0, 0, 0)
    pm = fg.Mesh.from_json(kat["mesh_a"])
    configs.apply_ops(pm, ops)
    gep = fg.galerkin_sample_gep_hcurl(fg.HierPoly, fg.CurlCurl, fg.L2Inner, fg.Domain.from_mesh(pm), None, ctx=ctx)
    _check(coo, gep)


def test_recompute_is_deterministic(oracle_lib, kat, ctx):
    w = configs.precision(seed=2, nx=4, ny=2)
    pm = configs.build_mesh(w)
    gep = fg.galerkin_sample_gep_hcurl(fg.KOLeg, fg.CurlCurl, fg.L2Inner, fg.Domain.from_mesh(pm), [10, 10], ctx=ctx)
    _, _, a1, b1 = gep.upper_coo()
    gep.recompute()
    _, _, a2, b2 = gep.upper_coo()
    assert np.array_equal(a1, a2) and np.array_equal(b1, b2)


def test_galerkin_errors(kat, ctx):
    m = fg.Mesh.from_json(kat["mesh_b"])
    m.global_p_refinement(fg.PRef(2, 2))
    d = fg.Domain.from_mesh(m)
    with pytest.raises(fg.Fem2dError) as e:
        fg.galerkin_sample_gep_hcurl(fg.HierPoly, fg.CurlCurl, fg.L2Inner, d, [3, 8], ctx=ctx)
    assert e.value.code == fg.E_INVALID_GLQ
    dw = fg.Domain.from_mesh(m, fg.ContinuityCondition.HDiv)
    with pytest.raises(fg.Fem2dError) as e:
        fg.galerkin_sample_gep_hcurl(fg.HierPoly, fg.CurlCurl, fg.L2Inner, dw, [8, 8], ctx=ctx)
    assert e.value.code == fg.E_WRONG_CC
    # orders (1,1) everywhere on a single Elem: every spec is on a boundary edge -> no DoFs
    one = fg.Mesh.from_json(kat["mesh_c"])
    with pytest.raises(fg.Fem2dError) as e:
        fg.galerkin_sample_gep_hcurl(fg.HierPoly, fg.CurlCurl, fg.L2Inner, fg.Domain.from_mesh(one), [8, 8], ctx=ctx)
    assert e.value.code == fg.E_EMPTY_DOFS


def test_print_to_petsc_binary_files(oracle_lib, kat, ctx, tmp_path):
    """GEP::print_to_petsc_binary_files (linalg.rs:44-52) from the device-assembled GEP: the two files
    hold exactly the AIJMatrixBinary bytes of the exported CSR, and read back to the same CSR."""
    import os

    n, ref_coo, gep = _assemble_both(oracle_lib, kat["mesh_b"], [("pref", 3, 3, None), ("href", 0, None, -1),
                                                                ("href", 0, [6, 9, 12], -1)], 0, (8, 8), ctx)
    os.makedirs(os.path.join(tmp_path, "tmp"))
    gep.print_to_petsc_binary_files(tmp_path, "p_00000001")
    for which, tag in ((0, "a"), (1, "b")):
        rp, col, val = gep.csr(which)
        rp2, col2, val2 = fg.aij_read(os.path.join(tmp_path, "tmp", "p_00000001_%s.dat" % tag))
        np.testing.assert_array_equal(rp2, rp)
        np.testing.assert_array_equal(col2, col)
        np.testing.assert_array_equal(val2, val)
        sm = oracle_lib.OracleSparseMatrix(n)
        r, c, a, b = gep.upper_coo()
        for i, j, v in zip(r, c, a if which == 0 else b):
            sm.insert((i, j), float(v))
        assert open(os.path.join(tmp_path, "tmp", "p_00000001_%s.dat" % tag), "rb").read() == sm.aij_bytes()
