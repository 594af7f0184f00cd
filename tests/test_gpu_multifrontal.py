"""The device multifrontal LU of the shifted pencil: residuals of (c_a A + c_b B) X = R (FP64)."""
import numpy as np
import pytest

import fem_2d_gb300 as fg
from fem_2d_gb300 import configs

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from fem_2d_gb300 import build

    build.build()
    return fg.Context(0)


@pytest.mark.parametrize("name,ca,cb,spd", [("kat_b", 1.0, -1.475, False), ("kat_b", 1.0, 0.07, True),
                                            ("prec", 1.0, -10.0, False), ("prec", 0.0, 1.0, True),
                                            ("batch", 1.0, -10.0, False)])
def test_shifted_solve_residual(kat, ctx, name, ca, cb, spd):
    if name == "kat_b":
        mj, ops, basis, glq = kat["mesh_b"], [("pref", 3, 3, None), ("href", 0, None, -1),
                                              ("href", 0, [6, 9, 12], -1)], 0, (8, 8)
    elif name == "prec":
        w = configs.precision(seed=0, nx=6, ny=3)
        mj, ops, basis, glq = w.mesh_json, w.ops, w.basis, w.glq
    else:
        w = configs.batch_member(3)
        mj, ops, basis, glq = w.mesh_json, w.ops, w.basis, w.glq
    pm = fg.Mesh.from_json(mj)
    configs.apply_ops(pm, ops)
    gep = fg.galerkin_sample_gep_hcurl(fg.KOLeg if basis else fg.HierPoly, fg.CurlCurl, fg.L2Inner,
                                       fg.Domain.from_mesh(pm), list(glq), ctx=ctx)
    A, B = gep.scipy()
    K = ca * A + cb * B
    R = np.random.default_rng(0).standard_normal((gep.dimension, 5))
    X = gep.shifted_solve(ca, cb, R, spd=spd)
    rel = np.linalg.norm(K @ X - R, axis=0) / np.linalg.norm(R, axis=0)
    import scipy.sparse.linalg as sla

    Xs = sla.splu(K.tocsc()).solve(R)
    rels = np.linalg.norm(K @ Xs - R, axis=0) / np.linalg.norm(R, axis=0)
    assert np.max(rel) <= max(1e-9, 100 * np.max(rels)), (rel, rels)


@pytest.mark.parametrize("ca,cb,spd", [(1.0, -10.0, False), (1.0, 10.0, True)])
def test_shifted_solve_wide_fronts(ctx, ca, cb, spd):
    """A 389,566-DoF full-form mesh whose top separator fronts have p > 160: the narrow upper levels are
    solved through the fronts' partitioned inverses (the wide ones inverted column-parallel); the
    normwise backward error ||K X - R|| / (||K|| ||X|| + ||R||) stays at the FP64 level."""
    w = configs.full_scale(seed=0, basis=0, nx=64, ny=32, rounds=1, fraction=0.44)
    dom = fg.Domain.from_mesh(configs.build_mesh(w))
    fronts = fg.factor_plan(dom)["fronts"]
    assert np.max(fronts[:, 3]) > 160   # the case the wide inversion covers
    gep = fg.galerkin_sample_gep_hcurl(fg.HierPoly, fg.CurlCurl, fg.L2Inner, dom, list(w.glq), ctx=ctx)
    A, B = gep.scipy()
    K = (ca * A + cb * B).tocsr()
    R = np.random.default_rng(1).standard_normal((gep.dimension, 4))
    X = gep.shifted_solve(ca, cb, R, spd=spd)
    knorm = np.max(np.asarray(abs(K).sum(axis=1)).ravel())
    bwd = np.max(np.abs(K @ X - R), axis=0) / (knorm * np.max(np.abs(X), axis=0) + np.max(np.abs(R), axis=0))
    assert np.all(np.isfinite(X))
    assert np.max(bwd) < 1e-13, bwd
