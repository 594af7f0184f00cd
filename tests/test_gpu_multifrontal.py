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
