"""The eigensolve on a full-form HierPoly mesh (monomial bases of orders 3..8, four refinement rounds).

HierPoly and KOLeg span the same discrete space on a mesh, so their Galerkin eigenvalues agree up to
rounding: the KOLeg pencil (well conditioned) is an independent check of the HierPoly pencil (cond(B)
orders of magnitude larger), whose attainable relative residual rises with ||A||. The domain is
[0,2]x[0,1] with PEC walls, whose Maxwell eigenvalues are (m pi / 2)^2 + (k pi)^2.
"""
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


def _solve(ctx, basis, nx, ny):
    w = configs.full_scale(seed=0, nx=nx, ny=ny, rounds=4, fraction=0.3, basis=basis)
    d = fg.Domain.from_mesh(configs.build_mesh(w))
    g = fg.galerkin_sample_gep_hcurl(fg.KOLeg if basis else fg.HierPoly, fg.CurlCurl, fg.L2Inner, d, [10, 10],
                                     ctx=ctx)
    return g, fg.gpu_solve_gep_n(g, 10.0, 20)


def _analytic(k, target=10.0):
    ana = np.sort([(a * np.pi / 2) ** 2 + (b * np.pi) ** 2 for a in range(40) for b in range(20) if a + b > 0])
    return np.sort(ana[np.argsort(np.abs(ana - target), kind="stable")[:k]])


@pytest.mark.parametrize("nx,ny", [(16, 8), (32, 16)])
def test_hierpoly_matches_koleg(ctx, nx, ny):
    g, hp = _solve(ctx, 0, nx, ny)
    _, ko = _solve(ctx, 1, nx, ny)
    assert hp.stats["converged"] and ko.stats["converged"]
    assert hp.stats["block_scaled"] == 1
    assert hp.stats["max_backward_error"] < 1e-10
    vh, vk = np.sort(hp.values), np.sort(ko.values)
    assert np.max(np.abs(vh - vk) / vk) < 1e-10
    assert np.max(np.abs(vh - _analytic(20)) / _analytic(20)) < 1e-5
    # the eigenvectors: B-normalised, residuals recomputed on the host in the original pencil
    A, B = g.scipy()
    X = hp.vectors.T
    th = hp.values
    R = A @ X - (B @ X) * th
    rel = np.linalg.norm(R, axis=0) / (np.abs(th) * np.linalg.norm(B @ X, axis=0))
    assert np.allclose(rel, hp.residuals, rtol=1e-3, atol=1e-14)
    assert np.allclose(np.einsum("ij,ij->j", X, B @ X), 1.0, atol=1e-8)


def test_hierpoly_repeat_solve_is_stable(ctx):
    g, first = _solve(ctx, 0, 16, 8)
    again = fg.gpu_solve_gep_n(g, 10.0, 20)
    assert again.stats["converged"]
    assert np.allclose(np.sort(first.values), np.sort(again.values), rtol=1e-11, atol=0)


def test_scaling_and_damping_options_agree(ctx):
    """Jacobi and row-run block scaling, and the two damping regimes, reach the same eigenvalues."""
    w = configs.precision(seed=1, nx=8, ny=4)
    d = fg.Domain.from_mesh(configs.build_mesh(w))
    g = fg.galerkin_sample_gep_hcurl(fg.KOLeg, fg.CurlCurl, fg.L2Inner, d, [10, 10], ctx=ctx)
    runs = [fg.gpu_solve_gep_n(g, 10.0, 6, scaling=sc, damping=dm) for sc in (1, 2) for dm in (0.05, 1.0)]
    ref = np.sort(runs[0].values)
    for r in runs:
        assert r.stats["converged"]
        assert np.allclose(np.sort(r.values), ref, rtol=1e-11, atol=0)
    assert [r.stats["block_scaled"] for r in runs] == [0, 0, 1, 1]
