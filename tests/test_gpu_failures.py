"""The solvers' failure modes, driven from the host (no GPU fault, trap or hang is provoked).

The reference maps its solver failures to error variants: FailedToInvertB, SpuriouslyConverged and
ProblemTooLarge in nalgebra_solve_gep (src/fem_problem/linalg/nalgebra_solve.rs:14-26, 52-77) and
FailedToConverge among SLEPc's exit codes (src/fem_problem/linalg/slepc_solve.rs:47-55). Here each one
is provoked with host data: an iteration cap, a B with a negative diagonal entry, an A of zeros, a
non-finite input value, and a GEP too large for the allocation-free path, each through the GEP's
public matrices (fem2d_gep_set_upper_values, the reference's `pub a`/`pub b` fields)."""
import numpy as np
import pytest

import fem_2d_gb300 as fg
from fem_2d_gb300 import configs

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    return fg.Context(0)


def _small(ctx, seed=1):
    w = configs.precision(seed=seed, nx=6, ny=3)
    d = fg.Domain.from_mesh(configs.build_mesh(w))
    return fg.galerkin_sample_gep_hcurl(fg.KOLeg, fg.CurlCurl, fg.L2Inner, d, list(w.glq), ctx=ctx)


def _waveguide(ctx):
    w = configs.waveguide_small()
    d = fg.Domain.from_mesh(configs.build_mesh(w))
    return fg.galerkin_sample_gep_hcurl(fg.HierPoly, fg.CurlCurl, fg.L2Inner, d, list(w.glq), ctx=ctx)


def _code(fn):
    with pytest.raises(fg.Fem2dError) as e:
        fn()
    return e.value.code


def test_iteration_cap_is_not_converged(ctx):
    g = _small(ctx)
    assert _code(lambda: fg.gpu_solve_gep_n(g, 10.0, 10, max_outer=1, krylov_steps=1, tol=1e-14)) == fg.E_NOT_CONVERGED
    # the same GEP still solves with the default cap afterwards (the context stays usable)
    r = fg.gpu_solve_gep_n(g, 10.0, 4)
    assert np.all(r.residuals < 1e-8)


def _negative_b_diagonal(g):
    r, c, a, b = g.upper_coo()
    d = np.nonzero(r == c)[0][len(np.nonzero(r == c)[0]) // 2]
    b = b.copy()
    b[d] = -1e3 * np.max(np.abs(b))
    g.set_upper_values(a, b)


def test_b_not_spd_dense(ctx):
    g = _waveguide(ctx)
    _negative_b_diagonal(g)
    assert _code(lambda: fg.nalgebra_solve_gep(g, 10.0)) == fg.E_B_NOT_SPD


def test_b_not_spd_sparse_and_shifted(ctx):
    g = _small(ctx)
    _negative_b_diagonal(g)
    assert _code(lambda: fg.gpu_solve_gep_n(g, 10.0, 4)) == fg.E_B_NOT_SPD
    rhs = np.ones((g.dimension, 1))
    assert _code(lambda: g.shifted_solve(0.0, 1.0, rhs, spd=True)) == fg.E_B_NOT_SPD


def test_zero_a_is_spurious(ctx):
    for g, solve in ((_waveguide(ctx), lambda g: fg.nalgebra_solve_gep(g, 10.0)),
                     (_small(ctx), lambda g: fg.gpu_solve_gep_n(g, 10.0, 4))):
        r, c, a, b = g.upper_coo()
        g.set_upper_values(np.zeros_like(a), b)
        assert _code(lambda: solve(g)) == fg.E_SPURIOUS


def test_non_finite_values_rejected(ctx):
    g = _small(ctx)
    r, c, a, b = g.upper_coo()
    for bad in (np.nan, np.inf):
        a2 = a.copy()
        a2[len(a2) // 3] = bad
        assert _code(lambda: g.set_upper_values(a2, b)) == fg.E_INVALID_ARG
    # rejected values leave the GEP as it was
    _, _, a3, b3 = g.upper_coo()
    assert np.array_equal(a3, a) and np.array_equal(b3, b)


def test_set_values_round_trip(ctx):
    g = _small(ctx)
    r, c, a, b = g.upper_coo()
    g.set_upper_values(2.0 * a, 3.0 * b)
    _, _, a2, b2 = g.upper_coo()
    assert np.array_equal(a2, 2.0 * a) and np.array_equal(b2, 3.0 * b)
    g.recompute()
    _, _, a3, b3 = g.upper_coo()
    assert np.array_equal(a3, a) and np.array_equal(b3, b)
