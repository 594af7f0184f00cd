"""gpu_solve_gep with iterative inner solves (the KSP solves of the external SLEPc process,
src/fem_problem/linalg/slepc_solve.rs:26-36): T's SPD system A + |s| B by preconditioned CG and its
indefinite system A - s B by preconditioned MINRES, with the plain additive-Schwarz preconditioner
(precond 1) or the learned two-level preconditioner of a PatchNet (precond 2). Both must give the
eigenpairs of the exact (multifrontal) path: eigenvalues within 1e-9 relative, residuals below the
outer solver's acceptance level (relative residual 1e-10, or a settled pair with backward error below
1e-11 in the scaled pencil, reported here in the original one), on a mesh of the learned-preconditioner
family."""
import numpy as np
import pytest

import fem_2d_gb300 as fg
from fem_2d_gb300 import configs

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gep():
    ctx = fg.Context(0)
    w = configs.learned_family(4, 8, 4)
    d = fg.Domain.from_mesh(configs.build_mesh(w))
    return fg.galerkin_sample_gep_hcurl(fg.KOLeg, fg.CurlCurl, fg.L2Inner, d, [10, 10], ctx=ctx)


@pytest.fixture(scope="module")
def exact(gep):
    return fg.gpu_solve_gep_n(gep, 10.0, 10)


def test_plain_inner_solves_match_exact(gep, exact):
    r = fg.gpu_solve_gep_n(gep, 10.0, 10, precond=fg.PRECOND_PLAIN)
    assert np.max(np.abs(np.sort(r.values) - np.sort(exact.values)) / np.abs(np.sort(exact.values))) <= 1e-9
    assert np.max(r.residuals) <= 1e-7 and r.stats["max_backward_error"] <= 1e-10
    assert r.stats["inner_cg_iters"] > 0 and r.stats["inner_minres_iters"] > 0
    assert r.stats["inner_max_relres"] <= 1e-10
    print("plain inner:", r.stats)


def test_learned_inner_solves_match_exact(gep, exact):
    net = fg.PatchNet(k=8, hidden=32, seed=3)
    r = fg.gpu_solve_gep_n(gep, 10.0, 10, precond=fg.PRECOND_LEARNED, net=net)
    assert np.max(np.abs(np.sort(r.values) - np.sort(exact.values)) / np.abs(np.sort(exact.values))) <= 1e-9
    assert np.max(r.residuals) <= 1e-7 and r.stats["max_backward_error"] <= 1e-10
    print("learned inner (untrained net):", r.stats)


def test_learned_needs_a_network(gep):
    with pytest.raises(fg.Fem2dError) as e:
        fg.gpu_solve_gep_n(gep, 10.0, 4, precond=fg.PRECOND_LEARNED)
    assert e.value.code == fg.E_INVALID_ARG
