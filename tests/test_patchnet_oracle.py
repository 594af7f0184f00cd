"""The learned preconditioner's CPU oracle (oracle/patchnet_ref.py) pinned by finite differences, and the
host-side patch features of a Domain (no GPU needed)."""
import numpy as np
import pytest

import fem_2d_gb300 as fg
from fem_2d_gb300 import configs
from oracle import patchnet_ref as pr


def _toy(seed=0, nin=16, hidden=12, k=3, P=5, S=7, n=40):
    rng = np.random.default_rng(seed)
    sizes = rng.integers(4, 9, P)
    ptr = np.concatenate([[0], np.cumsum(sizes)])
    dof = np.concatenate([rng.choice(n, s, replace=False) for s in sizes]).astype(np.int64)
    X = rng.standard_normal((ptr[-1], nin))
    npar = nin * hidden + hidden + hidden * hidden + hidden + hidden * k + k
    params = rng.standard_normal(npar) * 0.3
    E = rng.standard_normal((S, n))
    return params, X, ptr, dof, E, hidden, k


def test_oracle_gradient_matches_finite_differences():
    params, X, ptr, dof, E, hidden, k = _toy()
    loss, g = pr.loss_grad(params, X, ptr, dof, E, hidden, k)
    assert 0.0 < loss < 1.0
    rng = np.random.default_rng(1)
    for idx in rng.choice(params.size, 25, replace=False):
        h = 1e-6
        pp, pm = params.copy(), params.copy()
        pp[idx] += h
        pm[idx] -= h
        fd = (pr.loss_only(pp, X, ptr, dof, E, hidden, k) - pr.loss_only(pm, X, ptr, dof, E, hidden, k)) / (2 * h)
        assert abs(fd - g[idx]) <= 1e-6 * max(1.0, abs(fd)) + 1e-9, (idx, fd, g[idx])


def test_loss_is_zero_when_errors_lie_in_the_span():
    params, X, ptr, dof, E, hidden, k = _toy(seed=3)
    _, _, Z = pr.forward(params, X, hidden, k)
    # build samples whose restriction to patch 0 is a combination of its k vectors, zero elsewhere
    n = E.shape[1]
    E2 = np.zeros((4, n))
    r0, r1 = ptr[0], ptr[1]
    rng = np.random.default_rng(0)
    for s in range(4):
        E2[s, dof[r0:r1]] = Z[r0:r1] @ rng.standard_normal(k)
    loss, _ = pr.loss_grad(params, X, ptr[:2], dof, E2, hidden, k, lam=1e-14)
    assert loss < 1e-10


def test_patch_features_of_a_domain():
    w = configs.learned_family(seed=0, nx=4, ny=2)
    dom = fg.Domain.from_mesh(configs.build_mesh(w))
    ptr, dof, feat, wt = fg.patch_features(dom, 10.0)
    specs = dom.basis_specs()
    assert ptr[-1] == len(specs) == len(dof) == len(feat)
    assert np.array_equal(np.sort(np.unique(dof)), np.arange(dom.num_dofs))
    # partition of unity over the rows of each DoF
    tot = np.zeros(dom.num_dofs)
    np.add.at(tot, dof, wt)
    assert np.allclose(tot, 1.0)
    assert np.all(np.isfinite(feat)) and feat.shape[1] == 16
    assert set(np.unique(feat[:, 0])) <= {0.0, 1.0}
