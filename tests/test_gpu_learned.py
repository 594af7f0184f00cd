"""The learned per-Elem-patch preconditioner of the inner PCG solver (fem_2d_gb300/learned.py).

* The device forward/backward kernels agree with the FP64 numpy oracle (oracle/patchnet_ref.py, itself
  pinned by finite differences): loss within 1e-5 relative, gradient within 1e-3 relative (FP32 network).
* Plain PCG (additive Schwarz over Elem patches) solves K = A + 10 B to 1e-10 (checked with the GEP's
  own A and B on the host).
* A network trained on the GPU on error vectors the plain solver produced for three seeds of the
  learned-preconditioner family is evaluated on a held-out seed: its held-out loss is below the
  untrained network's, and the two-level PCG reaches the same tolerance in fewer iterations than the
  plain method. A caller-given coarse basis (the principal directions of the test mesh's own errors)
  shows the ceiling of this coarse-space form.
"""
import numpy as np
import pytest

import fem_2d_gb300 as fg
from fem_2d_gb300 import configs

pytestmark = pytest.mark.gpu
SHIFT = 10.0


@pytest.fixture(scope="module")
def ctx():
    from fem_2d_gb300 import build

    build.build()
    return fg.Context(0)


def _gep(ctx, seed, nx=8, ny=4):
    w = configs.learned_family(seed, nx, ny)
    d = fg.Domain.from_mesh(configs.build_mesh(w))
    return d, fg.galerkin_sample_gep_hcurl(fg.KOLeg, fg.CurlCurl, fg.L2Inner, d, [10, 10], ctx=ctx)


def test_gradient_matches_oracle(ctx):
    from oracle import patchnet_ref as pr

    d, g = _gep(ctx, 0, 4, 2)
    net = fg.PatchNet(k=8, hidden=32, seed=1)
    E = np.random.default_rng(0).standard_normal((16, g.dimension))
    loss, grad = net.loss_grad(g, SHIFT, E)
    ptr, dof, feat, wt = fg.patch_features(d, SHIFT)
    rl, rg = pr.loss_grad(net.get_params(), feat, ptr, dof, E, 32, 8)
    assert abs(loss - rl) <= 1e-5 * abs(rl)
    assert np.linalg.norm(grad - rg) <= 1e-3 * np.linalg.norm(rg)


def test_plain_pcg_solves_shifted_system(ctx):
    d, g = _gep(ctx, 4)
    rhs = np.random.default_rng(5).standard_normal((g.dimension, 4))
    x, st = fg.PCG(g, 1.0, SHIFT).solve(rhs, tol=1e-10)
    assert st["converged"] and st["relres"] <= 1e-10 and st["coarse_dim"] == 0
    A, B = g.scipy()
    res = np.linalg.norm((A + SHIFT * B) @ x - rhs, axis=0) / np.linalg.norm(rhs, axis=0)
    assert res.max() <= 1e-9
    with pytest.raises(fg.Fem2dError) as e:
        fg.PCG(g, 1.0, -SHIFT)
    assert e.value.code == fg.E_INVALID_ARG


def test_trained_network_gains_over_plain(ctx):
    train = [_gep(ctx, s) for s in (1, 2, 3)]
    d, g = _gep(ctx, 4)
    samples = []
    for _, gt in train:
        E = fg.harvest_errors(gt, 1.0, SHIFT, nrhs=16, every=2, max_samples=256, seed=1, first=150)
        samples.append(np.vstack([E] * (256 // len(E) + 1))[:256])
    net = fg.PatchNet(k=16, hidden=192, seed=0)
    E_test = fg.harvest_errors(g, 1.0, SHIFT, nrhs=16, every=2, max_samples=256, seed=3, first=150)
    loss0, _ = net.loss_grad(g, SHIFT, E_test)
    hist = net.train([gt for _, gt in train], SHIFT, samples, epochs=400, lr=2e-3)
    assert hist[-1] < hist[0]
    loss1, _ = net.loss_grad(g, SHIFT, E_test)
    assert loss1 < loss0
    rhs = np.random.default_rng(7).standard_normal((g.dimension, 8))
    _, plain = fg.PCG(g, 1.0, SHIFT).solve(rhs, tol=1e-10)
    x, learned = fg.PCG(g, 1.0, SHIFT, net).solve(rhs, tol=1e-10)
    assert learned["converged"] and learned["coarse_dim"] == 16 * (len(fg.patch_features(d, SHIFT)[0]) - 1)
    A, B = g.scipy()
    res = np.linalg.norm((A + SHIFT * B) @ x - rhs, axis=0) / np.linalg.norm(rhs, axis=0)
    assert res.max() <= 1e-9
    print("plain", plain, "learned", learned, "held-out loss", loss0, "->", loss1)
    assert learned["iters"] < plain["iters"]


def test_caller_basis_ceiling(ctx):
    d, g = _gep(ctx, 4)
    E = fg.harvest_errors(g, 1.0, SHIFT, nrhs=16, every=2, max_samples=256, seed=3, first=150)
    ptr, dof, feat, wt = fg.patch_features(d, SHIFT)
    Z = np.zeros((len(dof), 16), np.float32)
    for p in range(len(ptr) - 1):
        r0, r1 = ptr[p], ptr[p + 1]
        _, _, Vt = np.linalg.svd(E[:, dof[r0:r1]], full_matrices=False)
        Z[r0:r1, : min(16, Vt.shape[0])] = Vt[:16].T
    rhs = np.random.default_rng(7).standard_normal((g.dimension, 8))
    _, plain = fg.PCG(g, 1.0, SHIFT).solve(rhs, tol=1e-10)
    _, best = fg.PCG(g, 1.0, SHIFT, basis=Z).solve(rhs, tol=1e-10)
    assert best["converged"]
    assert best["iters"] < 0.75 * plain["iters"]
