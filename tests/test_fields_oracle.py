"""Field evaluation (UniformFieldSpace::xy_fields, fields.rs:63-122): the oracle's restatement checked
against properties the reference's discrete space guarantees, on the CPU.

* tangential continuity: the H(curl) space of an RBS mesh is conforming, so the tangential field is
  continuous across every interior line, hanging edges included, for ANY coefficient vector;
* the TE10 mode of the [0,1]x[0,0.5] waveguide (README.md:45-61 mesh, eigenvalue pi^2) has
  E = y_hat * sin(pi x), which the discrete eigenvector's fields must reproduce;
* MismatchedSolutionSize (fields.rs:68-72).
"""
import numpy as np
import pytest

import fem_2d_gb300 as fg
from fem_2d_gb300 import configs


def _oracle_and_geometry(oracle_lib, w):
    om = oracle_lib.OracleMesh(w.mesh_json)
    om.apply_ops(w.ops)
    n = om.domain()
    pm = configs.build_mesh(w)   # host-only Mesh (geometry of the leaves)
    info = pm.elem_info()
    leaves = np.nonzero(info[:, 0] == 1)[0]
    return om, n, pm.elem_bounds()[leaves]


@pytest.mark.parametrize("make,dens", [
    (configs.waveguide_small, (9, 9)),
    (lambda: configs.precision(seed=0, nx=4, ny=2, order=3, rounds=2), (7, 7)),
    (lambda: configs.precision(seed=3, nx=4, ny=2, order=5, rounds=3), (9, 5)),
    (lambda: configs.batch_member(7), (5, 9)),
])
def test_oracle_fields_tangential_continuity(oracle_lib, make, dens):
    w = make()
    om, n, bounds = _oracle_and_geometry(oracle_lib, w)
    sol = np.random.default_rng(11).standard_normal(n)
    ex, ey = om.xy_fields(sol, dens[0], dens[1], basis=w.basis)
    assert ex.shape == (len(bounds), dens[0], dens[1])
    jump, count = oracle_lib.tangential_jumps(bounds, ex, ey)
    assert count > 0
    assert jump <= 1e-13


def test_oracle_fields_te10(oracle_lib):
    w = configs.waveguide_small()
    om, n, bounds = _oracle_and_geometry(oracle_lib, w)
    r, c, a, b = om.galerkin(w.basis, *w.glq)
    A, B = oracle_lib.full_sym(n, r, c, a), oracle_lib.full_sym(n, r, c, b)
    vals, vecs = oracle_lib.gep_exact_dense(A, B, w.target)
    assert abs(vals[0] - np.pi ** 2) < 1e-3
    vec = vecs[:, 0] / np.linalg.norm(vecs[:, 0])   # normalized_eigenvector (linalg.rs:93-96)
    d = 9
    ex, ey = om.xy_fields(vec, d, d, basis=w.basis)
    xs = bounds[:, 0:1] + np.linspace(0, 1, d)[None, :] * (bounds[:, 2:3] - bounds[:, 0:1])
    s = np.repeat(np.sin(np.pi * xs)[:, :, None], d, axis=2)
    cfit = float((ey * s).sum() / (s * s).sum())
    assert np.max(np.abs(ex)) <= 1e-4 * np.max(np.abs(ey))
    assert np.linalg.norm(ey - cfit * s) <= 1e-4 * np.linalg.norm(ey)


def test_oracle_fields_mismatched_size(oracle_lib):
    w = configs.waveguide_small()
    om, n, _ = _oracle_and_geometry(oracle_lib, w)
    with pytest.raises(RuntimeError, match="MismatchedSolutionSize"):
        om.xy_fields(np.zeros(n + 1), 4, 4)
