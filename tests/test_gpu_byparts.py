"""integrate_by_parts over the Galerkin visit set on the device (fem2d_gep_by_parts) against the
oracle's restatement of integrals.rs:94-237 and 356-418, component by component, and the by-parts
identity (face + edges = A) on the device's own output."""
import numpy as np
import pytest

import fem_2d_gb300 as fg
from fem_2d_gb300 import configs
from oracle import ref

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from fem_2d_gb300 import build

    build.build()
    return fg.Context(0)


@pytest.mark.parametrize("basis", [ref.HIERPOLY, ref.KOLEG])
def test_by_parts_against_oracle(ctx, basis):
    w = configs.precision(seed=3, nx=2, ny=1)
    d = fg.Domain.from_mesh(configs.build_mesh(w))
    g = fg.galerkin_sample_gep_hcurl(fg.KOLeg if basis else fg.HierPoly, fg.CurlCurl, fg.L2Inner, d, [10, 10], ctx=ctx)
    r, c, v = g.by_parts()
    om = ref.OracleMesh(w.mesh_json)
    om.apply_ops(w.ops)
    om.domain()
    ro, co, vo = om.galerkin_by_parts(basis, 10, 10)
    assert np.array_equal(r, ro) and np.array_equal(c, co)
    for k in range(6):
        scale = np.max(np.abs(vo[:, k])) if k in (0, 5) else np.max(np.abs(vo[:, 1:5]))
        assert np.max(np.abs(v[:, k] - vo[:, k])) <= 1e-12 * scale, k
    _, _, a, _ = g.upper_coo()
    assert np.max(np.abs(v[:, 0] + v[:, 1:5].sum(axis=1) - a)) <= 1e-12 * np.max(np.abs(a))
