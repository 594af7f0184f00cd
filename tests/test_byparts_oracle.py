"""The oracle's integrate_by_parts restatement (integrals.rs:94-237, 356-418) on the CPU.

Integration by parts is exact under the quadrature (every integrand is a polynomial of degree below
2 nq), so for every Galerkin visit the CurlCurl face term plus its four edge terms equals the
CurlCurl integral of the integrate path, which the oracle pins against the reference's golden values;
the by-parts L2Inner value equals the integrate path's (same interior points). The split itself is
not trivial: both the face and the edge terms carry weight.
"""
import numpy as np
import pytest

from fem_2d_gb300 import configs
from oracle import ref


@pytest.mark.parametrize("basis", [ref.HIERPOLY, ref.KOLEG])
@pytest.mark.parametrize("seed", [0, 3])
def test_by_parts_sums_to_integrate(basis, seed):
    w = configs.precision(seed=seed, nx=2, ny=1)
    om = ref.OracleMesh(w.mesh_json)
    om.apply_ops(w.ops)
    om.domain()
    r, c, a, b = om.galerkin(basis, 10, 10)
    rb, cb, v = om.galerkin_by_parts(basis, 10, 10)
    assert np.array_equal(r, rb) and np.array_equal(c, cb)
    full = v[:, 0] + v[:, 1:5].sum(axis=1)
    assert np.max(np.abs(full - a)) <= 1e-12 * np.max(np.abs(a))
    assert np.max(np.abs(v[:, 5] - b)) <= 1e-13 * np.max(np.abs(b))
    assert np.max(np.abs(v[:, 1:5])) > 1e-3 * np.max(np.abs(a))
    assert np.max(np.abs(v[:, 0] - a)) > 1e-3 * np.max(np.abs(a))


def test_quadratures_match_reference_doc_examples():
    """glq.rs:36-52 and 79-100: with 10 GLQ points plus the endpoints, the interior sum of u^2 v^2 is 4/9
    and each edge sum 2/3."""
    out = ref.quad_doc(10)
    assert abs(out[0] - 4.0 / 9.0) < 1e-12
    assert np.all(np.abs(out[1:] - 2.0 / 3.0) < 1e-12)
