"""Device field evaluation (fem2d_fields_*, UniformFieldSpace) against the oracle's restatement of
xy_fields (fields.rs:63-122) and the reference's own test flow (src/lib.rs:85-120: slepc eigenvector ->
xy_fields -> expression_2arg -> print_all_to_vtk).

Tolerance: FIELD_TOL relative to the largest field magnitude (FP64 shape functions evaluated by a
different routine; the sums run in the reference's order with unfused multiplies and adds).
"""
import os

import numpy as np
import pytest

import fem_2d_gb300 as fg
from fem_2d_gb300 import configs

pytestmark = pytest.mark.gpu
FIELD_TOL = 1e-12


@pytest.fixture(scope="module")
def ctx():
    from fem_2d_gb300 import build

    build.build()
    return fg.Context(0)


def _both(oracle_lib, w):
    om = oracle_lib.OracleMesh(w.mesh_json)
    om.apply_ops(w.ops)
    om.domain()
    pm = configs.build_mesh(w)
    dom = fg.Domain.from_mesh(pm)
    assert dom.num_dofs == om.ndofs
    return om, dom


def _rel(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def _kat_slepc_workload(kat):
    k = kat["kat_slepc_problem"]
    return configs.Workload("kat_slepc", kat[k["mesh"]], [("pref", 3, 3, None), ("href", 0, None, -1),
                                                         ("href", 0, [6, 9, 12], -1)], basis=0)


def test_fields_slepc_eigenvector(oracle_lib, kat, ctx, tmp_path):
    """src/lib.rs:85-120 with the reference's stored eigenvector (test_input/test_evec.dat)."""
    w = _kat_slepc_workload(kat)
    om, dom = _both(oracle_lib, w)
    evec = np.asarray(kat["slepc_evec"])
    pair = fg.EigenPair(kat["slepc_eval"], evec)
    sol = pair.normalized_eigenvector()
    ufs = fg.UniformFieldSpace(dom, [8, 8], ctx=ctx)
    names = ufs.xy_fields(fg.HierPoly, "E", sol)
    assert names == ["E_x", "E_y"]
    ox, oy = om.xy_fields(sol, 8, 8, basis=0)
    assert _rel(ufs.quantity("E_x"), ox) <= FIELD_TOL
    assert _rel(ufs.quantity("E_y"), oy) <= FIELD_TOL
    ufs.expression_2arg(names, "E_mag", lambda ex, ey: (ex ** 2 + ey ** 2) ** 0.5)
    np.testing.assert_allclose(ufs.quantity("E_mag"), np.hypot(ox, oy), rtol=1e-12, atol=1e-14)
    ufs.map_to_quantity("E_x", "X_abs", abs)
    path = os.path.join(tmp_path, "mesh_b_fields.vtk")
    ufs.print_all_to_vtk(path)
    text = open(path).read()
    nl = len(ufs.leaves)
    assert text.startswith("# vtk DataFile Version 3.0\n")
    assert "DATASET UNSTRUCTURED_GRID" in text
    assert "POINTS %d double" % (64 * nl) in text
    assert "CELLS %d %d" % (49 * nl, 5 * 49 * nl) in text
    assert "POINT_DATA %d" % (64 * nl) in text
    for q in ("E_x", "E_y", "E_mag", "X_abs"):
        assert "SCALARS %s double 1 \nLOOKUP_TABLE default\n" % q in text
    vals = text.split("SCALARS E_y double 1 \nLOOKUP_TABLE default\n")[1].split("SCALARS")[0].split()
    np.testing.assert_allclose(np.asarray(vals, dtype=float), oy.ravel(), rtol=0, atol=1e-14)


@pytest.mark.parametrize("make,dens", [
    (configs.waveguide_small, (9, 9)),
    (lambda: configs.precision(seed=0, nx=4, ny=2, order=3, rounds=2), (7, 7)),
    (lambda: configs.precision(seed=3, nx=4, ny=2, order=6, rounds=3), (9, 5)),
    (lambda: configs.batch_member(7), (5, 9)),
    (lambda: configs.batch_member(21), (2, 2)),
])
def test_fields_vs_oracle_random(oracle_lib, ctx, make, dens):
    w = make()
    om, dom = _both(oracle_lib, w)
    sol = np.random.default_rng(5).standard_normal(dom.num_dofs)
    bs = fg.KOLeg if w.basis == 1 else fg.HierPoly
    ufs = fg.UniformFieldSpace(dom, dens, ctx=ctx)
    xn, yn = ufs.xy_fields(bs, "F", sol)
    ox, oy = om.xy_fields(sol, dens[0], dens[1], basis=w.basis)
    assert ufs.quantity(xn).shape == ox.shape
    assert _rel(ufs.quantity(xn), ox) <= FIELD_TOL
    assert _rel(ufs.quantity(yn), oy) <= FIELD_TOL


def test_fields_full_size_continuity(oracle_lib, ctx):
    """The 1,070,625-DoF KOLeg workload (18,502 leaves): tangential continuity of the device fields for
    a random coefficient vector, a size-independent property (the oracle is not run at this size)."""
    w = configs.full_scale(seed=0, basis=1, fraction=0.44)
    dom = fg.Domain.from_mesh(configs.build_mesh(w))
    assert dom.num_dofs == 1070625
    sol = np.random.default_rng(2).standard_normal(dom.num_dofs)
    ufs = fg.UniformFieldSpace(dom, (5, 5), ctx=ctx)
    xn, yn = ufs.xy_fields(fg.KOLeg, "F", sol)
    leaves, bounds = ufs._geometry()
    assert len(leaves) == 18502
    jump, count = oracle_lib.tangential_jumps(bounds, ufs.quantity(xn), ufs.quantity(yn))
    assert count > 50000
    assert jump <= 1e-11


def test_fields_device_pointers(oracle_lib, ctx):
    torch = pytest.importorskip("torch")
    w = configs.waveguide_small()
    om, dom = _both(oracle_lib, w)
    sol = np.random.default_rng(9).standard_normal(dom.num_dofs)
    ufs = fg.UniformFieldSpace(dom, (6, 6), ctx=ctx)
    dev = ufs._device(fg.HierPoly)
    nl = dev.num_leaves
    ds = torch.tensor(sol, dtype=torch.float64, device="cuda:0")
    dx = torch.empty(nl * 36, dtype=torch.float64, device="cuda:0")
    dy = torch.empty_like(dx)
    torch.cuda.synchronize()
    dev.xy_device(ds.data_ptr(), dom.num_dofs, dx.data_ptr(), dy.data_ptr())
    ctx.synchronize()
    ox, oy = om.xy_fields(sol, 6, 6)
    assert _rel(dx.cpu().numpy().reshape(ox.shape), ox) <= FIELD_TOL
    assert _rel(dy.cpu().numpy().reshape(oy.shape), oy) <= FIELD_TOL


def test_fields_errors(ctx):
    w = configs.waveguide_small()
    dom = fg.Domain.from_mesh(configs.build_mesh(w))
    ufs = fg.UniformFieldSpace(dom, (4, 4), ctx=ctx)
    with pytest.raises(fg.UniformFieldError, match="does not match solution size"):
        ufs.xy_fields(fg.HierPoly, "E", np.zeros(dom.num_dofs + 1))
    with pytest.raises(fg.UniformFieldError, match="Missing quantity"):
        ufs.expression_2arg(["A", "B"], "C", lambda a, b: a + b)
    with pytest.raises(fg.UniformFieldError):
        fg.UniformFieldSpace(dom, (1, 4), ctx=ctx)
    # the C entry point checks the size too
    dev = ufs._device(fg.HierPoly)
    with pytest.raises(fg.Fem2dError, match="does not match solution size"):
        dev.xy(np.zeros(3), 4, 4)
