"""Host-side parity (no GPU): the native mesh and DoF enumeration against the oracle, bit-exact.

Domain::from_mesh (domain.rs:69-159) is integer work; every (elem, elem_idx, i, j, dir, dof) tuple of
Domain::basis_specs must match, on the reference's own test meshes and on seeded workloads.
"""
import json
import os
import re

import numpy as np
import pytest

import fem_2d_gb300 as fg
from fem_2d_gb300 import configs

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def native():
    from fem_2d_gb300 import build

    build.build()
    return fg.lib()


def _compare(ref, mesh_json, ops, check_pattern=True):
    om = ref.OracleMesh(mesh_json)
    om.apply_ops(ops)
    pm = fg.Mesh.from_json(mesh_json)
    configs.apply_ops(pm, ops)
    assert np.array_equal(om.elem_info(), pm.elem_info())
    nd = om.domain()
    pd = fg.Domain.from_mesh(pm)
    assert pd.num_dofs == nd
    assert np.array_equal(om.specs(), pd.basis_specs())
    if check_pattern:
        r, c, _, _ = om.galerkin(ref.HIERPOLY, 4, 4)
        pr, pc = fg.domain_pattern(pd)
        assert np.array_equal(r, pr) and np.array_equal(c, pc)
    return nd


def test_abi_exports_every_declared_symbol(native):
    with open(os.path.join(ROOT, "include", "fem2d_gb300.h")) as f:
        hdr = f.read()
    names = set(re.findall(r"\b(fem2d_[a-z0-9_]+)\s*\(", hdr))
    assert len(names) > 30
    for n in sorted(names):
        assert hasattr(native, n), n


def test_kat_meshes(native, oracle_lib, kat):
    ref = oracle_lib
    n = _compare(ref, kat["mesh_b"], [("pref", 3, 3, None), ("href", 0, None, -1), ("href", 0, [6, 9, 12], -1)])
    assert n == 624
    _compare(ref, kat["mesh_a"], [("pref", 2, 2, None)])
    # domain.rs:392-412 create_domain test sequence
    _compare(ref, kat["mesh_a"], [("orders", 5, 5, None), ("href", 0, None, -1), ("href", 0, [4, 5], -1),
                                  ("href", 1, [6, 7], -1), ("href", 2, [8, 9], -1), ("pref", 2, -1, [10, 11, 12, 13])])
    _compare(ref, kat["mesh_c"], [("orders", 3, 4, None), ("href", 1, None, 1), ("href", 0, None, -1)])


def test_unit_mesh(native, oracle_lib):
    ref = oracle_lib
    om = ref.OracleMesh()
    om.set_orders(3, 2)
    om.h_refine(ref.HREF_T)
    om.h_refine(ref.HREF_V, ids=[2])
    pm = fg.Mesh.unit()
    pm.set_global_expansion_orders(fg.Orders(3, 2))
    pm.global_h_refinement(fg.HRef.T)
    pm.h_refine_elems([2], fg.HRef.V)
    assert np.array_equal(om.elem_info(), pm.elem_info())
    assert om.domain() == fg.Domain.from_mesh(pm).num_dofs
    assert np.array_equal(om.specs(), fg.Domain.from_mesh(pm).basis_specs())


def test_waveguide_small(native, oracle_lib):
    w = configs.waveguide_small()
    n = _compare(oracle_lib, w.mesh_json, w.ops)
    assert 100 < n < 1000


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_precision_family(native, oracle_lib, seed):
    w = configs.precision(seed=seed, nx=6, ny=3)
    _compare(oracle_lib, w.mesh_json, w.ops)


@pytest.mark.parametrize("seed", [0, 3])
def test_full_scale_family_small(native, oracle_lib, seed):
    w = configs.full_scale(seed=seed, nx=8, ny=4, rounds=3)
    _compare(oracle_lib, w.mesh_json, w.ops)


@pytest.mark.parametrize("seed", range(6))
def test_batch_family(native, oracle_lib, seed):
    w = configs.batch_member(seed)
    _compare(oracle_lib, w.mesh_json, w.ops)


def test_refinement_errors(native, kat):
    m = fg.Mesh.from_json(kat["mesh_a"])
    with pytest.raises(fg.Fem2dError) as e:
        m.h_refine_elems([0, 0], fg.HRef.T)
    assert e.value.code == fg.E_HREF
    m.h_refine_elems([0], fg.HRef.T)
    with pytest.raises(fg.Fem2dError) as e:
        m.h_refine_elems([0], fg.HRef.U)
    assert e.value.code == fg.E_HREF
    with pytest.raises(fg.Fem2dError) as e:
        m.set_global_expansion_orders(fg.Orders(0, 3))
    assert e.value.code == fg.E_PREF
    with pytest.raises(fg.Fem2dError) as e:
        m.p_refine_elems([1], fg.PRef(25, 0))
    assert e.value.code == fg.E_PREF
    with pytest.raises(fg.Fem2dError) as e:
        fg.Mesh.from_json('{"Elements": [], "Nodes": [[0,0],[0,0]]}')
    assert e.value.code == fg.E_MESH
    with pytest.raises(fg.Fem2dError) as e:
        fg.Mesh.from_json('{"Elements": [{"materials": [1,0,1,0], "node_ids": [0,1,2]}], "Nodes": [[0,0],[1,0],[0,1]]}')
    assert e.value.code == fg.E_MESH


def test_galerkin_argument_errors_without_gpu(native, kat):
    """The galerkin checks (galerkin.rs:42-59) come before any device work."""
    m = fg.Mesh.from_json(kat["mesh_b"])
    d = fg.Domain.from_mesh(m, fg.ContinuityCondition.HDiv)
    assert d.num_dofs == 0


def test_global_p_refinement_clamps(native, kat):
    m = fg.Mesh.from_json(kat["mesh_a"])
    m.global_p_refinement(fg.PRef(30, -5))
    info = m.elem_info()
    assert np.all(info[:, 1] == 20) and np.all(info[:, 2] == 1)
