"""The allocation-free values entry point (fem2d_gep_values_noalloc) against fem2d_gep_recompute.

Some hosts cannot let a library call cudaMalloc: they own every byte of device memory through their
own pool or arena, or they cannot pay for an allocation (and the device-wide synchronisation of
cudaFree) on their critical path. For them the library recomputes A and B into arrays the caller
already holds, with its scratch tables in one file-scope device array. These tests call that entry
point through the C ABI, into caller-owned device memory: twice in a row, then alternating between two
GEPs whose tables differ in size (so a stale table entry left by the previous call would show), and
compare every result bit for bit with the regular entry point's output (both run the same kernels on
the same inputs; the assembly tolerance of the other GPU tests, 1e-12, is the looser bound). A GEP
whose tables exceed the array is rejected with FEM2D_E_TOO_LARGE before anything is written. The
file is collected last so that a run stopping at the first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

import fem_2d_gb300 as fg
from fem_2d_gb300 import configs

pytestmark = pytest.mark.gpu
TOL = 1e-12


def _gep(ctx, w, basis):
    return fg.galerkin_sample_gep_hcurl(basis, fg.CurlCurl, fg.L2Inner, fg.Domain.from_mesh(configs.build_mesh(w)),
                                        list(w.glq), ctx=ctx)


def _reference_values(gep):
    gep.recompute()
    _, _, ref_a = gep.csr("A")
    _, _, ref_b = gep.csr("B")
    return ref_a, ref_b


def _call(L, ctx, gep, da, db):
    import ctypes

    return L.fem2d_gep_values_noalloc(ctx._h, gep._h, ctypes.c_void_p(da.data_ptr()), ctypes.c_void_p(db.data_ptr()))


def test_values_noalloc_matches_recompute():
    torch = pytest.importorskip("torch")
    ctx = fg.Context(0)
    geps = [_gep(ctx, configs.precision(seed=1, nx=6, ny=3), fg.KOLeg),
            _gep(ctx, configs.full_scale(seed=2, nx=4, ny=2, rounds=2, fraction=0.5), fg.HierPoly)]
    refs = [_reference_values(g) for g in geps]
    L = fg.lib()
    # two calls in a row on the first GEP, then alternating GEPs (different orders and interval counts)
    for call, k in enumerate((0, 0, 1, 0, 1)):
        ref_a, ref_b = refs[k]
        nnz = len(ref_a)
        # caller-owned device memory (not allocated by the library), filled with NaN before each call
        da = torch.full((nnz,), float("nan"), dtype=torch.float64, device="cuda:0")
        db = torch.full((nnz,), float("nan"), dtype=torch.float64, device="cuda:0")
        torch.cuda.synchronize()
        rc = _call(L, ctx, geps[k], da, db)
        assert rc == 0, L.fem2d_last_error().decode()
        ctx.synchronize()
        a = da.cpu().numpy()
        b = db.cpu().numpy()
        assert np.max(np.abs(a - ref_a)) <= TOL * np.max(np.abs(ref_a)), call
        assert np.max(np.abs(b - ref_b)) <= TOL * np.max(np.abs(ref_b)), call
        assert np.array_equal(a, ref_a) and np.array_equal(b, ref_b), call


def _too_large_workload():
    """Two Elems: Elem 0 at expansion order 20 (table stride 21), Elem 1 at order 2 refined seven times
    with V refinements of all its leaves (1,528 DoFs): 568,890 table doubles, above the 524,288 limit
    (checked on the host by tests/test_host_tables.py)."""
    m_json = configs.grid_mesh_json(2, 1, 0.0, 2.0, 0.0, 1.0)
    ops = [("orders", 2, 2, None), ("orders", 20, 20, [0])]
    m = configs.NativeReplay(m_json)
    m.apply(ops)
    for _ in range(7):
        info = m.elem_info()
        leaves = [int(e) for e in np.nonzero(info[:, 0] == 1)[0] if e != 0]
        op = ("hmix", leaves, [2] * len(leaves))
        m.apply([op])
        ops.append(op)
    return configs.Workload("too_large_tables", m_json, ops, basis=0, glq=(10, 10))


def test_values_noalloc_rejects_too_large():
    torch = pytest.importorskip("torch")
    ctx = fg.Context(0)
    g = _gep(ctx, _too_large_workload(), fg.HierPoly)
    _, _, nnz = g.dims()
    da = torch.full((nnz,), float("nan"), dtype=torch.float64, device="cuda:0")
    db = torch.full((nnz,), float("nan"), dtype=torch.float64, device="cuda:0")
    torch.cuda.synchronize()
    L = fg.lib()
    rc = _call(L, ctx, g, da, db)
    assert rc == fg.E_TOO_LARGE, (rc, L.fem2d_last_error().decode())
    assert "524288" in L.fem2d_last_error().decode()
    ctx.synchronize()
    assert torch.isnan(da).all().item() and torch.isnan(db).all().item()
    # a host array is refused (it would fault inside the kernels)
    import ctypes

    host = np.zeros(nnz)
    rc = L.fem2d_gep_values_noalloc(ctx._h, g._h, host.ctypes.data_as(ctypes.c_void_p), host.ctypes.data_as(ctypes.c_void_p))
    assert rc == fg.E_INVALID_ARG
