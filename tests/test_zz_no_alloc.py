"""The allocation-free values entry point (fem2d_gep_values_noalloc) against fem2d_gep_recompute.

Some hosts cannot let a library call cudaMalloc: they own every byte of device memory through their
own pool or arena, or they cannot pay for an allocation (and the device-wide synchronisation of
cudaFree) on their critical path. For them the library recomputes A and B into arrays the caller
already holds, with its scratch tables in one file-scope device array. This test calls that entry
point through the C ABI twice in a row, into caller-owned device memory, and compares both results
with the regular entry point's output within the assembly tolerance used by the other GPU tests.
It is collected last so that a run stopping at the first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

import fem_2d_gb300 as fg
from fem_2d_gb300 import configs

pytestmark = pytest.mark.gpu
TOL = 1e-12


def test_values_noalloc_matches_recompute():
    torch = pytest.importorskip("torch")
    from fem_2d_gb300 import build

    build.build()
    ctx = fg.Context(0)
    w = configs.precision(seed=1, nx=6, ny=3)
    gep = fg.galerkin_sample_gep_hcurl(fg.KOLeg, fg.CurlCurl, fg.L2Inner, fg.Domain.from_mesh(configs.build_mesh(w)),
                                       list(w.glq), ctx=ctx)
    gep.recompute()
    _, _, ref_a = gep.csr("A")
    _, _, ref_b = gep.csr("B")
    nnz = len(ref_a)
    # caller-owned device memory (not allocated by the library)
    da = torch.full((nnz,), float("nan"), dtype=torch.float64, device="cuda:0")
    db = torch.full((nnz,), float("nan"), dtype=torch.float64, device="cuda:0")
    torch.cuda.synchronize()
    L = fg.lib()
    for call in range(2):
        rc = L.fem2d_gep_values_noalloc(ctx._h, gep._h, ctypes.c_void_p(da.data_ptr()), ctypes.c_void_p(db.data_ptr()))
        assert rc == 0, L.fem2d_last_error().decode()
        ctx.synchronize()
        a = da.cpu().numpy()
        b = db.cpu().numpy()
        assert np.max(np.abs(a - ref_a)) <= TOL * np.max(np.abs(ref_a)), call
        assert np.max(np.abs(b - ref_b)) <= TOL * np.max(np.abs(ref_b)), call
        da.fill_(float("nan"))
        db.fill_(float("nan"))
        torch.cuda.synchronize()
