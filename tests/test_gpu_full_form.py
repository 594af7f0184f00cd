"""The full-form family at 160,346 DoFs (32x16 base Elems, orders 3..8, three T/U/V rounds of 44% of
the leaves, HierPoly, GLQ [10,10]) against the committed FP64 oracle fixture
tests/golden/full_form_full_160k.json (made by tests/golden/make_full_form_fixture.py: the oracle's
literal 2-D assembly, then ARPACK shift-invert Lanczos with SuperLU solves, cross-checked by a second
oracle method to 2.1e-11): the pattern bit for bit, a seeded sample of 4,096 entries of A and B
entrywise, and the 20 eigenvalues nearest 10.0 to 1e-9 relative (the reference's sparse-solve pin,
src/lib.rs:100-104)."""
import hashlib
import json
import os

import numpy as np
import pytest

import fem_2d_gb300 as fg
from fem_2d_gb300 import configs

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def fixture():
    with open(os.path.join(ROOT, "tests", "golden", "full_form_full_160k.json")) as f:
        return json.load(f)


@pytest.fixture(scope="module")
def gep():
    ctx = fg.Context(0)
    w = configs.full_scale(seed=0, basis=0, nx=32, ny=16, rounds=3, fraction=0.44)
    d = fg.Domain.from_mesh(configs.build_mesh(w))
    return fg.galerkin_sample_gep_hcurl(fg.HierPoly, fg.CurlCurl, fg.L2Inner, d, list(w.glq), ctx=ctx)


def test_assembly_against_oracle_fixture(gep, fixture):
    assert gep.dimension == fixture["ndofs"]
    r, c, a, b = gep.upper_coo()
    assert len(r) == fixture["nnz_upper"]
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(r, dtype="<i4").tobytes())
    h.update(np.ascontiguousarray(c, dtype="<i4").tobytes())
    assert h.hexdigest() == fixture["pattern_sha256"]
    sm = fixture["sample"]
    keys = r.astype(np.int64) * gep.dimension + c
    want = np.asarray(sm["rows"], np.int64) * gep.dimension + np.asarray(sm["cols"], np.int64)
    pos = np.searchsorted(keys, want)
    assert np.array_equal(keys[pos], want)
    assert np.max(np.abs(a[pos] - np.asarray(sm["a"]))) <= 1e-12 * fixture["max_abs_a"]
    assert np.max(np.abs(b[pos] - np.asarray(sm["b"]))) <= 1e-12 * fixture["max_abs_b"]


@pytest.mark.parametrize("dense", [0, 1])
def test_eigenvalues_against_oracle_fixture(gep, fixture, dense):
    res = fg.gpu_solve_gep_n(gep, 10.0, 20, dense=dense)
    ov = np.asarray(fixture["eigenvalues"])
    gv = np.sort(res.values)
    assert len(ov) == len(gv) == 20
    assert np.max(np.abs(gv - ov) / np.abs(ov)) <= 1e-9
    assert res.stats["max_backward_error"] <= 1e-9
