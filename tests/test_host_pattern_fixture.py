"""Host symbolic phase at full-form scale (no GPU): the GEP pattern of the 160k-DoF full-form mesh against
the committed FP64 oracle fixture, bit for bit.

The small meshes of test_host_parity.py stay below the size from which the symbolic phase of
galerkin_sample_gep_hcurl (galerkin.rs:33-187) splits its bucketing, prefix sums and transpose over
host threads; this mesh (160,346 DoFs, 8.8 M upper entries) runs every threaded path. The fixture's
pattern hash was computed from the oracle's literal assembly (tests/golden/make_full_form_fixture.py).
"""
import hashlib
import json
import os

import numpy as np
import pytest

import fem_2d_gb300 as fg
from fem_2d_gb300 import configs

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
FIXTURE = os.path.join(ROOT, "tests", "golden", "full_form_full_160k.json")


@pytest.fixture(scope="module")
def native():
    from fem_2d_gb300 import build

    build.build()
    return fg.lib()


def test_full_form_160k_pattern_matches_oracle_fixture(native):
    if not os.path.exists(FIXTURE):
        pytest.skip("full_160k oracle fixture not generated")
    with open(FIXTURE) as f:
        fx = json.load(f)
    # the fixture's workload: 32 x 16 base Elems, orders 3..8, three T/U/V rounds refining 44% of the
    # leaves, HierPoly (the same arguments the bench's full_160k workload uses)
    w = configs.full_scale(seed=0, basis=0, nx=32, ny=16, rounds=3, fraction=0.44)
    dom = fg.Domain.from_mesh(configs.build_mesh(w))
    assert dom.num_dofs == fx["ndofs"]
    rows, cols = fg.domain_pattern(dom)
    assert len(rows) == fx["nnz_upper"]
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(rows, dtype="<i4").tobytes())
    h.update(np.ascontiguousarray(cols, dtype="<i4").tobytes())
    assert h.hexdigest() == fx["pattern_sha256"]
