"""Host side of the batched-assembly autotuner: the launch-shape cache's text/JSON round trip and its
validation (no GPU needed: the cache lives in the host library)."""
import json
import os

import pytest

import fem_2d_gb300 as fg


@pytest.fixture(autouse=True)
def clean_cache():
    fg.autotune_clear()
    yield
    fg.autotune_clear()


def test_autotune_json_round_trip(tmp_path):
    p = tmp_path / "tune.json"
    with open(p, "w") as f:
        json.dump({"NVIDIA_GB300|values|P9|nnz2^22": [512, 2], "NVIDIA_GB300|values|P7|nnz2^18": [256, 8]}, f)
    assert fg.autotune_load(str(p)) == 2
    c = fg.autotune_cache()
    assert c["NVIDIA_GB300|values|P9|nnz2^22"] == (512, 2)
    assert c["NVIDIA_GB300|values|P7|nnz2^18"] == (256, 8)
    q = tmp_path / "out.json"
    fg.autotune_save(str(q))
    with open(q) as f:
        d = json.load(f)
    assert d == {"NVIDIA_GB300|values|P9|nnz2^22": [512, 2], "NVIDIA_GB300|values|P7|nnz2^18": [256, 8]}
    fg.autotune_clear()
    assert fg.autotune_cache() == {}


def test_autotune_rejects_unknown_shape(tmp_path):
    p = tmp_path / "bad.json"
    with open(p, "w") as f:
        json.dump({"x|values|P9|nnz2^10": [96, 3]}, f)
    with pytest.raises(fg.Fem2dError) as e:
        fg.autotune_load(str(p))
    assert e.value.code == fg.E_INVALID_ARG
    assert fg.autotune_cache() == {}


def test_batch_symbols_exported():
    L = fg.lib()
    for name in ("fem2d_galerkin_sample_gep_hcurl_batch", "fem2d_gep_batch_recompute", "fem2d_autotune_export",
                 "fem2d_autotune_import", "fem2d_autotune_clear"):
        assert hasattr(L, name)
    assert os.path.exists(fg.LIB_PATH)
