"""Files of the reference's external-solver hand-off, on the CPU (no device work):

* AIJMatrixBinary (sparse_matrix.rs:184-265), written by the product from a CSR, byte-identical to
  the oracle's restatement built through SparseMatrix::insert semantics; on the reference's own
  petsc_binary_format test inputs (sparse_matrix.rs:271-287) and on a KAT-mesh GEP;
* the PETSc Vec / scalar files retrieve_solution reads (slepc_solve.rs:104-147): writing the
  reference's golden eigenpair reproduces test_input/test_evec.dat and test_eval.dat byte for byte
  (SHA-256 pinned in tests/golden/kat.json), and reading returns the values.
"""
import hashlib
import os
import struct

import numpy as np
import pytest

import fem_2d_gb300 as fg


def _full_csr(osm):
    n = osm.dimension
    full = {}
    for (r, c), v in osm.entries.items():
        full[(r, c)] = v
        full[(c, r)] = v
    keys = sorted(full)
    rp = np.zeros(n + 1, dtype=np.int64)
    for (r, _) in keys:
        rp[r + 1] += 1
    rp = np.cumsum(rp)
    col = np.array([c for (_, c) in keys], dtype=np.int32)
    val = np.array([full[k] for k in keys])
    return rp, col, val


def test_aij_reference_test_inputs(oracle_lib, tmp_path):
    sm = oracle_lib.OracleSparseMatrix(10)
    for rc, v in [([0, 0], 1.0), ([0, 0], 1.0), ([9, 9], 10.0), ([4, 3], 0.25), ([0, 8], 0.125), ([8, 0], 0.125)]:
        sm.insert(rc, v)
    assert sm.entries == {(0, 0): 2.0, (9, 9): 10.0, (3, 4): 0.25, (0, 8): 0.25}   # value_insertion test
    want = sm.aij_bytes()
    path = os.path.join(tmp_path, "test.bin")
    fg.aij_write(path, *_full_csr(sm))
    assert open(path, "rb").read() == want
    rp, col, val = fg.aij_read(path)
    np.testing.assert_array_equal(rp, _full_csr(sm)[0])
    np.testing.assert_array_equal(col, [0, 8, 4, 3, 0, 9])
    np.testing.assert_array_equal(val, [2.0, 0.25, 0.25, 0.25, 0.25, 10.0])


def test_aij_kat_gep(oracle_lib, kat, tmp_path):
    om = oracle_lib.OracleMesh(kat["mesh_b"])
    om.apply_ops([("pref", 3, 3, None), ("href", 0, None, -1), ("href", 0, [6, 9, 12], -1)])
    n = om.domain()
    rows, cols, a, b = om.galerkin(0, 8, 8)
    for vals, tag in ((a, "a"), (b, "b")):
        sm = oracle_lib.OracleSparseMatrix(n)
        for r, c, v in zip(rows, cols, vals):
            sm.insert((r, c), float(v))
        path = os.path.join(tmp_path, "p_%s.dat" % tag)
        rp, col, val = _full_csr(sm)
        fg.aij_write(path, rp, col, val)
        assert open(path, "rb").read() == sm.aij_bytes()
        rp2, col2, val2 = fg.aij_read(path)
        np.testing.assert_array_equal(rp2, rp)
        np.testing.assert_array_equal(col2, col)
        np.testing.assert_array_equal(val2, val)


def test_aij_standard_class_id(tmp_path):
    path = os.path.join(tmp_path, "std.dat")
    body = struct.pack(">iiii", 1211216, 2, 2, 3) + struct.pack(">ii", 2, 1) + struct.pack(">iii", 0, 1, 1)
    body += struct.pack(">ddd", 4.0, -1.0, 3.0)
    open(path, "wb").write(body)
    rp, col, val = fg.aij_read(path)
    np.testing.assert_array_equal(rp, [0, 2, 3])
    np.testing.assert_array_equal(col, [0, 1, 1])
    np.testing.assert_array_equal(val, [4.0, -1.0, 3.0])


def test_golden_eigenpair_files(oracle_lib, kat, tmp_path):
    os.makedirs(os.path.join(tmp_path, "tmp"))
    base = os.path.join(tmp_path, "tmp", "p_12345678")
    evec = np.asarray(kat["slepc_evec"])
    fg.petsc_vec_write(base + "_evec.dat", evec)
    fg.petsc_scalar_write(base + "_eval.dat", kat["slepc_eval"])
    raw = open(base + "_evec.dat", "rb").read()
    assert len(raw) == kat["slepc_evec_bytes"]
    assert raw == oracle_lib.petsc_vec_bytes(list(evec))
    assert hashlib.sha256(raw).hexdigest() == kat["slepc_evec_sha256"]
    assert hashlib.sha256(open(base + "_eval.dat", "rb").read()).hexdigest() == kat["slepc_eval_sha256"]
    pair = fg.retrieve_solution(tmp_path, "p_12345678")
    assert pair.value == kat["slepc_eval"]
    np.testing.assert_array_equal(pair.vector, evec)


def test_io_errors(tmp_path):
    missing = os.path.join(tmp_path, "nope.dat")
    with pytest.raises(fg.Fem2dError) as e:
        fg.retrieve_eigenvector(missing)
    assert e.value.code == fg.E_IO
    bad = os.path.join(tmp_path, "bad.dat")
    open(bad, "wb").write(struct.pack(">ii", 1211214, 10) + b"\0" * 16)
    with pytest.raises(fg.Fem2dError, match="truncated"):
        fg.retrieve_eigenvector(bad)
    open(bad, "wb").write(b"\0{P" + struct.pack(">III", 3, 3, 9))
    with pytest.raises(fg.Fem2dError, match="truncated"):
        fg.aij_read(bad)
    with pytest.raises(fg.Fem2dError, match="ascend"):
        fg.aij_write(bad, [0, 2], [1, 0], [1.0, 2.0])
