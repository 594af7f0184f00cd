"""Generate tests/golden/kat.json from the reference's own test inputs and test constants.

Run in a container where the reference checkout exists (pass its root as argv[1]). The GPU machine and the
test suite only read the committed kat.json. Contents:

* the three mesh files of test_input/ (src/lib.rs:46-120 use a and b);
* test_input/test_eval.dat (big-endian f64) and test_input/test_evec.dat (PETSc Vec, classid 1211214,
  big-endian i32 header then f64 values), the slepc_problem known answer (src/lib.rs:83-120), and the
  SHA-256 of both files (pins the byte layout that slepc_solve.rs:114-147 reads);
* the 20-point Gauss-Legendre tables X_20, W_20 and X_20_SCALED, parsed from the test module of
  src/fem_problem/integration/glq.rs (lines 255-375) as text;
* the scalar known answers asserted in src/lib.rs (2.6479657 at 1e-6, 1.4745880937 at 1e-9).
"""
import hashlib
import json
import os
import re
import struct
import sys


def parse_rust_f64_array(src, name):
    m = re.search(r"const\s+%s\s*:\s*\[f64;\s*(\d+)\]\s*=\s*\[(.*?)\];" % name, src, re.S)
    if not m:
        raise SystemExit("constant %s not found" % name)
    vals = [float(t) for t in re.findall(r"-?\d+\.\d+(?:e-?\d+)?", m.group(2))]
    assert len(vals) == int(m.group(1)), name
    return vals


def main(root):
    ti = os.path.join(root, "test_input")
    out = {}
    for tag in ("a", "b", "c"):
        with open(os.path.join(ti, "test_mesh_%s.json" % tag)) as f:
            out["mesh_" + tag] = json.load(f)
    with open(os.path.join(ti, "test_eval.dat"), "rb") as f:
        raw_eval = f.read()
    out["slepc_eval"] = struct.unpack(">d", raw_eval[:8])[0]
    out["slepc_eval_sha256"] = hashlib.sha256(raw_eval).hexdigest()
    with open(os.path.join(ti, "test_evec.dat"), "rb") as f:
        raw = f.read()
    out["slepc_evec_sha256"] = hashlib.sha256(raw).hexdigest()
    out["slepc_evec_bytes"] = len(raw)
    classid, m = struct.unpack(">ii", raw[:8])
    assert classid == 1211214
    out["slepc_evec"] = list(struct.unpack(">%dd" % m, raw[8:8 + 8 * m]))
    with open(os.path.join(root, "src", "fem_problem", "integration", "glq.rs")) as f:
        glq_src = f.read()
    out["glq_x20"] = parse_rust_f64_array(glq_src, "X_20")
    out["glq_w20"] = parse_rust_f64_array(glq_src, "W_20")
    out["glq_x20_scaled_025_05"] = parse_rust_f64_array(glq_src, "X_20_SCALED")
    out["kat_nalg_problem"] = {"mesh": "mesh_a", "p_refine": [2, 2], "glq": [8, 8], "target": 2.64,
                               "value": 2.6479657, "tol": 1e-6}
    out["kat_slepc_problem"] = {"mesh": "mesh_b", "p_refine": [3, 3], "global_h": "T", "h_refine_T": [6, 9, 12],
                                "glq": [8, 8], "target": 1.475, "value": 1.4745880937, "tol": 1e-9,
                                "ndofs": m}
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "kat.json")
    with open(dst, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", dst)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of the fem_2d source tree>")
    main(sys.argv[1])
