"""Make the FP64 oracle fixtures of the full-form workloads (test infrastructure; CPU only).

For each workload this runs, once, on the host:

* the oracle's literal 2-D quadrature assembly (oracle/fem2d_oracle.cpp) of the HierPoly pencil;
* the SHA-256 of its upper-triangle pattern (row, col as little-endian int32), max |A|, max |B| and a
  seeded sample of upper entries (row, col, A, B), so a GPU run can check its pattern bit for bit and
  its values entrywise without re-running the assembly;
* the 20 eigenvalues nearest 10.0 (non-spurious) by the ARPACK oracle ``arpack_nearest_physical``
  (Lanczos on T = (A - s B)^-1 A (A + s B)^-1 B with SuperLU solves under the oracle's own nested
  dissection ordering; above 500k DoFs, SuperLU on 16 subdomains plus a dense Schur complement), with
  their residuals and error bounds;
* with ``--cross-check``, the same 20 by the second oracle method ``sparse_nearest_physical`` (block
  Krylov with CGS2 and Rayleigh-Ritz), and the largest relative difference of the two.

The result is ``tests/golden/full_form_<workload>.json``. No GPU and no product library is used:
workload scripts are replayed on the oracle mesh.

    python tests/golden/make_full_form_fixture.py full_160k --cross-check
    python tests/golden/make_full_form_fixture.py full_1m --eig-basis koleg

At 1M DoFs the monomial (HierPoly) pencil is so ill-conditioned that the rounding of the oracle's
solves breaks the B-symmetry ARPACK relies on (one member of each degenerate eigenvalue pair came out
wrong by up to 1e-3); the eigenvalue reference there is computed on the KOLeg pencil of the same mesh,
which spans the same discrete space, while the assembly checks stay on the HierPoly pencil.
"""
import argparse
import hashlib
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from fem_2d_gb300 import configs  # noqa: E402  (pure Python; loads no library)
from oracle import build as oracle_build  # noqa: E402
from oracle import ref  # noqa: E402

# the full-form workloads: (configs.full_scale keyword arguments)
WORKLOADS = {
    "full_1m": dict(nx=64, ny=32, rounds=4, fraction=0.44),
    "full_160k": dict(nx=32, ny=16, rounds=3, fraction=0.44),
}


def pattern_sha(rows, cols):
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(rows, dtype="<i4").tobytes())
    h.update(np.ascontiguousarray(cols, dtype="<i4").tobytes())
    return h.hexdigest()


def make(name, cross_check=False, samples=4096, threads=None, eig_basis="hierpoly"):
    oracle_build.build_oracle()
    w = configs.full_scale(seed=0, basis=0, replay=ref.OracleReplay, **WORKLOADS[name])
    t0 = time.time()
    om = ref.OracleMesh(w.mesh_json)
    om.apply_ops(w.ops)
    n = om.domain()
    r, c, a, b = om.galerkin(w.basis, w.glq[0], w.glq[1], threads=threads or os.cpu_count() or 4)
    t_asm = time.time() - t0
    rng = np.random.default_rng(12345)
    pick = np.sort(rng.choice(len(r), size=min(samples, len(r)), replace=False))
    out = {"workload": w.name, "key": name, "ndofs": int(n), "nnz_upper": int(len(r)),
           "basis": "HierPoly", "glq": list(w.glq), "target": w.target, "n_pairs": w.n_pairs,
           "pattern_sha256": pattern_sha(r, c), "max_abs_a": float(np.max(np.abs(a))),
           "max_abs_b": float(np.max(np.abs(b))),
           "sample": {"rows": r[pick].tolist(), "cols": c[pick].tolist(), "a": a[pick].tolist(),
                      "b": b[pick].tolist()},
           "t_oracle_assembly_s": t_asm, "threads": threads or os.cpu_count()}
    print("%s: %d DoFs, %d upper entries, assembly %.1f s" % (w.name, n, len(r), t_asm), flush=True)
    if eig_basis == "koleg":
        # the eigenvalue reference from the KOLeg pencil of the same mesh: the same discrete space
        # (equal eigenvalues in exact arithmetic) with Legendre-based shape functions, whose pencil is
        # far better conditioned than the monomial one at this size
        del r, c, a, b
        t0 = time.time()
        r, c, a, b = om.galerkin(ref.KOLEG, w.glq[0], w.glq[1], threads=threads or os.cpu_count() or 4)
        out["eig_pencil"] = "KOLeg (oracle assembly of the same mesh, %.1f s)" % (time.time() - t0)
    else:
        out["eig_pencil"] = "HierPoly (the assembled pencil itself)"
    A = ref.full_sym(n, r, c, a)
    B = ref.full_sym(n, r, c, b)
    del r, c, a, b
    box = ref.dof_boxes(om)
    t0 = time.time()
    if n > 500000:
        # SuperLU's first fill estimate (about 20 x nnz) overflows its 32-bit sizes at this nnz: two-level
        # substructuring over 16 subdomains (SuperLU each) and a dense Schur complement instead (checked
        # against the direct SuperLU fixture at 160k DoFs: eigenvalues within 6.2e-12)
        parts, sep = ref.nd_parts(box, 4)
        res = ref.arpack_nearest_physical(A, B, w.target, w.n_pairs, None, refine=0, schur=(box, parts, sep))
        solver = "SchurLU: 16 SuperLU subdomains + dense Schur complement of %d separator DoFs" % len(sep)
    else:
        res = ref.arpack_nearest_physical(A, B, w.target, w.n_pairs, ref.nd_order(box), refine=0)
        solver = "SuperLU under the oracle's nested-dissection ordering"
    t_eig = time.time() - t0
    # eigenvalues: from ARPACK's mu (robust to the solves' rounding noise); the Rayleigh-Ritz values of
    # the Lanczos vectors on (A, B), where they pass the residual filter, are kept as a cross-check
    out["eigenvalues"] = np.sort(res["values_from_mu"]).tolist()
    o = np.argsort(res["values"])
    out["rr_eigenvalues"] = res["values"][o].tolist()
    out["rr_rel_residual"] = res["rel_residual"][o].tolist()
    out["rr_backward_error"] = res["backward_error"][o].tolist()
    out["rr_resid_binv"] = res["resid_binv"][o].tolist()
    out["rr_err_bound"] = res["err_bound"][o].tolist()
    n_rr = len(out["rr_eigenvalues"])
    ev = np.asarray(out["eigenvalues"])
    rr = np.asarray(out["rr_eigenvalues"])
    # each Rayleigh-Ritz value against the nearest mu-value
    out["rr_vs_mu_max_rel_diff"] = float(max(np.min(np.abs(ev - t)) / abs(t) for t in rr)) if n_rr else None
    out["mu_min"] = res["mu_min"]
    out["arpack_applications"] = res["applications"]
    out["t_oracle_eigensolve_s"] = t_eig
    out["sparse_solver"] = solver
    print("ARPACK: %.1f s, %d applications of T" % (t_eig, res["applications"]), flush=True)
    if cross_check:
        t0 = time.time()
        ws, _, rel = ref.sparse_nearest_physical(A, B, w.target, w.n_pairs, perm=ref.nd_order(box), tol=1e-12,
                                                 max_cycles=25)
        ws = np.sort(ws)
        out["cross_check"] = {"method": "block Krylov (sparse_nearest_physical)", "eigenvalues": ws.tolist(),
                              "max_rel_diff": float(np.max(np.abs(ws - np.asarray(out["eigenvalues"])) / np.abs(ws))),
                              "max_rel_residual": float(np.max(rel)), "t_s": time.time() - t0}
        print("cross-check: max rel diff %.3e" % out["cross_check"]["max_rel_diff"], flush=True)
    path = os.path.join(ROOT, "tests", "golden", "full_form_%s.json" % name)
    with open(path, "w") as f:
        json.dump(out, f)
    print("wrote", path)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("workload", choices=sorted(WORKLOADS))
    ap.add_argument("--cross-check", action="store_true")
    ap.add_argument("--threads", type=int, default=None)
    ap.add_argument("--eig-basis", choices=["hierpoly", "koleg"], default="hierpoly",
                    help="pencil the eigenvalue reference is computed on (koleg: same space, better conditioned)")
    args = ap.parse_args()
    make(args.workload, args.cross_check, threads=args.threads, eig_basis=args.eig_basis)


if __name__ == "__main__":
    main()
