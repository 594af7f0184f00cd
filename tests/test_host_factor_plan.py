"""The multifrontal factorization plan (host only, no GPU): structural invariants of the symbolic
analysis behind gpu_solve_gep's exact shift-invert solves (the solver that stands in for the external
KSP of slepc_solve.rs:26-36).

On a 70,902-DoF full-form mesh (large enough for every threaded path of the analysis):
- the fronts' pivots are a permutation of the DoFs, and the fronts are numbered in post-order;
- every child's update rows sit in its parent front at the positions its extend-add map gives;
- every assembly record puts its CSR entry (or, for a record of the mirrored half, the entry's
  transpose) at the front position of the matching DoF pair, and every entry of the full pattern is
  assembled, directly or through its transpose.
"""
import numpy as np
import pytest

import fem_2d_gb300 as fg
from fem_2d_gb300 import configs


@pytest.fixture(scope="module")
def plan():
    from fem_2d_gb300 import build

    build.build()
    w = configs.full_scale(seed=0, basis=0, nx=16, ny=8, rounds=4, fraction=0.44)
    dom = fg.Domain.from_mesh(configs.build_mesh(w))
    return dom, fg.factor_plan(dom), fg.domain_pattern(dom)


def _full_csr(n, ru, cu):
    """The full symmetric pattern in CSR order (rows ascending, columns ascending within a row) from the
    upper keys, with the index of each entry's transpose."""
    off = ru != cu
    rows = np.concatenate([ru, cu[off]]).astype(np.int64)
    cols = np.concatenate([cu, ru[off]]).astype(np.int64)
    order = np.lexsort((cols, rows))
    rows, cols = rows[order], cols[order]
    keys = rows * n + cols
    tpos = np.searchsorted(keys, cols * n + rows)
    assert np.array_equal(keys[tpos], cols * n + rows)
    return rows, cols, tpos


def test_pivots_are_a_permutation_in_postorder(plan):
    dom, p, _ = plan
    n = dom.num_dofs
    fr, dp, dofs = p["fronts"], p["dof_ptr"], p["dofs"]
    assert n > 65536   # the threaded paths of the analysis run
    parent, level, f, piv = fr[:, 0], fr[:, 1], fr[:, 2], fr[:, 3]
    assert np.array_equal(np.diff(dp), f) and np.all(piv <= f)
    pivots = np.concatenate([dofs[dp[k]:dp[k] + piv[k]] for k in range(len(fr))])
    assert np.array_equal(np.sort(pivots), np.arange(n))
    child = np.nonzero(parent >= 0)[0]
    assert np.all(parent[child] > child)              # post-order numbering
    assert np.all(level[parent[child]] > level[child])


def test_update_rows_land_in_the_parent_front(plan):
    _, p, _ = plan
    fr, dp, dofs, ep, em = p["fronts"], p["dof_ptr"], p["dofs"], p["ea_ptr"], p["ea_map"]
    for k in np.nonzero(fr[:, 0] >= 0)[0]:
        upd = dofs[dp[k] + fr[k, 3]:dp[k + 1]]
        m = em[ep[k]:ep[k + 1]]
        par = fr[k, 0]
        assert len(m) == len(upd)
        assert np.array_equal(dofs[dp[par] + m], upd), k


def test_assembly_records_cover_the_pattern(plan):
    dom, p, (ru, cu) = plan
    n = dom.num_dofs
    rows, cols, tpos = _full_csr(n, ru, cu)
    fr, dp, dofs, ap, apos, acsr = p["fronts"], p["dof_ptr"], p["dofs"], p["asm_ptr"], p["asm_pos"], p["asm_csr"]
    assert np.all((acsr >= 0) & (acsr < len(rows)))
    front = np.repeat(np.arange(len(fr)), np.diff(ap))
    F = fr[front, 2].astype(np.int64)
    assert np.all((apos >= 0) & (apos < F * F))
    a, b = apos // F, apos % F
    da, db = dofs[dp[front] + a], dofs[dp[front] + b]
    direct = (da == rows[acsr]) & (db == cols[acsr])
    mirror = (da == cols[acsr]) & (db == rows[acsr])
    assert np.all(direct | mirror)
    # a record's row index is a pivot of its front (a < p) unless it is the mirrored copy
    assert np.all((a < fr[front, 3]) | mirror)
    covered = np.zeros(len(rows), bool)
    covered[acsr] = True
    covered[tpos[acsr]] = True
    assert np.all(covered)


def test_plan_is_deterministic(plan):
    """The threaded analysis gives the same plan every time (the solves' bitwise reproducibility rests on
    it: the assembly maps fix the order in which entries enter the fronts)."""
    dom, p, _ = plan
    q = fg.factor_plan(dom)
    for k in p:
        assert np.array_equal(p[k], q[k]), k
