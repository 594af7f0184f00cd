"""Host-side size of the assembly's 1-D contraction tables (fem2d_domain_table_doubles), the quantity
the allocation-free values entry point checks against its 524,288-double capacity; no GPU needed."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "tests"))

import fem_2d_gb300 as fg  # noqa: E402
from fem_2d_gb300 import configs  # noqa: E402


def _tables(w, basis):
    return fg.domain_table_doubles(fg.Domain.from_mesh(configs.build_mesh(w)), basis, w.glq)


def test_table_sizes():
    import test_zz_no_alloc as nz

    big = _tables(nz._too_large_workload(), fg.HierPoly)
    assert big == 568890 and big > 524288
    small = _tables(configs.precision(seed=1, nx=6, ny=3), fg.KOLeg)
    other = _tables(configs.full_scale(seed=2, nx=4, ny=2, rounds=2, fraction=0.5), fg.HierPoly)
    assert small <= 524288 and other <= 524288 and small != other
