"""UniformFieldSpace: field quantities sampled on a uniform grid over every leaf Elem
(src/fem_domain/domain/fields.rs:17-433), with xy_fields evaluated by the device kernel.

Quantities are stored per leaf Elem (ascending id) as arrays of shape (num_leaves, d0, d1), m along
u (x) and n along v (y). The reference allocates its per-leaf arrays [d1][d0] and fills them [m][n],
which only runs when d0 == d1; here every (d0, d1) works and the square case is identical.
"""
from __future__ import annotations

import ctypes
import time

import numpy as np

from . import Context, Fem2dError, E_INVALID_ARG, _check, _ptr, lib


class UniformFieldError(Fem2dError):
    """fields.rs:391-416: MismatchedSolutionSize(domain, solution) or MissingQuantity(name)."""

    def __init__(self, kind, msg):
        super().__init__(E_INVALID_ARG, msg)
        self.kind = kind


def uniform_range(lo, hi, n):
    """fields.rs:386-389"""
    step = (hi - lo) / float(n - 1)
    return np.array([float(i) * step + lo for i in range(n)])


class _DeviceFields:
    """One fem2d_fields handle (plan uploaded once per basis space)."""

    def __init__(self, ctx, domain, basis_id, d0, d1):
        h = ctypes.c_void_p()
        _check(lib().fem2d_fields_create(ctx._h, domain._h, int(basis_id), int(d0), int(d1), ctypes.byref(h)))
        self._h = h
        self.ctx = ctx
        self.num_leaves = int(lib().fem2d_fields_num_leaves(h))
        self.leaves = np.zeros(self.num_leaves, dtype=np.int64)
        self.bounds = np.zeros((self.num_leaves, 4))
        if self.num_leaves:
            _check(lib().fem2d_fields_leaves(h, _ptr(self.leaves, ctypes.c_int64)))
            _check(lib().fem2d_fields_leaf_bounds(h, _ptr(self.bounds, ctypes.c_double)))

    def __del__(self):
        L = lib() if getattr(self, "_h", None) else None
        if L is not None:
            L.fem2d_fields_free(self._h)
            self._h = None

    def xy(self, solution, d0, d1):
        sol = np.ascontiguousarray(solution, dtype=np.float64)
        x = np.zeros((self.num_leaves, d0, d1))
        y = np.zeros((self.num_leaves, d0, d1))
        _check(lib().fem2d_fields_xy(self._h, _ptr(sol, ctypes.c_double), len(sol), _ptr(x, ctypes.c_double),
                                     _ptr(y, ctypes.c_double)))
        return x, y

    def xy_device(self, d_solution, n_solution, d_x, d_y):
        """Device-pointer form (integers from torch's data_ptr() or any allocator); asynchronous."""
        _check(lib().fem2d_fields_xy_device(self._h, ctypes.c_void_p(d_solution), int(n_solution),
                                            ctypes.c_void_p(d_x), ctypes.c_void_p(d_y)))


class UniformFieldSpace:
    """UniformFieldSpace::new(&domain, densities) (fields.rs:29-39)."""

    def __init__(self, domain, densities, ctx=None):
        d0, d1 = int(densities[0]), int(densities[1])
        if d0 < 2 or d1 < 2:
            raise UniformFieldError("InvalidDensities", "field densities must be at least 2 per axis")
        self.domain = domain
        self.densities = (d0, d1)
        self.parametric_points = (uniform_range(-1.0, 1.0, d0), uniform_range(-1.0, 1.0, d1))
        self.quantities = {}
        self._ctx = ctx
        self._dev = {}

    def _device(self, bspace):
        if bspace.ID not in self._dev:
            ctx = self._ctx or Context.default()
            self._dev[bspace.ID] = _DeviceFields(ctx, self.domain, bspace.ID, *self.densities)
        return self._dev[bspace.ID]

    @property
    def leaves(self):
        """Leaf Elem ids in the order the quantities store them."""
        return self._geometry()[0]

    def xy_fields(self, bspace, vector_name, solution):
        """xy_fields::<BSpace>(vector_name, solution) (fields.rs:63-122): stores `{name}_x` and `{name}_y`
        and returns the two names."""
        n = self.domain.num_dofs
        if len(solution) != n:
            raise UniformFieldError(
                "MismatchedSolutionSize",
                "Domain size (%d) does not match solution size (%d)!" % (n, len(solution)))
        x, y = self._device(bspace).xy(solution, *self.densities)
        xn, yn = "%s_x" % vector_name, "%s_y" % vector_name
        self.quantities[xn] = x
        self.quantities[yn] = y
        return [xn, yn]

    def quantity(self, name):
        if name not in self.quantities:
            raise UniformFieldError("MissingQuantity", "Missing quantity '%s', Cannot apply operation!" % name)
        return self.quantities[name]

    def map_to_quantity(self, name, result_name, operator):
        """map_to_quantity (fields.rs:254-277): operator applied to every value."""
        q = self.quantity(name)
        self.quantities[result_name] = np.vectorize(operator, otypes=[np.float64])(q)

    def expression_2arg(self, operand_names, result_name, expression):
        """expression_2arg (fields.rs:300-336): expression(a, b) applied pointwise."""
        a = self.quantity(operand_names[0])
        b = self.quantity(operand_names[1])
        self.quantities[result_name] = np.vectorize(expression, otypes=[np.float64])(a, b)

    def print_all_to_vtk(self, path):
        """print_all_to_vtk (fields.rs:131-134): every quantity, in insertion order."""
        self.print_quantities_to_vtk(path, list(self.quantities))

    def print_quantities_to_vtk(self, path, quantity_names):
        """print_quantities_to_vkt (fields.rs:141-234): legacy ASCII VTK unstructured grid of quads."""
        for qn in quantity_names:
            self.quantity(qn)
        nx, ny = self.densities
        leaves, bounds = self._geometry()
        ns = len(leaves)
        ns_now = time.time_ns()
        secs, nanos = divmod(ns_now, 1_000_000_000)
        stamp = ("%d.%09d" % (secs, nanos)).rstrip("0").rstrip(".") + "s"
        out = ["# vtk DataFile Version 3.0\n", "# File generated by fem_2d_gb300 on: %s\n\n" % stamp,
               "ASCII\n", "DATASET UNSTRUCTURED_GRID\n"]
        num_points = nx * ny * ns
        out.append("\nPOINTS %d double\n" % num_points)
        for k in range(ns):
            x0, y0, x1, y1 = bounds[k]
            xs = uniform_range(x0, x1, nx)
            ys = uniform_range(y0, y1, ny)
            for x in xs:
                for y in ys:
                    out.append("%.10f %.10f 0.0\n" % (x, y))
        num_cells = (nx - 1) * (ny - 1) * ns
        out.append("\nCELLS %d %d\n" % (num_cells, 5 * num_cells))
        for k in range(ns):
            for i in range(nx - 1):
                for j in range(ny - 1):
                    p = ny * i + j + nx * ny * k
                    out.append("4\t%d\t%d\t%d\t%d\n" % (p, p + 1, p + ny + 1, p + ny))
        out.append("\nCELL_TYPES %d\n" % num_cells)
        out.append(" 9" * num_cells)
        out.append("\n")
        out.append("POINT_DATA %d\n" % num_points)
        for qn in quantity_names:
            out.append("SCALARS %s double 1 \nLOOKUP_TABLE default\n" % qn)
            out.append("".join("%.15f " % v for v in self.quantities[qn].ravel()))
        out.append("\n")
        with open(path, "w") as f:
            f.write("".join(out))

    print_quantities_to_vkt = print_quantities_to_vtk

    def _geometry(self):
        """Leaf Elem ids (ascending) and their real-space diagonal points (x0, y0, x3, y3), as
        elem_diag_points returns them (mesh.rs), taken from the Domain's own mesh."""
        if not self._dev:
            from . import HierPoly
            self._device(HierPoly)
        dev = next(iter(self._dev.values()))
        return dev.leaves, dev.bounds
