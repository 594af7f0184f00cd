"""fem_2d_gb300: GB300 implementation of fem_2d's Galerkin generalized-eigenproblem path.

A thin Python face over the C ABI in ``include/fem2d_gb300.h`` (``libfem2d_gb300.so``, built in-tree
by ``fem_2d_gb300/build.py``). Names follow the reference's prelude (src/lib.rs:14-39):

    mesh = Mesh.from_file("mesh.json"); mesh.global_p_refinement(PRef.from_(3, 3))
    mesh.global_h_refinement(HRef.T); mesh.h_refine_elems([6, 9, 12], HRef.T)
    domain = Domain.from_mesh(mesh, ContinuityCondition.HCurl)
    gep = galerkin_sample_gep_hcurl(HierPoly, CurlCurl, L2Inner, domain, [8, 8])
    pair = gpu_solve_gep(gep, 1.475)            # stands beside slepc_solve_gep
    pair = nalgebra_solve_gep(gep, 2.64)        # nalgebra_solve_gep restated on the device

There is no CPU fallback: the GPU entry points raise if the library or a CUDA device is missing.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass, field

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libfem2d_gb300.so")
_lib = None


class Fem2dError(RuntimeError):
    """A failed call through the C ABI; ``code`` is one of the FEM2D_E_* status codes."""

    def __init__(self, code, msg):
        super().__init__("[%d] %s" % (code, msg))
        self.code = code


# status codes (include/fem2d_gb300.h)
E_OK, E_INVALID_ARG, E_MESH, E_HREF, E_PREF, E_WRONG_CC, E_EMPTY_DOFS, E_INVALID_GLQ = range(8)
E_B_NOT_SPD, E_SPURIOUS, E_TOO_LARGE, E_NOT_CONVERGED, E_CUDA, E_TIMEOUT, E_NO_DEVICE, E_IO = range(8, 16)


class _fem2d_solve_opts(ctypes.Structure):
    _fields_ = [("precond", ctypes.c_int), ("max_outer", ctypes.c_int), ("max_inner", ctypes.c_int),
                ("tol", ctypes.c_double), ("inner_tol", ctypes.c_double), ("block", ctypes.c_int),
                ("verbose", ctypes.c_int), ("krylov_steps", ctypes.c_int),
                ("damping", ctypes.c_double), ("scaling", ctypes.c_int), ("dense", ctypes.c_int),
                ("net", ctypes.c_void_p), ("refine", ctypes.c_int)]


class _fem2d_solve_stats(ctypes.Structure):
    _fields_ = [("outer_iters", ctypes.c_int), ("inner_iters_total", ctypes.c_int), ("converged", ctypes.c_int),
                ("t_setup_ms", ctypes.c_double), ("t_solve_ms", ctypes.c_double),
                ("max_rel_residual", ctypes.c_double), ("spmv_count", ctypes.c_int64),
                ("refine_spd", ctypes.c_int), ("refine_indefinite", ctypes.c_int), ("dense_plan", ctypes.c_int),
                ("floor_reached", ctypes.c_int), ("block_scaled", ctypes.c_int), ("delayed_pivots", ctypes.c_int),
                ("max_backward_error", ctypes.c_double), ("inner_cg_iters", ctypes.c_int64),
                ("inner_minres_iters", ctypes.c_int64), ("inner_max_relres", ctypes.c_double)]


def lib():
    """Load libfem2d_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError("libfem2d_gb300.so is not built; run `python -c 'import __graft_entry__ as g; g.build()'`")
    L = ctypes.CDLL(LIB_PATH)
    P, i64, i32, d = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32, ctypes.c_double
    PP = ctypes.POINTER(ctypes.c_void_p)
    i64p, i32p, dp = ctypes.POINTER(i64), ctypes.POINTER(i32), ctypes.POINTER(d)
    sig = {
        "fem2d_last_error": (ctypes.c_char_p, []),
        "fem2d_version": (ctypes.c_char_p, []),
        "fem2d_mesh_from_json": (ctypes.c_int, [ctypes.c_char_p, PP]),
        "fem2d_mesh_from_file": (ctypes.c_int, [ctypes.c_char_p, PP]),
        "fem2d_mesh_unit": (ctypes.c_int, [PP]),
        "fem2d_mesh_clone": (ctypes.c_int, [P, PP]),
        "fem2d_mesh_free": (None, [P]),
        "fem2d_mesh_set_expansion_orders": (ctypes.c_int, [P, i64p, i64, ctypes.c_int, ctypes.c_int]),
        "fem2d_mesh_p_refine": (ctypes.c_int, [P, i64p, i64, ctypes.c_int, ctypes.c_int]),
        "fem2d_mesh_h_refine": (ctypes.c_int, [P, i64p, i64, ctypes.c_int, ctypes.c_int]),
        "fem2d_mesh_execute_h_refinements": (ctypes.c_int, [P, i64p, i32p, i64]),
        "fem2d_mesh_num_elems": (i64, [P]),
        "fem2d_mesh_num_edges": (i64, [P]),
        "fem2d_mesh_num_nodes": (i64, [P]),
        "fem2d_mesh_elem_info": (ctypes.c_int, [P, i64p]),
        "fem2d_mesh_elem_bounds": (ctypes.c_int, [P, dp]),
        "fem2d_domain_from_mesh": (ctypes.c_int, [P, ctypes.c_int, PP]),
        "fem2d_domain_free": (None, [P]),
        "fem2d_domain_num_dofs": (i64, [P]),
        "fem2d_domain_num_specs": (i64, [P]),
        "fem2d_domain_basis_specs": (ctypes.c_int, [P, i64p]),
        "fem2d_domain_pattern": (ctypes.c_int, [P, i64p, i32p, i32p]),
        "fem2d_domain_factor_plan": (ctypes.c_int, [P, i64p, i32p, i64p, i32p, i64p, i64p, i64p, i64p, i32p]),
        "fem2d_ctx_create": (ctypes.c_int, [ctypes.c_int, PP]),
        "fem2d_ctx_destroy": (None, [P]),
        "fem2d_ctx_synchronize": (ctypes.c_int, [P]),
        "fem2d_ctx_flush_l2": (ctypes.c_int, [P]),
        "fem2d_ctx_kernel_launches": (i64, [P]),
        "fem2d_galerkin_sample_gep_hcurl": (ctypes.c_int, [P, P, ctypes.c_int, ctypes.c_int, ctypes.c_int, PP]),
        "fem2d_gep_recompute": (ctypes.c_int, [P, P]),
        "fem2d_gep_values_noalloc": (ctypes.c_int, [P, P, ctypes.c_void_p, ctypes.c_void_p]),
        "fem2d_gep_set_upper_values": (ctypes.c_int, [P, dp, dp]),
        "fem2d_block_gemm_device": (ctypes.c_int, [P, ctypes.c_int, i64, ctypes.c_void_p, i64, ctypes.c_int,
                                                   ctypes.c_void_p, ctypes.c_int, d, d, ctypes.c_void_p, i64]),
        "fem2d_gep_spmm_tensor_device": (ctypes.c_int, [P, P, ctypes.c_int, d, ctypes.c_void_p, i64, ctypes.c_int,
                                                        ctypes.c_void_p, i64]),
        "fem2d_domain_table_doubles": (ctypes.c_int, [P, ctypes.c_int, ctypes.c_int, ctypes.c_int, i64p]),
        "fem2d_block_gram_device": (ctypes.c_int, [P, ctypes.c_int, i64, ctypes.c_void_p, i64, ctypes.c_int,
                                                   ctypes.c_void_p, i64, ctypes.c_int, ctypes.c_void_p]),
        "fem2d_galerkin_sample_gep_hcurl_batch": (ctypes.c_int, [P, PP, i64, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                                          ctypes.c_int, PP, dp]),
        "fem2d_gep_batch_recompute": (ctypes.c_int, [P, PP, i64, ctypes.c_int, dp]),
        "fem2d_autotune_export": (ctypes.c_int, [ctypes.c_char_p, i64, i64p]),
        "fem2d_autotune_import": (ctypes.c_int, [ctypes.c_char_p, i64p]),
        "fem2d_autotune_clear": (ctypes.c_int, []),
        "fem2d_patchnet_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_uint64, PP]),
        "fem2d_patchnet_free": (None, [P]),
        "fem2d_patchnet_num_params": (i64, [P]),
        "fem2d_patchnet_get_params": (ctypes.c_int, [P, ctypes.POINTER(ctypes.c_float)]),
        "fem2d_patchnet_set_params": (ctypes.c_int, [P, ctypes.POINTER(ctypes.c_float)]),
        "fem2d_patchnet_features": (ctypes.c_int, [P, d, i64p, i64p, i32p, ctypes.POINTER(ctypes.c_float),
                                                   ctypes.POINTER(ctypes.c_float)]),
        "fem2d_patchnet_loss_grad": (ctypes.c_int, [P, P, P, d, dp, ctypes.c_int, dp, ctypes.POINTER(ctypes.c_float)]),
        "fem2d_patchnet_train": (ctypes.c_int, [P, P, PP, ctypes.c_int, d, ctypes.POINTER(dp), ctypes.c_int,
                                                ctypes.c_int, d, dp]),
        "fem2d_pcg_create": (ctypes.c_int, [P, P, d, d, P, PP]),
        "fem2d_pcg_solve": (ctypes.c_int, [P, ctypes.c_int, dp, dp, d, ctypes.c_int, dp]),
        "fem2d_pcg_harvest": (ctypes.c_int, [P, ctypes.c_int, dp, dp, d, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                             ctypes.c_int, dp, ctypes.POINTER(ctypes.c_int)]),
        "fem2d_pcg_create_with_basis": (ctypes.c_int, [P, P, d, d, ctypes.c_int, ctypes.POINTER(ctypes.c_float), PP]),
        "fem2d_pcg_free": (None, [P]),
        "fem2d_gep_free": (None, [P]),
        "fem2d_gep_dims": (ctypes.c_int, [P, i64p, i64p, i64p]),
        "fem2d_gep_export_upper": (ctypes.c_int, [P, i32p, i32p, dp, dp]),
        "fem2d_gep_export_csr": (ctypes.c_int, [P, ctypes.c_int, i64p, i32p, dp]),
        "fem2d_gep_timings": (ctypes.c_int, [P, dp]),
        "fem2d_gep_by_parts": (ctypes.c_int, [P, P, dp]),
        "fem2d_gep_num_visits": (i64, [P]),
        "fem2d_gep_h2d_bytes": (i64, [P]),
        "fem2d_ctx_timer_start": (ctypes.c_int, [P]),
        "fem2d_ctx_timer_stop": (ctypes.c_int, [P, dp]),
        "fem2d_ctx_set_profiling": (ctypes.c_int, [P, ctypes.c_int]),
        "fem2d_ctx_profile_reset": (ctypes.c_int, [P]),
        "fem2d_ctx_profile_query": (ctypes.c_int, [P, ctypes.c_char_p, dp, i64p, dp]),
        "fem2d_ctx_profile_flops": (ctypes.c_int, [P, ctypes.c_char_p, dp]),
        "fem2d_ctx_fp64_peak": (ctypes.c_int, [P, dp]),
        "fem2d_ctx_mma_ns": (ctypes.c_int, [P, ctypes.c_int, dp]),
        "fem2d_dense_solve_gep": (ctypes.c_int, [P, P, d, dp, dp]),
        "fem2d_gep_shifted_solve": (ctypes.c_int, [P, P, d, d, ctypes.c_int, ctypes.c_int, dp, dp]),
        "fem2d_gpu_solve_gep": (ctypes.c_int, [P, P, d, ctypes.c_int, ctypes.POINTER(_fem2d_solve_opts), dp, dp, dp,
                                                ctypes.POINTER(_fem2d_solve_stats)]),
        "fem2d_gep_spmm_device": (ctypes.c_int, [P, P, d, d, ctypes.c_void_p, i64, ctypes.c_int, ctypes.c_void_p, i64]),
        "fem2d_gep_print_to_petsc_binary_files": (ctypes.c_int, [P, ctypes.c_char_p, ctypes.c_char_p]),
        "fem2d_aij_write": (ctypes.c_int, [ctypes.c_char_p, i64, i64p, i32p, dp]),
        "fem2d_aij_read": (ctypes.c_int, [ctypes.c_char_p, i64p, i64p, i64p, i32p, dp]),
        "fem2d_petsc_vec_write": (ctypes.c_int, [ctypes.c_char_p, dp, i64]),
        "fem2d_petsc_vec_read": (ctypes.c_int, [ctypes.c_char_p, dp, i64, i64p]),
        "fem2d_petsc_scalar_write": (ctypes.c_int, [ctypes.c_char_p, d]),
        "fem2d_petsc_scalar_read": (ctypes.c_int, [ctypes.c_char_p, dp]),
        "fem2d_fields_create": (ctypes.c_int, [P, P, ctypes.c_int, ctypes.c_int, ctypes.c_int, PP]),
        "fem2d_fields_free": (None, [P]),
        "fem2d_fields_num_leaves": (i64, [P]),
        "fem2d_fields_leaves": (ctypes.c_int, [P, i64p]),
        "fem2d_fields_leaf_bounds": (ctypes.c_int, [P, dp]),
        "fem2d_fields_xy": (ctypes.c_int, [P, dp, i64, dp, dp]),
        "fem2d_fields_xy_device": (ctypes.c_int, [P, ctypes.c_void_p, i64, ctypes.c_void_p, ctypes.c_void_p]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def _check(rc):
    if rc != 0:
        raise Fem2dError(rc, lib().fem2d_last_error().decode())


def _ptr(a, ct):
    return a.ctypes.data_as(ctypes.POINTER(ct)) if a is not None else None


def _ids(ids):
    if ids is None:
        return None, None, 0
    a = np.ascontiguousarray(np.asarray(list(ids), dtype=np.int64))
    return a, _ptr(a, ctypes.c_int64), len(a)


# ----------------------------------------------------------------------------- prelude-style types
class ContinuityCondition:
    HCurl, HDiv, Discontinuous = 0, 1, 2


class HRef:
    """h-refinement kinds (h_refinement.rs:56-61). Use HRef.T / HRef.U / HRef.V or HRef.u_extended(i)."""
    T, U, V = (0, -1), (1, -1), (2, -1)

    @staticmethod
    def t():
        return HRef.T

    @staticmethod
    def u():
        return HRef.U

    @staticmethod
    def v():
        return HRef.V

    @staticmethod
    def u_extended(child_idx):
        if child_idx not in (0, 1):
            raise Fem2dError(E_HREF, "Extended refinement index must be 0 or 1!")
        return (1, child_idx)

    @staticmethod
    def v_extended(child_idx):
        if child_idx not in (0, 1):
            raise Fem2dError(E_HREF, "Extended refinement index must be 0 or 1!")
        return (2, child_idx)


@dataclass(frozen=True)
class PRef:
    di: int
    dj: int

    @staticmethod
    def from_(di, dj):
        return PRef(di, dj)


@dataclass(frozen=True)
class Orders:
    i: int
    j: int


class HierPoly:
    ID = 0


class KOLeg:
    ID = 1


class CurlCurl:
    pass


class L2Inner:
    pass


class Mesh:
    """RBS mesh (src/fem_domain/domain/mesh.rs), held by the native library."""

    def __init__(self, handle):
        self._h = ctypes.c_void_p(handle)

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.fem2d_mesh_free(self._h)
            self._h = None

    @staticmethod
    def from_file(path):
        h = ctypes.c_void_p()
        _check(lib().fem2d_mesh_from_file(os.fsencode(path), ctypes.byref(h)))
        return Mesh(h.value)

    @staticmethod
    def from_json(text):
        h = ctypes.c_void_p()
        if not isinstance(text, (bytes, str)):
            import json
            text = json.dumps(text)
        if isinstance(text, str):
            text = text.encode()
        _check(lib().fem2d_mesh_from_json(text, ctypes.byref(h)))
        return Mesh(h.value)

    @staticmethod
    def unit():
        h = ctypes.c_void_p()
        _check(lib().fem2d_mesh_unit(ctypes.byref(h)))
        return Mesh(h.value)

    def clone(self):
        h = ctypes.c_void_p()
        _check(lib().fem2d_mesh_clone(self._h, ctypes.byref(h)))
        return Mesh(h.value)

    # p-refinement
    def set_global_expansion_orders(self, orders):
        _check(lib().fem2d_mesh_set_expansion_orders(self._h, None, 0, orders.i, orders.j))

    def set_expansion_on_elems(self, elems, orders):
        a, p, n = _ids(elems)
        _check(lib().fem2d_mesh_set_expansion_orders(self._h, p, n, orders.i, orders.j))

    def global_p_refinement(self, pref):
        _check(lib().fem2d_mesh_p_refine(self._h, None, 0, pref.di, pref.dj))

    def p_refine_elems(self, elems, pref):
        a, p, n = _ids(elems)
        _check(lib().fem2d_mesh_p_refine(self._h, p, n, pref.di, pref.dj))

    # h-refinement
    def global_h_refinement(self, href):
        _check(lib().fem2d_mesh_h_refine(self._h, None, 0, href[0], href[1]))

    def h_refine_elems(self, elems, href):
        a, p, n = _ids(elems)
        _check(lib().fem2d_mesh_h_refine(self._h, p, n, href[0], href[1]))

    def execute_h_refinements(self, refinements):
        """refinements: iterable of (elem_id, HRef) with HRef in {T, U, V} (mesh.rs:844-914)."""
        refinements = list(refinements)
        ids = np.ascontiguousarray(np.asarray([r[0] for r in refinements], dtype=np.int64))
        kinds = np.ascontiguousarray(np.asarray([r[1][0] for r in refinements], dtype=np.int32))
        _check(lib().fem2d_mesh_execute_h_refinements(self._h, _ptr(ids, ctypes.c_int64),
                                                      _ptr(kinds, ctypes.c_int32), len(ids)))

    def h_refine_with_filter(self, filt):
        """mesh.rs:728-750: filt(elem_info_row) -> HRef or None, over refineable (leaf) Elems."""
        info = self.elem_info()
        refs = []
        for e in range(len(info)):
            if info[e, 0] == 1:
                r = filt(e, info[e])
                if r is not None:
                    refs.append((e, r))
        if refs:
            self.execute_h_refinements(refs)

    # queries
    @property
    def num_elems(self):
        return lib().fem2d_mesh_num_elems(self._h)

    @property
    def num_edges(self):
        return lib().fem2d_mesh_num_edges(self._h)

    @property
    def num_nodes(self):
        return lib().fem2d_mesh_num_nodes(self._h)

    def elem_info(self):
        """Per Elem: [is_leaf, ni, nj, parent, nodes(4), edges(4), h_u, h_v]."""
        out = np.zeros((self.num_elems, 14), dtype=np.int64)
        _check(lib().fem2d_mesh_elem_info(self._h, _ptr(out, ctypes.c_int64)))
        return out

    def elem_bounds(self):
        out = np.zeros((self.num_elems, 4), dtype=np.float64)
        _check(lib().fem2d_mesh_elem_bounds(self._h, _ptr(out, ctypes.c_double)))
        return out


class Domain:
    """DoF enumeration (src/fem_domain/domain.rs:69-159)."""

    def __init__(self, handle):
        self._h = ctypes.c_void_p(handle)

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.fem2d_domain_free(self._h)
            self._h = None

    @staticmethod
    def from_mesh(mesh, cc=ContinuityCondition.HCurl):
        h = ctypes.c_void_p()
        _check(lib().fem2d_domain_from_mesh(mesh._h, cc, ctypes.byref(h)))
        return Domain(h.value)

    @property
    def num_dofs(self):
        return lib().fem2d_domain_num_dofs(self._h)

    def basis_specs(self):
        """Per spec: [elem_id, elem_idx, i, j, dir(0=U,1=V), dof_id] in Domain::basis_specs order."""
        n = lib().fem2d_domain_num_specs(self._h)
        out = np.zeros((n, 6), dtype=np.int64)
        _check(lib().fem2d_domain_basis_specs(self._h, _ptr(out, ctypes.c_int64)))
        return out


def domain_table_doubles(domain, bspace, glq=(0, 0)):
    """FP64 contraction-table size (doubles) a GEP of this Domain needs with basis space ``bspace``
    (HierPoly or KOLeg) and GLQ sizes ``glq`` (host only, no GPU)."""
    out = ctypes.c_int64(0)
    _check(lib().fem2d_domain_table_doubles(domain._h, int(bspace.ID), int(glq[0]), int(glq[1]), ctypes.byref(out)))
    return out.value


def domain_pattern(domain):
    """Upper-triangle keys (rows, cols) of the GEP sparsity pattern, built on the host."""
    nu = ctypes.c_int64()
    _check(lib().fem2d_domain_pattern(domain._h, ctypes.byref(nu), None, None))
    r = np.zeros(nu.value, np.int32)
    c = np.zeros(nu.value, np.int32)
    _check(lib().fem2d_domain_pattern(domain._h, ctypes.byref(nu), _ptr(r, ctypes.c_int32), _ptr(c, ctypes.c_int32)))
    return r, c


def factor_plan(domain):
    """The multifrontal factorization plan (host-only), as a dict of numpy arrays."""
    sz = np.zeros(8, np.int64)
    L = lib()
    _check(L.fem2d_domain_factor_plan(domain._h, _ptr(sz, ctypes.c_int64), *([None] * 8)))
    nf, nd, na, ne = (int(x) for x in sz[:4])
    fr = np.zeros((nf, 4), np.int32)
    dp = np.zeros(nf + 1, np.int64)
    dofs = np.zeros(nd, np.int32)
    ap = np.zeros(nf + 1, np.int64)
    apos = np.zeros(na, np.int64)
    acsr = np.zeros(na, np.int64)
    ep = np.zeros(nf + 1, np.int64)
    emap = np.zeros(ne, np.int32)
    c64, c32 = ctypes.c_int64, ctypes.c_int32
    _check(L.fem2d_domain_factor_plan(domain._h, _ptr(sz, c64), _ptr(fr, c32), _ptr(dp, c64), _ptr(dofs, c32),
                                      _ptr(ap, c64), _ptr(apos, c64), _ptr(acsr, c64), _ptr(ep, c64),
                                      _ptr(emap, c32)))
    return dict(sizes=sz, fronts=fr, dof_ptr=dp, dofs=dofs, asm_ptr=ap, asm_pos=apos, asm_csr=acsr, ea_ptr=ep,
                ea_map=emap)


class Context:
    """A CUDA device and stream owned by the native library."""

    _default = None

    def __init__(self, device=0):
        h = ctypes.c_void_p()
        _check(lib().fem2d_ctx_create(device, ctypes.byref(h)))
        self._h = h
        self.device = device

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.fem2d_ctx_destroy(self._h)
            self._h = None

    @classmethod
    def default(cls):
        if cls._default is None:
            cls._default = Context(0)
        return cls._default

    def synchronize(self):
        _check(lib().fem2d_ctx_synchronize(self._h))

    def flush_l2(self):
        _check(lib().fem2d_ctx_flush_l2(self._h))

    @property
    def kernel_launches(self):
        return lib().fem2d_ctx_kernel_launches(self._h)

    def timer_start(self):
        _check(lib().fem2d_ctx_timer_start(self._h))

    def timer_stop(self):
        ms = ctypes.c_double()
        _check(lib().fem2d_ctx_timer_stop(self._h, ctypes.byref(ms)))
        return ms.value

    def set_profiling(self, on):
        _check(lib().fem2d_ctx_set_profiling(self._h, 1 if on else 0))

    def profile_reset(self):
        _check(lib().fem2d_ctx_profile_reset(self._h))

    def profile(self, region):
        ms, cnt, by, fl = ctypes.c_double(), ctypes.c_int64(), ctypes.c_double(), ctypes.c_double()
        _check(lib().fem2d_ctx_profile_query(self._h, region.encode(), ctypes.byref(ms), ctypes.byref(cnt),
                                             ctypes.byref(by)))
        _check(lib().fem2d_ctx_profile_flops(self._h, region.encode(), ctypes.byref(fl)))
        return {"ms": ms.value, "count": cnt.value, "bytes": by.value, "flops": fl.value}

    def mma_ns(self, n):
        """Measured issue cost (ns per instruction and SM) of tcgen05.mma kind::f16, M = 128, K = 16, N = n."""
        t = ctypes.c_double()
        _check(lib().fem2d_ctx_mma_ns(self._h, int(n), ctypes.byref(t)))
        return t.value

    def fp64_peak(self):
        """Measured FP64 FMA throughput of the device in TFLOP/s (library microbenchmark)."""
        t = ctypes.c_double()
        _check(lib().fem2d_ctx_fp64_peak(self._h, ctypes.byref(t)))
        return t.value


class GEP:
    """A generalized eigenproblem whose A and B live in device memory (linalg.rs:29-57)."""

    def __init__(self, handle, ctx):
        self._h = ctypes.c_void_p(handle)
        self.ctx = ctx

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.fem2d_gep_free(self._h)
            self._h = None

    def dims(self):
        n, u, f = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        _check(lib().fem2d_gep_dims(self._h, ctypes.byref(n), ctypes.byref(u), ctypes.byref(f)))
        return n.value, u.value, f.value

    @property
    def dimension(self):
        return self.dims()[0]

    @property
    def num_visits(self):
        return lib().fem2d_gep_num_visits(self._h)

    @property
    def h2d_bytes(self):
        return lib().fem2d_gep_h2d_bytes(self._h)

    def recompute(self):
        _check(lib().fem2d_gep_recompute(self.ctx._h, self._h))

    def timings(self):
        """[tables, values, tables + values] ms of the last assembly, then [host symbolic, upload] ms."""
        out = np.zeros(5)
        _check(lib().fem2d_gep_timings(self._h, _ptr(out, ctypes.c_double)))
        return out

    def by_parts(self):
        """integrate_by_parts over the Galerkin visit set on the device: (rows, cols, vals) in upper_coo's
        order, vals[:, 0] the CurlCurl face term, vals[:, 1:5] its edge terms, vals[:, 5] the L2Inner
        value (integrals.rs:94-237, 356-418)."""
        r, c, _, _ = self.upper_coo()
        v = np.zeros((len(r), 6))
        _check(lib().fem2d_gep_by_parts(self.ctx._h, self._h, _ptr(v, ctypes.c_double)))
        return r, c, v

    def upper_coo(self):
        n, nu, nf = self.dims()
        r = np.zeros(nu, np.int32)
        c = np.zeros(nu, np.int32)
        a = np.zeros(nu)
        b = np.zeros(nu)
        _check(lib().fem2d_gep_export_upper(self._h, _ptr(r, ctypes.c_int32), _ptr(c, ctypes.c_int32),
                                            _ptr(a, ctypes.c_double), _ptr(b, ctypes.c_double)))
        return r, c, a, b

    def set_upper_values(self, a, b):
        """Replace A and B by the given upper-triangle values (in ``upper_coo`` order); the reference's
        GEP exposes its matrices as public fields (linalg.rs:29-34) that callers may edit."""
        n, nu, nf = self.dims()
        a = np.ascontiguousarray(a, dtype=np.float64)
        b = np.ascontiguousarray(b, dtype=np.float64)
        if a.shape != (nu,) or b.shape != (nu,):
            raise ValueError("expected %d upper-triangle values for A and for B" % nu)
        _check(lib().fem2d_gep_set_upper_values(self._h, _ptr(a, ctypes.c_double), _ptr(b, ctypes.c_double)))

    def csr(self, which):
        n, nu, nf = self.dims()
        rp = np.zeros(n + 1, np.int64)
        col = np.zeros(nf, np.int32)
        val = np.zeros(nf)
        _check(lib().fem2d_gep_export_csr(self._h, 0 if which in ("A", 0) else 1, _ptr(rp, ctypes.c_int64),
                                          _ptr(col, ctypes.c_int32), _ptr(val, ctypes.c_double)))
        return rp, col, val

    def shifted_solve(self, c_a, c_b, rhs, spd=False):
        """Solve (c_a A + c_b B) X = rhs (n or n x k) on the device with the multifrontal LU."""
        r = np.ascontiguousarray(np.asarray(rhs, dtype=np.float64))
        one = r.ndim == 1
        r2 = r.reshape(len(r), -1)
        x = np.zeros_like(r2)
        _check(lib().fem2d_gep_shifted_solve(self.ctx._h, self._h, float(c_a), float(c_b), 1 if spd else 0,
                                             r2.shape[1], _ptr(r2, ctypes.c_double), _ptr(x, ctypes.c_double)))
        return x[:, 0] if one else x

    def spmm_device(self, c_a, c_b, d_x, ldx, nb, d_y, ldy, ctx=None):
        """Y = c_a A X + c_b B X on the device (raw device pointers, row-major n x nb blocks)."""
        ctx = ctx or self.ctx
        _check(lib().fem2d_gep_spmm_device(ctx._h, self._h, float(c_a), float(c_b), ctypes.c_void_p(d_x), int(ldx),
                                           int(nb), ctypes.c_void_p(d_y), int(ldy)))

    def spmm_tensor_device(self, which, coef, d_x, ldx, nb, d_y, ldy, ctx=None):
        """Y = coef M X with M = A (which 0) or B (1) through the tensor-core product (synchronises)."""
        ctx = ctx or self.ctx
        _check(lib().fem2d_gep_spmm_tensor_device(ctx._h, self._h, int(which), float(coef), ctypes.c_void_p(d_x),
                                                  int(ldx), int(nb), ctypes.c_void_p(d_y), int(ldy)))

    def print_to_petsc_binary_files(self, dir, prefix):
        """GEP::print_to_petsc_binary_files (linalg.rs:44-52): {dir}/tmp/{prefix}_a.dat and _b.dat."""
        _check(lib().fem2d_gep_print_to_petsc_binary_files(self._h, str(dir).encode(), str(prefix).encode()))

    def scipy(self):
        import scipy.sparse as sp

        n = self.dimension
        out = []
        for w in ("A", "B"):
            rp, col, val = self.csr(w)
            out.append(sp.csr_matrix((val, col, rp), shape=(n, n)))
        return tuple(out)


def galerkin_sample_gep_hcurl(bspace, a_integral, b_integral, domain, glq_grid_dim=None, ctx=None):
    """galerkin_sample_gep_hcurl::<BSpace, CurlCurl, L2Inner>(&domain, glq_grid_dim) (galerkin.rs:33-187)."""
    if a_integral is not CurlCurl or b_integral is not L2Inner:
        raise Fem2dError(E_INVALID_ARG, "only <CurlCurl, L2Inner> is provided")
    ctx = ctx or Context.default()
    nu, nv = (0, 0) if glq_grid_dim is None else (int(glq_grid_dim[0]), int(glq_grid_dim[1]))
    h = ctypes.c_void_p()
    _check(lib().fem2d_galerkin_sample_gep_hcurl(ctx._h, domain._h, bspace.ID, nu, nv, ctypes.byref(h)))
    return GEP(h.value, ctx)


def _batch_report(rep):
    return {"ms_tables": float(rep[0]), "ms_values": float(rep[1]), "threads": int(rep[2]),
            "ctas_per_sm": int(rep[3]), "entries": int(rep[4]), "codes": int(rep[5])}


def galerkin_sample_gep_hcurl_batch(bspace, a_integral, b_integral, domains, glq_grid_dim=None, ctx=None,
                                    autotune=True):
    """galerkin_sample_gep_hcurl for many Domains: one GEP per Domain, the device numeric phase of all of
    them in one table launch plus one persistent value launch (launch shape autotuned and cached).

    Returns (list of GEP, report dict with the two launches' device times and the chosen launch shape).
    """
    if a_integral is not CurlCurl or b_integral is not L2Inner:
        raise Fem2dError(E_INVALID_ARG, "only <CurlCurl, L2Inner> is provided")
    ctx = ctx or Context.default()
    nu, nv = (0, 0) if glq_grid_dim is None else (int(glq_grid_dim[0]), int(glq_grid_dim[1]))
    n = len(domains)
    hs = (ctypes.c_void_p * max(n, 1))(*[d._h.value for d in domains])
    out = (ctypes.c_void_p * max(n, 1))()
    rep = np.zeros(6)
    _check(lib().fem2d_galerkin_sample_gep_hcurl_batch(ctx._h, hs, n, bspace.ID, nu, nv, 1 if autotune else 0, out,
                                                       _ptr(rep, ctypes.c_double)))
    return [GEP(out[i], ctx) for i in range(n)], _batch_report(rep)


def gep_batch_recompute(geps, ctx=None, autotune=True):
    """Recompute the values of many GEPs (same device) with the two batched launches; returns the report."""
    ctx = ctx or geps[0].ctx
    hs = (ctypes.c_void_p * max(len(geps), 1))(*[g._h.value for g in geps])
    rep = np.zeros(6)
    _check(lib().fem2d_gep_batch_recompute(ctx._h, hs, len(geps), 1 if autotune else 0, _ptr(rep, ctypes.c_double)))
    return _batch_report(rep)


def autotune_cache():
    """The autotuner's launch-shape cache as {key: (threads, ctas_per_sm)}."""
    n = ctypes.c_int64()
    _check(lib().fem2d_autotune_export(None, 0, ctypes.byref(n)))
    buf = ctypes.create_string_buffer(n.value + 1)
    _check(lib().fem2d_autotune_export(buf, n.value + 1, ctypes.byref(n)))
    out = {}
    for line in buf.value.decode().splitlines():
        k, t, c = line.split()
        out[k] = (int(t), int(c))
    return out


def autotune_save(path):
    """Write the autotuner cache to a JSON file."""
    import json

    with open(path, "w") as f:
        json.dump({k: list(v) for k, v in autotune_cache().items()}, f, indent=1, sort_keys=True)


def autotune_load(path):
    """Merge a JSON file written by autotune_save into the cache; returns the number of entries read."""
    import json

    with open(path) as f:
        d = json.load(f)
    text = "".join("%s %d %d\n" % (k, int(v[0]), int(v[1])) for k, v in d.items())
    n = ctypes.c_int64()
    _check(lib().fem2d_autotune_import(text.encode(), ctypes.byref(n)))
    return n.value


def autotune_clear():
    _check(lib().fem2d_autotune_clear())


def gpu_solve_gep_batch(geps, target, n_pairs, workers=8, device=None, **kw):
    """gpu_solve_gep_n for many independent GEPs on one GPU: `workers` host threads, each with its own
    Context (CUDA stream), so the small latency-bound solves of different meshes overlap on the device.
    Returns the list of SolveResult in input order (an exception of any solve is re-raised)."""
    import concurrent.futures as cf
    import threading

    dev = geps[0].ctx.device if device is None else device
    local = threading.local()

    def one(g):
        if getattr(local, "ctx", None) is None:
            local.ctx = Context(dev)
        return gpu_solve_gep_n(g, target, n_pairs, ctx=local.ctx, **kw)

    with cf.ThreadPoolExecutor(max_workers=max(1, workers)) as ex:
        return list(ex.map(one, geps))


# ----------------------------------------------------------------------------- external-solver files
def aij_write(path, row_ptr, col, val):
    """Full symmetric CSR -> the AIJMatrixBinary file layout (sparse_matrix.rs:184-265)."""
    rp = np.ascontiguousarray(row_ptr, dtype=np.int64)
    c = np.ascontiguousarray(col, dtype=np.int32)
    v = np.ascontiguousarray(val, dtype=np.float64)
    _check(lib().fem2d_aij_write(str(path).encode(), len(rp) - 1, _ptr(rp, ctypes.c_int64), _ptr(c, ctypes.c_int32),
                                 _ptr(v, ctypes.c_double)))


def aij_read(path):
    """AIJMatrixBinary (or standard PETSc AIJ) file -> (row_ptr, col, val)."""
    n, nnz = ctypes.c_int64(), ctypes.c_int64()
    _check(lib().fem2d_aij_read(str(path).encode(), ctypes.byref(n), ctypes.byref(nnz), None, None, None))
    rp = np.zeros(n.value + 1, dtype=np.int64)
    c = np.zeros(nnz.value, dtype=np.int32)
    v = np.zeros(nnz.value)
    _check(lib().fem2d_aij_read(str(path).encode(), ctypes.byref(n), ctypes.byref(nnz), _ptr(rp, ctypes.c_int64),
                                _ptr(c, ctypes.c_int32), _ptr(v, ctypes.c_double)))
    return rp, c, v


def petsc_vec_write(path, values):
    v = np.ascontiguousarray(values, dtype=np.float64)
    _check(lib().fem2d_petsc_vec_write(str(path).encode(), _ptr(v, ctypes.c_double), len(v)))


def retrieve_eigenvector(path):
    """retrieve_eigenvector (slepc_solve.rs:114-135)."""
    n = ctypes.c_int64()
    _check(lib().fem2d_petsc_vec_read(str(path).encode(), None, 0, ctypes.byref(n)))
    v = np.zeros(n.value)
    _check(lib().fem2d_petsc_vec_read(str(path).encode(), _ptr(v, ctypes.c_double), len(v), ctypes.byref(n)))
    return v


def petsc_scalar_write(path, value):
    _check(lib().fem2d_petsc_scalar_write(str(path).encode(), float(value)))


def retrieve_eigenvalue(path):
    """retrieve_eigenvalue (slepc_solve.rs:137-147)."""
    x = ctypes.c_double()
    _check(lib().fem2d_petsc_scalar_read(str(path).encode(), ctypes.byref(x)))
    return x.value


def retrieve_solution(dir, prefix):
    """retrieve_solution (slepc_solve.rs:104-112): {dir}/tmp/{prefix}_evec.dat and _eval.dat."""
    base = os.path.join(str(dir), "tmp", str(prefix))
    return EigenPair(retrieve_eigenvalue(base + "_eval.dat"), retrieve_eigenvector(base + "_evec.dat"))


@dataclass
class EigenPair:
    """linalg.rs:84-96"""
    value: float
    vector: np.ndarray
    residual: float = float("nan")

    def normalized_eigenvector(self):
        return self.vector / np.linalg.norm(self.vector)


@dataclass
class SolveResult:
    values: np.ndarray
    vectors: np.ndarray
    residuals: np.ndarray
    stats: dict = field(default_factory=dict)

    def pairs(self):
        return [EigenPair(float(v), self.vectors[k], float(self.residuals[k])) for k, v in enumerate(self.values)]


def nalgebra_solve_gep(gep, target_eigenvalue):
    """nalgebra_solve_gep (nalgebra_solve.rs:14-50) computed on the device; ndofs <= 1000."""
    n = gep.dimension
    val = ctypes.c_double()
    vec = np.zeros(n)
    _check(lib().fem2d_dense_solve_gep(gep.ctx._h, gep._h, float(target_eigenvalue), ctypes.byref(val),
                                       _ptr(vec, ctypes.c_double)))
    return EigenPair(val.value, vec)


PRECOND_EXACT, PRECOND_PLAIN, PRECOND_LEARNED = 0, 1, 2
PRECOND_BLOCK_JACOBI = PRECOND_PLAIN
GRAM_TENSOR, GRAM_FP64 = 0, 1


def block_gram_device(ctx, method, n, d_x, ldx, a, d_y, ldy, b, d_c):
    """C = X^T Y on device blocks (raw pointers, row-major): method GRAM_TENSOR (tcgen05 FP64 emulation)
    or GRAM_FP64 (CUDA cores). Synchronises."""
    _check(lib().fem2d_block_gram_device(ctx._h, int(method), int(n), ctypes.c_void_p(d_x), int(ldx), int(a),
                                         ctypes.c_void_p(d_y), int(ldy), int(b), ctypes.c_void_p(d_c)))


def block_gemm_device(ctx, method, n, d_x, ldx, a, d_c, b, alpha, beta, d_z, ldz):
    """Z = beta Z + alpha X C on device blocks (raw pointers, row-major; C is a x b): method GRAM_TENSOR
    (tcgen05 FP64 emulation) or GRAM_FP64 (CUDA cores). Synchronises."""
    _check(lib().fem2d_block_gemm_device(ctx._h, int(method), int(n), ctypes.c_void_p(d_x), int(ldx), int(a),
                                         ctypes.c_void_p(d_c), int(b), float(alpha), float(beta), ctypes.c_void_p(d_z),
                                         int(ldz)))


def gpu_solve_gep_n(gep, target_eigenvalue, n_pairs, precond=0, tol=0.0, max_outer=0,
                    max_inner=0, inner_tol=0.0, block=0, verbose=0, ctx=None, krylov_steps=0, damping=0.0, scaling=0,
                    dense=0, net=None, refine=0):
    """The n_pairs eigenpairs nearest target by the device shift-invert solver (on ctx's stream; default:
    the context the GEP was built on). dense=0 (default) runs the Gram products and block updates from 50,000
    DoFs, and the operator products from 1,000,000 nonzeros, on the tensor cores (FP64 emulation); dense=1 keeps
    everything on the FP64 CUDA cores; dense=2 uses the tensor cores for all of them at every size; dense=3 uses
    them for the Gram products and block updates at every size and keeps the operator products on the CUDA cores. precond: PRECOND_EXACT (multifrontal LU, default), PRECOND_PLAIN
    (inner CG / MINRES with the additive-Schwarz preconditioner) or PRECOND_LEARNED (the same with the
    two-level preconditioner of the trained PatchNet `net`)."""
    ctx = ctx or gep.ctx
    n = gep.dimension
    vals = np.zeros(n_pairs)
    vecs = np.zeros((n_pairs, n))
    res = np.zeros(n_pairs)
    o = _fem2d_solve_opts(precond, max_outer, max_inner, tol, inner_tol, block, verbose, krylov_steps, damping,
                          scaling, dense, net._h if net is not None else None, refine)
    st = _fem2d_solve_stats()
    _check(lib().fem2d_gpu_solve_gep(ctx._h, gep._h, float(target_eigenvalue), int(n_pairs), ctypes.byref(o),
                                     _ptr(vals, ctypes.c_double), _ptr(vecs, ctypes.c_double),
                                     _ptr(res, ctypes.c_double), ctypes.byref(st)))
    stats = {k: getattr(st, k) for k, _ in _fem2d_solve_stats._fields_}
    return SolveResult(vals, vecs, res, stats)


def gpu_solve_gep(gep, target_eigenvalue, **kw):
    """gpu_solve_gep(gep, target) -> EigenPair, beside slepc_solve_gep (slepc_solve.rs:14-68)."""
    return gpu_solve_gep_n(gep, target_eigenvalue, 1, **kw).pairs()[0]


from .fields import UniformFieldError, UniformFieldSpace  # noqa: E402
from .learned import PCG, PatchNet, harvest_errors, patch_features  # noqa: E402
