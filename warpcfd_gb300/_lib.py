"""ctypes binding of libwcfd.so (the C ABI in include/wcfd.h).

The library is the only compute path: if it cannot be loaded every operation raises,
there is no CPU or PyTorch fallback.
"""
from __future__ import annotations

import ctypes as ct
import os
from pathlib import Path

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "libwcfd.so"

WCFD_OK = 0
WCFD_ERR_ARGUMENT = 1
WCFD_ERR_CUDA = 2
WCFD_KRYLOV_BREAKDOWN = 3
WCFD_NOT_CONVERGED = 4
WCFD_BARRIER_TIMEOUT = 5
WCFD_ERR_TOO_LARGE = 6
STATUS_NAMES = {0: "ok", 1: "bad argument", 2: "cuda error", 3: "krylov breakdown", 4: "not converged",
                5: "barrier timeout", 6: "too large"}

WCFD_U, WCFD_V, WCFD_W, WCFD_P, WCFD_ALL = 1, 2, 4, 8, 15
# wcfd_params.convection per ConvectionTerm interpolation scheme
CONVECTION = {"upwind": 0, "upwindLinear": 0, "central difference": 1}
MAX_BLOCKS = 2048
BARRIER_WORDS = MAX_BLOCKS + 4
STATS_BYTES = 32

try:  # numpy view of wcfd_solve_stats
    import numpy as _np
    STATS_DTYPE = _np.dtype([("iterations", "<i4"), ("status", "<i4"), ("residual", "<f8"),
                             ("initial_residual", "<f8"), ("rhs_norm", "<f8")])
except ImportError:  # pragma: no cover
    STATS_DTYPE = None

vp = ct.c_void_p


class Mesh_t(ct.Structure):
    _fields_ = [("n_cells", ct.c_int32), ("n_faces", ct.c_int32), ("n_bfaces", ct.c_int32),
                ("faces_per_cell", ct.c_int32), ("ell_width", ct.c_int32), ("pad_", ct.c_int32),
                ("face_owner", vp), ("face_nbr", vp), ("face_brow", vp), ("face_interp", vp),
                ("face_normal", vp), ("face_gdiff", vp), ("face_rpf", vp), ("cell_slot", vp),
                ("cell_volume", vp), ("ell_col", vp), ("boundary_face", vp), ("face_dvec", vp),
                ("ell_dcol", vp)]


class BC_t(ct.Structure):
    _fields_ = [("type", vp), ("value", vp)]


class State_t(ct.Structure):
    _fields_ = [("cell_values", vp), ("cell_gradients", vp), ("face_values", vp),
                ("face_gradients", vp), ("mass_fluxes", vp)]


class System_t(ct.Structure):
    _fields_ = [("diag", vp), ("off", vp), ("rhs", vp), ("ncomp", ct.c_int32), ("pad_", ct.c_int32)]


class KrylovWS_t(ct.Structure):
    _fields_ = [("vec", vp), ("partials", vp), ("results", vp), ("barrier", vp)]


class Stats_t(ct.Structure):
    _fields_ = [("iterations", ct.c_int32), ("status", ct.c_int32), ("residual", ct.c_double),
                ("initial_residual", ct.c_double), ("rhs_norm", ct.c_double)]


class Params_t(ct.Structure):
    _fields_ = [("nu", ct.c_float), ("rho", ct.c_float), ("u_relax", ct.c_float), ("p_relax", ct.c_float),
                ("dt", ct.c_float), ("ref_value", ct.c_float), ("ref_cell", ct.c_int32), ("steady", ct.c_int32),
                ("n_inner", ct.c_int32), ("n_ortho", ct.c_int32), ("maxiter", ct.c_int32), ("skew", ct.c_int32),
                ("atol_u", ct.c_double), ("atol_p", ct.c_double), ("p_refine", ct.c_int32), ("rhie_chow", ct.c_int32),
                ("p_refine_rtol", ct.c_double), ("rtol_u", ct.c_double), ("rtol_p", ct.c_double),
                ("explicit_terms", ct.c_int32), ("convection", ct.c_int32)]


class Case_t(ct.Structure):
    _fields_ = [("mesh", Mesh_t), ("bc", BC_t), ("state", State_t), ("mom", System_t), ("pres", System_t),
                ("hbya", vp), ("p_x", vp), ("rua", vp), ("rua_faces", vp), ("div", vp), ("p_x64", vp), ("p_work", vp),
                ("ws_u", KrylovWS_t), ("ws_p", KrylovWS_t), ("stats", vp), ("prm", Params_t),
                ("events", vp)]


class BatchDims_t(ct.Structure):
    _fields_ = [("max_cells", ct.c_int32), ("max_faces", ct.c_int32), ("faces_per_cell", ct.c_int32),
                ("ell_width", ct.c_int32), ("n_inner", ct.c_int32), ("n_ortho", ct.c_int32),
                ("cluster_size", ct.c_int32), ("field_block", ct.c_int32), ("explicit_terms", ct.c_int32),
                ("p_refine", ct.c_int32), ("cg_variant", ct.c_int32)]


class TermFields_t(ct.Structure):
    _fields_ = [("n", ct.c_int32), ("index", ct.c_int32 * 3)]


class Term_t(ct.Structure):
    _fields_ = [("weights", vp), ("scale", ct.c_float), ("cell_based", ct.c_int32)]


MAX_TERMS = 8


class MeshCells_t(ct.Structure):
    _fields_ = [("n_cells", ct.c_int32), ("n_points", ct.c_int32), ("faces_per_cell", ct.c_int32),
                ("tri_slots", ct.c_int32), ("quad_slots", ct.c_int32), ("pad_", ct.c_int32),
                ("points", vp), ("cells", vp), ("cell_type", vp)]


class MeshFaces_t(ct.Structure):
    _fields_ = [("cell_faces", vp), ("unique_faces", vp), ("face_nodes", vp), ("face_cells", vp),
                ("face_slots", vp), ("centroid", vp), ("volume", vp), ("area", vp), ("normal", vp),
                ("to_face", vp), ("face_centroid", vp), ("node_width", ct.c_int32), ("pad_", ct.c_int32)]


# name -> (restype, argtypes)
_SIGS = {
    "wcfd_version": (ct.c_int, []),
    "wcfd_last_error": (ct.c_char_p, []),
    "wcfd_krylov_workspace_floats": (ct.c_int64, [ct.c_int32, ct.c_int32]),
    "wcfd_set_boundary_conditions": (ct.c_int, [ct.POINTER(Mesh_t), BC_t, State_t, vp]),
    "wcfd_face_interpolation": (ct.c_int, [ct.POINTER(Mesh_t), BC_t, State_t, ct.c_uint32, ct.c_int32,
                                           ct.c_int32, vp]),
    "wcfd_face_pass_flags": (ct.c_int, [ct.POINTER(Mesh_t), BC_t, State_t, ct.c_uint32, ct.c_uint32, vp]),
    "wcfd_calculate_mass_flux": (ct.c_int, [ct.POINTER(Mesh_t), State_t, vp]),
    "wcfd_calculate_gradients": (ct.c_int, [ct.POINTER(Mesh_t), State_t, ct.c_uint32, vp]),
    "wcfd_div_flux": (ct.c_int, [ct.POINTER(Mesh_t), vp, vp, vp]),
    "wcfd_cell_to_face": (ct.c_int, [ct.POINTER(Mesh_t), vp, vp, vp]),
    "wcfd_assemble_momentum": (ct.c_int, [ct.POINTER(Case_t), vp]),
    "wcfd_assemble_pressure": (ct.c_int, [ct.POINTER(Case_t), vp]),
    "wcfd_spmv": (ct.c_int, [ct.POINTER(Mesh_t), System_t, vp, vp, vp]),
    "wcfd_cg": (ct.c_int, [ct.POINTER(Mesh_t), System_t, vp, KrylovWS_t, ct.c_double, ct.c_int32, vp, vp]),
    "wcfd_bicgstab": (ct.c_int, [ct.POINTER(Mesh_t), System_t, vp, KrylovWS_t, ct.c_double, ct.c_int32, vp, vp]),
    "wcfd_rua": (ct.c_int, [ct.POINTER(Mesh_t), vp, ct.c_float, vp, vp]),
    "wcfd_hbya_add": (ct.c_int, [ct.c_int32, vp, vp, vp, vp]),
    "wcfd_relax": (ct.c_int, [ct.POINTER(Mesh_t), System_t, vp, ct.c_int32, ct.c_float, vp]),
    "wcfd_convection_weights": (ct.c_int, [ct.POINTER(Mesh_t), State_t, TermFields_t, ct.c_int32, vp, vp]),
    "wcfd_diffusion_weights": (ct.c_int, [ct.POINTER(Mesh_t), BC_t, State_t, TermFields_t, ct.c_float, vp, ct.c_int32,
                                          ct.c_int32, ct.c_float, vp, vp]),
    "wcfd_ddt_weights": (ct.c_int, [ct.POINTER(Mesh_t), State_t, TermFields_t, ct.c_float, vp, vp]),
    "wcfd_grad_weights": (ct.c_int, [ct.POINTER(Mesh_t), State_t, ct.c_int32, vp, vp]),
    "wcfd_assemble_terms": (ct.c_int, [ct.POINTER(Mesh_t), System_t, ct.POINTER(Term_t), ct.c_int32, vp]),
    "wcfd_add_rhs": (ct.c_int, [vp, vp, ct.c_float, ct.c_int64, vp]),
    "wcfd_replace_row": (ct.c_int, [ct.POINTER(Mesh_t), System_t, ct.c_int32, ct.c_float, vp]),
    "wcfd_krylov_solve": (ct.c_int, [ct.POINTER(Mesh_t), System_t, vp, KrylovWS_t, ct.c_int32, ct.c_double,
                                     ct.c_double, ct.c_int32, vp, vp]),
    "wcfd_simple_iteration": (ct.c_int, [ct.POINTER(Case_t), vp]),
    "wcfd_set_krylov_path": (ct.c_int, [ct.c_int32]),
    "wcfd_cg_refine": (ct.c_int, [ct.POINTER(Mesh_t), System_t, vp, vp, vp, KrylovWS_t, ct.c_int32, ct.c_double,
                                  ct.c_int32, vp, vp]),
    "wcfd_cg_noalloc": (ct.c_int, [ct.POINTER(Mesh_t), System_t, vp, ct.c_double, ct.c_int32, vp, vp]),
    "wcfd_batch_cluster_size": (ct.c_int, [ct.POINTER(BatchDims_t)]),
    "wcfd_batch_max_rows": (ct.c_int, [ct.c_int32]),
    "wcfd_batch_prepare": (ct.c_int, [ct.POINTER(BatchDims_t)]),
    "wcfd_convergence_scratch_floats": (ct.c_int64, []),
    "wcfd_convergence_norms": (ct.c_int, [ct.POINTER(Mesh_t), System_t, vp, vp, vp, vp, vp, vp, vp, vp]),
    "wcfd_batch_simple_iteration": (ct.c_int, [vp, ct.c_int32, ct.POINTER(BatchDims_t), vp]),
    "wcfd_batch_last_error": (ct.c_char_p, []),
    "wcfd_mesh_workspace_bytes": (ct.c_size_t, [ct.POINTER(MeshCells_t)]),
    "wcfd_mesh_match_faces": (ct.c_int, [ct.POINTER(MeshCells_t), vp, ct.c_size_t, ct.POINTER(ct.c_int32), vp]),
    "wcfd_mesh_emit": (ct.c_int, [ct.POINTER(MeshCells_t), vp, ct.c_size_t, ct.POINTER(ct.c_int32),
                                  ct.POINTER(MeshFaces_t), vp]),
    "wcfd_mesh_last_error": (ct.c_char_p, []),
    "wcfd_check_mesh": (ct.c_int, [ct.POINTER(Mesh_t), ct.POINTER(ct.c_int32), vp]),
    "wcfd_grid_barrier_check": (ct.c_int, [ct.c_int32, ct.c_int32, ct.POINTER(ct.c_int32), vp]),
}

EXPORTED = tuple(_SIGS.keys())


class WcfdError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"libwcfd error {code} ({STATUS_NAMES.get(code, '?')}): {msg}")
        self.code = code


_lib = None


def load(path: str | os.PathLike | None = None):
    """Load libwcfd.so once; raise ImportError (never fall back) if it is missing."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise ImportError(f"{p} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
                          "(warpcfd_gb300.build.build_library); there is no CPU fallback")
    lib = ct.CDLL(str(p))
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def check(rc: int):
    if rc != WCFD_OK:
        raise WcfdError(rc, load().wcfd_last_error().decode(errors="replace"))


def call(name: str, *args):
    check(getattr(load(), name)(*args))
