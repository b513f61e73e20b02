"""The C-ABI library builds, loads and exports every entry point include/wcfd.h
declares; struct layouts agree with the header; argument errors come back as status
codes without touching a GPU."""
import ctypes as ct
import os
import re
import subprocess

import pytest

from tests.conftest import ROOT

HEADER = os.path.join(ROOT, "include", "wcfd.h")


def declared():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(wcfd_[a-z0-9_]+)\s*\(", src)))


def test_exports_every_declared_symbol(built_lib):
    from warpcfd_gb300 import _lib

    lib = ct.CDLL(str(built_lib))
    names = declared()
    assert "wcfd_simple_iteration" in names and len(names) >= 15
    for n in names:
        assert hasattr(lib, n), n
    assert set(_lib.EXPORTED) <= set(names)
    out = subprocess.run(["nm", "-D", "--defined-only", str(built_lib)], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (wcfd_\w+)", out))
    assert set(names) <= exported


def test_struct_layout_matches_header(tmp_path):
    from warpcfd_gb300 import _lib

    prog = tmp_path / "layout.c"
    prog.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "wcfd.h"\nint main(){printf("%zu %zu %zu '
                    '%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\\n", sizeof(wcfd_mesh), sizeof(wcfd_bc), '
                    'sizeof(wcfd_state), sizeof(wcfd_system), sizeof(wcfd_krylov_ws), sizeof(wcfd_solve_stats), '
                    'sizeof(wcfd_params), sizeof(wcfd_case), offsetof(wcfd_case, prm), offsetof(wcfd_case, stats), '
                    'sizeof(wcfd_mesh_cells), sizeof(wcfd_mesh_faces), offsetof(wcfd_mesh_faces, node_width), '
                    'sizeof(wcfd_batch_dims)); printf("%zu %zu %zu %zu %zu %zu %zu\\n", sizeof(wcfd_term_fields), '
                    'sizeof(wcfd_term), offsetof(wcfd_term, scale), offsetof(wcfd_batch_dims, p_refine), '
                    '(size_t)WCFD_MAX_TERMS, offsetof(wcfd_mesh, ell_dcol), offsetof(wcfd_batch_dims, cg_variant));}\n')
    exe = tmp_path / "layout"
    subprocess.run(["gcc", f"-I{os.path.join(ROOT, 'include')}", str(prog), "-o", str(exe)], check=True)
    got = list(map(int, subprocess.run([str(exe)], capture_output=True, text=True).stdout.split()))
    want = [ct.sizeof(t) for t in (_lib.Mesh_t, _lib.BC_t, _lib.State_t, _lib.System_t, _lib.KrylovWS_t,
                                   _lib.Stats_t, _lib.Params_t, _lib.Case_t)]
    want += [_lib.Case_t.prm.offset, _lib.Case_t.stats.offset, ct.sizeof(_lib.MeshCells_t),
             ct.sizeof(_lib.MeshFaces_t), _lib.MeshFaces_t.node_width.offset, ct.sizeof(_lib.BatchDims_t)]
    want += [ct.sizeof(_lib.TermFields_t), ct.sizeof(_lib.Term_t), _lib.Term_t.scale.offset,
             _lib.BatchDims_t.p_refine.offset, _lib.MAX_TERMS, _lib.Mesh_t.ell_dcol.offset,
             _lib.BatchDims_t.cg_variant.offset]
    assert got == want


def test_argument_errors_are_status_codes(built_lib):
    from warpcfd_gb300 import _lib

    lib = _lib.load()
    assert lib.wcfd_version() >= 100
    assert lib.wcfd_krylov_workspace_floats(100, 1) == 600
    assert lib.wcfd_krylov_workspace_floats(100, 3) == 2700
    assert lib.wcfd_krylov_workspace_floats(0, 1) == -1
    rc = lib.wcfd_simple_iteration(None, None)
    assert rc == _lib.WCFD_ERR_ARGUMENT
    assert b"null" in lib.wcfd_last_error()
    m = _lib.Mesh_t()
    m.n_cells, m.n_faces, m.faces_per_cell, m.ell_width = 10, 20, 7, 0
    assert lib.wcfd_div_flux(ct.byref(m), None, None, None) == _lib.WCFD_ERR_ARGUMENT
    with pytest.raises(_lib.WcfdError):
        _lib.call("wcfd_div_flux", ct.byref(m), None, None, None)


def test_missing_library_fails_loudly(tmp_path):
    from warpcfd_gb300 import _lib

    with pytest.raises(ImportError):
        _lib.load(tmp_path / "nope.so")


def test_misaligned_krylov_partials_are_refused(built_lib):
    """wcfd_cg refuses a partial-sum buffer that is not 16-byte aligned (the grid barrier
    stores each block's sums there as one float4) before any device call: path 1 (grid
    solver only) skips the cluster set-up, and the pointers below are only checked, never
    dereferenced."""
    from warpcfd_gb300 import _lib

    lib = _lib.load()
    buf = (ct.c_double * 64)()
    base = (ct.addressof(buf) + 15) // 16 * 16
    m = _lib.Mesh_t()
    m.n_cells, m.n_faces, m.faces_per_cell, m.ell_width = 10, 20, 4, 4
    for name, typ in _lib.Mesh_t._fields_:
        if typ is ct.c_void_p:
            setattr(m, name, base)
    A = _lib.System_t(base, base, base, 1, 0)
    ws = _lib.KrylovWS_t(base, base + 8, None, base)
    assert lib.wcfd_set_krylov_path(1) == 0
    try:
        rc = lib.wcfd_cg(ct.byref(m), A, ct.c_void_p(base), ws, 1e-6, 10, ct.c_void_p(base), ct.c_void_p(None))
    finally:
        lib.wcfd_set_krylov_path(0)
    assert rc == _lib.WCFD_ERR_ARGUMENT
    assert b"16-byte" in lib.wcfd_last_error()
