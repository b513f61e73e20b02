"""The oracle and the mesh pass pinned against the reference's own code.

tests/golden/ref_*.npz hold what the unmodified warp_cfd solver computed when run on the
numpy Warp stand-in (tests/golden/make_reference_golden.py): its mesh pass's arrays, the
boundary table and the fields after a fixed number of SIMPLE iterations (PISO time
steps), in float64 with the Krylov solves tightened to 1e-13.

* The oracle (oracle/simple_ref.py, float64, the same tightened stop), given the
  reference's own mesh arrays, must reproduce the reference's fields to 1e-9 on every
  case: steady cavity, channel, skew-corrected and non-orthogonally corrected jittered
  cavities, PISO.
* This package's host mesh pass (warpcfd_gb300.preprocess.Mesh) on the same grid must
  give the reference's topology exactly and its float32 geometry to the reference's own
  float32 rounding (~1e-6 on the normals of jittered cells).
"""
import glob
import os

import numpy as np
import pytest

from oracle.simple_ref import OracleCase, geometry_from_reference_arrays

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FIXTURES = sorted(glob.glob(os.path.join(GOLDEN, "ref_*.npz")))
NAMES = [os.path.basename(p)[:-4] for p in FIXTURES]


def load(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def oracle_run(d, T=np.float64, atol=None, maxiter=None, p_refine=0):
    ref = int(d["reference_cell"])
    oc = OracleCase(geometry_from_reference_arrays(d), d["bc_type"], d["bc_value"], float(d["viscosity"]),
                    float(d["density"]), T=T, reference_cell=None if ref < 0 else ref,
                    correction=bool(d["correction"]), atol=float(d["tol"]) if atol is None else atol,
                    maxiter=int(d["maxiter"]) if maxiter is None else maxiter, p_refine=p_refine)
    if bool(d["piso"]):
        oc.run(None, None, n_outer=1, n_inner=int(d["correctors"]), steady=False, n_time=int(d["steps"]),
               dt=float(d["dt"]))
    else:
        r = d["relax"]
        oc.run(float(r[0]), float(r[1]), n_outer=int(d["steps"]))
    return oc.cell_values.astype(np.float64)


def field_errors(got, ref):
    """u, v, w on the velocity scale ||U_ref||; p relative to ||p_ref||."""
    un = np.linalg.norm(ref[:, 0:3])
    out = {f: float(np.linalg.norm(got[:, i] - ref[:, i]) / un) for i, f in enumerate("uvw")}
    out["p"] = float(np.linalg.norm(got[:, 3] - ref[:, 3]) / np.linalg.norm(ref[:, 3]))
    return out


def test_reference_fixtures_present():
    assert {"ref_ldc16", "ref_channel80x16", "ref_ldc12_skew", "ref_ldc12_corrected", "ref_piso_ldc12"} <= set(NAMES)


@pytest.mark.parametrize("name", NAMES)
def test_oracle_reproduces_the_reference(name):
    d = load(name)
    ref = d["cell_values"]
    assert np.isfinite(ref).all() and np.abs(ref[:, 0:2]).max() > 1e-2   # a flow, not zeros
    e = field_errors(oracle_run(d), ref)
    print(name, e)
    assert max(e.values()) <= 1e-9, e


def _grid_for(name):
    from warpcfd_gb300.preprocess.grid import create_2D_grid

    if "channel" in name:
        return create_2D_grid((0, 0, 0), 80, 16, 10.0, 1.0, 0.1)
    if "ldc16" in name:
        return create_2D_grid((0, 0, 0), 16, 16, 1.0, 1.0, 0.1)
    if "skew" in name or "corrected" in name:
        return create_2D_grid((0, 0, 0), 12, 12, 1.0, 1.0, 0.1, jitter=0.2, seed=1)
    return create_2D_grid((0, 0, 0), 12, 12, 1.0, 1.0, 0.1)


@pytest.mark.parametrize("name", NAMES)
def test_mesh_pass_matches_the_reference(name):
    from warpcfd_gb300.preprocess import Mesh

    d = load(name)
    m = Mesh(_grid_for(name))
    cp, fp = m.cell_properties, m.face_properties
    assert np.array_equal(m.cells, d["mesh_cells"])
    for ours, key in ((cp.faces, "cell_faces"), (cp.neighbors, "cell_neighbors"), (cp.face_side, "cell_face_side"),
                      (cp.nnz_per_cell, "cell_nnz_per_cell"), (cp.face_offset_index, "cell_face_offset_index"),
                      (fp.unique_faces, "face_unique_faces"), (fp.adjacent_cells, "face_adjacent_cells"),
                      (fp.cell_face_index, "face_cell_face_index"), (fp.is_boundary, "face_is_boundary"),
                      (fp.boundary_face_ids, "face_boundary_face_ids"),
                      (fp.internal_face_ids, "face_internal_face_ids")):
        assert np.array_equal(np.asarray(ours), d["mesh_" + key]), key
    for ours, key in ((cp.normal, "cell_normal"), (cp.area, "cell_area"), (cp.centroids, "cell_centroids"),
                      (cp.volumes, "cell_volumes"), (cp.cell_centroid_to_face_centroid,
                                                     "cell_cell_centroid_to_face_centroid"),
                      (fp.centroid, "face_centroid"), (fp.distance, "face_distance")):
        a, b = np.asarray(ours, dtype=np.float64), d["mesh_" + key].astype(np.float64)
        assert a.shape == b.shape, key
        # the reference computes its geometry in float32 (preprocess/mesh.py:161-183: cross
        # products of node differences), this package in float64 rounded once: on jittered
        # cells the reference's normals carry ~1e-6 of float32 cancellation error
        assert np.allclose(a, b, rtol=1e-5, atol=2e-6), (key, np.abs(a - b).max())
