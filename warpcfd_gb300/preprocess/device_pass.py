"""Face matching and mesh geometry on the GPU (libwcfd's mesh pass, ``wcfd_mesh_*``).

The preprocessing of warp_cfd/preprocess/mesh.py:64-302 for meshes of millions of cells:
the host pass spends its time sorting the (cell, face) node rows and in the vectorised
fan triangulation; here both run in CUDA kernels (a counting sort on each face's lowest
node id, per-node bucket sorts, float64 geometry in the host pass's order of operations)
and only the finished arrays come back to the host.  The topology (face numbering, owner
and neighbour, slots) is bit-identical to the host pass.  There is no fallback: without
the library or a CUDA device this raises.
"""
from __future__ import annotations

import ctypes as ct

import numpy as np

from .mesh import CELL_FACES


def _slots(types) -> tuple[int, int, int]:
    present = [int(t) for t in np.unique(types)]
    F = max(len(CELL_FACES[t]) for t in present)
    tri = max(sum(1 for f in CELL_FACES[t] if len(f) == 3) for t in present)
    quad = max(sum(1 for f in CELL_FACES[t] if len(f) == 4) for t in present)
    return F, tri, quad


def device_topology(mesh, device) -> dict:
    """The raw arrays of ``Mesh._host_topology`` (plus the cell volumes), computed on
    ``device``."""
    import torch

    from .. import _lib

    lib = _lib.load()
    dev = torch.device(device)
    if dev.type != "cuda":
        raise ValueError("the device mesh pass needs a CUDA device")
    C = int(mesh.cells.shape[0])
    P = int(mesh._nodes64.shape[0])
    F, tri, quad = _slots(mesh.cell_types)
    conn = np.full((C, 8), -1, dtype=np.int32)
    conn[:, :mesh.cells.shape[1]] = mesh.cells
    pts_d = torch.from_numpy(np.ascontiguousarray(mesh._nodes64)).to(dev)
    conn_d = torch.from_numpy(conn).to(dev)
    type_d = torch.from_numpy(np.ascontiguousarray(mesh.cell_types, dtype=np.int32)).to(dev)
    mc = _lib.MeshCells_t(C, P, F, tri, quad, 0, pts_d.data_ptr(), conn_d.data_ptr(), type_d.data_ptr())
    ws_bytes = int(lib.wcfd_mesh_workspace_bytes(ct.byref(mc)))
    if ws_bytes == 0:
        raise _lib.WcfdError(_lib.WCFD_ERR_ARGUMENT, lib.wcfd_mesh_last_error().decode(errors="replace"))
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=dev)
    stream = ct.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    n_faces = (ct.c_int32 * 2)()

    def check(rc):
        if rc != _lib.WCFD_OK:
            raise _lib.WcfdError(rc, lib.wcfd_mesh_last_error().decode(errors="replace"))

    with torch.cuda.device(dev):
        check(lib.wcfd_mesh_match_faces(ct.byref(mc), ws.data_ptr(), ws_bytes, n_faces, stream))
        K = int(n_faces[0]) + int(n_faces[1])
        width = 4 if quad else 3
        i32 = dict(dtype=torch.int32, device=dev)
        f64 = dict(dtype=torch.float64, device=dev)
        out = dict(cell_faces=torch.empty((C, F), **i32), unique_faces=torch.empty((K, width), **i32),
                   face_nodes=torch.empty(K, **i32), face_cells=torch.empty((K, 2), **i32),
                   face_slots=torch.empty((K, 2), **i32), centroid=torch.empty((C, 3), **f64),
                   volume=torch.empty(C, **f64), area=torch.empty((C, F), **f64),
                   normal=torch.empty((C, F, 3), **f64), to_face=torch.empty((C, F, 3), **f64),
                   face_centroid=torch.empty((K, 3), **f64))
        mf = _lib.MeshFaces_t(*(out[k].data_ptr() for k in (
            "cell_faces", "unique_faces", "face_nodes", "face_cells", "face_slots", "centroid", "volume", "area",
            "normal", "to_face", "face_centroid")), width, 0)
        check(lib.wcfd_mesh_emit(ct.byref(mc), ws.data_ptr(), ws_bytes, n_faces, ct.byref(mf), stream))
        host = {k: v.cpu().numpy() for k, v in out.items()}
    del ws
    fc, fs = host["face_cells"].astype(np.int64), host["face_slots"].astype(np.int64)
    return dict(unique_faces=host["unique_faces"], cell_face_ids=host["cell_faces"], area=host["area"],
                normal=host["normal"], nodes_per_face=host["face_nodes"], face_centroid=host["face_centroid"],
                to_face=host["to_face"], own_cell=fc[:, 0], own_slot=fs[:, 0], nb_cell=fc[:, 1],
                nb_slot=fs[:, 1], volume=host["volume"], centroid=host["centroid"])
