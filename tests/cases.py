"""Seeded case builders shared by the tests (small versions of the benchmark cases)."""
import numpy as np

from warpcfd_gb300.FV.boundary import Boundary
from warpcfd_gb300.FV.field import Field
from warpcfd_gb300.preprocess import Mesh, create_2D_grid, create_3D_grid, define_boundary_walls

FIELDS = {k: Field(k, i) for i, k in enumerate("uvwp")}


def cavity_mesh(n=16, jitter=0.0, seed=0):
    m = Mesh(create_2D_grid((0, 0, 0), n, n, 1.0, 1.0, 0.1, jitter=jitter, seed=seed))
    define_boundary_walls(m)
    return m


def cavity_bc(b, lid=1.0):
    """examples/LDC/LDC.py:38-45 (lid on +Y)."""
    b.no_slip_wall("-X")
    b.no_slip_wall("+X")
    b.no_slip_wall("-Y")
    b.velocity_BC("+Y", u=lid, v=0, w=0)
    b.slip_wall("+Z")
    b.slip_wall("-Z")


def channel_mesh(nx=40, ny=8, lx=10.0, ly=1.0, jitter=0.0, seed=0):
    m = Mesh(create_2D_grid((0, 0, 0), nx, ny, lx, ly, 0.1, jitter=jitter, seed=seed))
    define_boundary_walls(m)
    return m


def channel_bc(b, u_in=1.0):
    b.velocity_BC("-X", u=u_in, v=0, w=0)
    b.pressure_BC("+X", p=0.0)
    b.no_slip_wall("-Y")
    b.no_slip_wall("+Y")
    b.slip_wall("-Z")
    b.slip_wall("+Z")


def cavity3d_mesh(n=6, jitter=0.0, seed=0):
    m = Mesh(create_3D_grid((0, 0, 0), n, n, n, 1.0, 1.0, 1.0, jitter=jitter, seed=seed))
    define_boundary_walls(m)
    return m


def cavity3d_bc(b, lid=1.0):
    for w in ("-X", "+X", "-Y", "-Z", "+Z"):
        b.no_slip_wall(w)
    b.velocity_BC("+Y", u=lid, v=0, w=0)


def prism_cavity_mesh(n=16, element_type="mixed", jitter=0.0, seed=0):
    """The 2D cavity with prisms: 'wedge' cuts every quad, 'mixed' the right half."""
    m = Mesh(create_2D_grid((0, 0, 0), n, n, 1.0, 1.0, 0.1, element_type=element_type, jitter=jitter, seed=seed))
    define_boundary_walls(m)
    return m


def prism_channel_mesh(nx=40, ny=8, lx=10.0, ly=1.0, element_type="wedge"):
    m = Mesh(create_2D_grid((0, 0, 0), nx, ny, lx, ly, 0.1, element_type=element_type))
    define_boundary_walls(m)
    return m


def mixed_cavity3d_mesh(n=6, prism_fraction=0.5, seed=0):
    """The 3D cavity with a seeded fraction of its hexes cut into two prisms each."""
    m = Mesh(create_3D_grid((0, 0, 0), n, n, n, 1.0, 1.0, 1.0, prism_fraction=prism_fraction, seed=seed))
    define_boundary_walls(m)
    return m


def tet_cavity3d_mesh(n=4, jitter=0.0, seed=0):
    """The 3D cavity with every hex cut into six tetrahedra."""
    m = Mesh(create_3D_grid((0, 0, 0), n, n, n, 1.0, 1.0, 1.0, element_type="tetra", jitter=jitter, seed=seed))
    define_boundary_walls(m)
    return m


def host_boundary(m, bc_fn, **kw):
    b = Boundary(FIELDS, m.groups, m.face_properties.boundary_face_ids)
    bc_fn(b, **kw)
    b.check()
    return b
