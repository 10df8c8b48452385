"""Structured Q1 hexahedral meshes with the numbering the reference's grids produce.

The reference builds its cantilevers on ``Dune::YaspGrid<3>`` (tests/src/testcantileverbeam.hh:42-53):
vertices are numbered lexicographically with x fastest, elements likewise, and the eight
corners of an element follow the Dune reference-cube order (vertex ``v`` sits at
``(v & 1, v >> 1 & 1, v >> 2 & 1)``).  The flat dof index of component ``c`` of vertex ``n``
is ``3 * n + c`` (FlatInterleaved, ikarus/utils/flatprebasis.hh:57-76).  Faces of a hexahedron
use the Dune numbering: face ``2 d`` lies on ``xi_d = 0`` and face ``2 d + 1`` on ``xi_d = 1``.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass
class HexMesh:
    coords: np.ndarray  # (n_nodes, 3) float64
    conn: np.ndarray  # (n_elems, 8) int32, Dune corner order
    shape: tuple = ()  # (nx, ny, nz) for structured meshes
    lengths: tuple = ()
    origin: tuple = (0.0, 0.0, 0.0)
    meta: dict = field(default_factory=dict)

    @property
    def n_nodes(self) -> int:
        return int(self.coords.shape[0])

    @property
    def n_elems(self) -> int:
        return int(self.conn.shape[0])

    @property
    def n_dofs(self) -> int:
        return 3 * self.n_nodes


def structured_hex_grid(nx: int, ny: int, nz: int, lengths=(1.0, 1.0, 1.0), origin=(0.0, 0.0, 0.0)) -> HexMesh:
    """Box ``origin + [0,Lx]x[0,Ly]x[0,Lz]`` meshed with ``nx*ny*nz`` Q1 hexahedra (YaspGrid numbering)."""
    lx, ly, lz = (float(v) for v in lengths)
    xs = origin[0] + lx * np.arange(nx + 1) / nx
    ys = origin[1] + ly * np.arange(ny + 1) / ny
    zs = origin[2] + lz * np.arange(nz + 1) / nz
    Z, Y, X = np.meshgrid(zs, ys, xs, indexing="ij")
    coords = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1).astype(np.float64)
    ex, ey, ez = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    ex, ey, ez = ex.transpose(2, 1, 0).ravel(), ey.transpose(2, 1, 0).ravel(), ez.transpose(2, 1, 0).ravel()
    conn = np.empty((nx * ny * nz, 8), dtype=np.int32)
    for v in range(8):
        i = ex + (v & 1)
        j = ey + ((v >> 1) & 1)
        k = ez + ((v >> 2) & 1)
        conn[:, v] = i + (nx + 1) * (j + (ny + 1) * k)
    return HexMesh(coords, conn, (nx, ny, nz), (lx, ly, lz), tuple(float(o) for o in origin))


def jitter_interior(mesh: HexMesh, fraction: float, seed: int) -> HexMesh:
    """Move every interior vertex by ``U(-fraction*h_d, fraction*h_d)`` per axis; boundary vertices stay put."""
    nx, ny, nz = mesh.shape
    h = np.array(mesh.lengths) / np.array([nx, ny, nz])
    rng = np.random.default_rng(seed)
    idx = np.arange(mesh.n_nodes)
    i = idx % (nx + 1)
    j = (idx // (nx + 1)) % (ny + 1)
    k = idx // ((nx + 1) * (ny + 1))
    interior = (i > 0) & (i < nx) & (j > 0) & (j < ny) & (k > 0) & (k < nz)
    d = rng.uniform(-1.0, 1.0, size=(mesh.n_nodes, 3)) * (fraction * h)
    coords = mesh.coords.copy()
    coords[interior] += d[interior]
    return HexMesh(coords, mesh.conn.copy(), mesh.shape, mesh.lengths, mesh.origin, dict(mesh.meta, jitter=(fraction, seed)))


def boundary_faces(mesh: HexMesh, side: str):
    """Element faces on one side of a structured box: side in {'x-','x+','y-','y+','z-','z+'}.

    Returns ``(face_elem, face_local)`` int32 arrays, element order ascending.
    """
    nx, ny, nz = mesh.shape
    axis = "xyz".index(side[0])
    upper = side[1] == "+"
    e = np.arange(mesh.n_elems)
    ijk = (e % nx, (e // nx) % ny, e // (nx * ny))
    n = (nx, ny, nz)[axis]
    sel = ijk[axis] == (n - 1 if upper else 0)
    fe = e[sel].astype(np.int32)
    fl = np.full(fe.shape, 2 * axis + (1 if upper else 0), dtype=np.int32)
    return fe, fl


def face_centers(mesh: HexMesh, face_elem, face_local) -> np.ndarray:
    """Centre (mean of the four corners, = the bilinear face map at (1/2,1/2)) of each face."""
    out = np.empty((len(face_elem), 3))
    for k, (e, f) in enumerate(zip(face_elem, face_local)):
        d, s = divmod(int(f), 2)
        corners = [v for v in range(8) if ((v >> d) & 1) == s]
        out[k] = mesh.coords[mesh.conn[e, corners]].mean(axis=0)
    return out


def fixed_dofs_where(mesh: HexMesh, predicate, components=(0, 1, 2)) -> np.ndarray:
    """uint8 mask over the flat dofs: 1 for the listed components of every vertex where predicate(coords) holds."""
    sel = np.asarray(predicate(mesh.coords), dtype=bool)
    mask = np.zeros(mesh.n_dofs, dtype=np.uint8)
    for c in components:
        mask[3 * np.nonzero(sel)[0] + c] = 1
    return mask


def vertex_at(mesh: HexMesh, point, tol=1e-9) -> int:
    d = np.linalg.norm(mesh.coords - np.asarray(point, dtype=float), axis=1)
    i = int(np.argmin(d))
    if d[i] > tol:
        raise ValueError(f"no vertex at {point}")
    return i
