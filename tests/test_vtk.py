"""The .vtu result export: cell connectivity in VTK's hexahedron order, point and cell data round trip."""
import xml.etree.ElementTree as ET

import numpy as np

from ikarus_gb300 import problems
from ikarus_gb300.vtk import DUNE_TO_VTK_HEX, write_vtu


def test_vtu_round_trip(tmp_path):
    p = problems.cantilever(3, 2, 1)
    u = np.arange(p.n_dofs, dtype=float).reshape(-1, 3)
    s = np.arange(6 * p.mesh.n_elems, dtype=float).reshape(-1, 6)
    path = tmp_path / "r.vtu"
    write_vtu(path, p.mesh.coords, p.mesh.conn, {"displacement": u}, {"cauchyStress": s})
    root = ET.parse(path).getroot()
    piece = root.find("UnstructuredGrid/Piece")
    assert int(piece.get("NumberOfPoints")) == p.mesh.n_nodes and int(piece.get("NumberOfCells")) == p.mesh.n_elems
    arrays = {a.get("Name"): a for a in root.iter("DataArray")}
    conn = np.array(arrays["connectivity"].text.split(), dtype=int).reshape(-1, 8)
    assert np.array_equal(conn, np.asarray(p.mesh.conn).reshape(-1, 8)[:, DUNE_TO_VTK_HEX])
    # VTK's first hexahedron face is the bottom quad in cyclic order: corners 0,1,2,3 go around the face
    X = np.asarray(p.mesh.coords)
    q = X[conn[0, :4]]
    assert np.allclose(q[:, 2], q[0, 2]) and np.linalg.norm(q[2] - q[0]) > np.linalg.norm(q[1] - q[0])
    assert np.array_equal(np.array(arrays["displacement"].text.split(), dtype=float), u.ravel())
    assert np.array_equal(np.array(arrays["cauchyStress"].text.split(), dtype=float), s.ravel())
