"""Result export as a VTK XML unstructured grid (.vtu), the format the reference's writer produces through
Dune's VTKWriter (ikarus/io/vtkwriter.hh): points, hexahedral cells, point data (e.g. the displacement) and cell
data (e.g. a stress from calculateAt).  ASCII, no dependencies."""
from __future__ import annotations

import numpy as np

# Dune's reference-cube vertex v sits at (v&1, v>>1&1, v>>2&1); VTK_HEXAHEDRON lists the bottom face
# counter-clockwise, then the top face
DUNE_TO_VTK_HEX = (0, 1, 3, 2, 4, 5, 7, 6)
VTK_HEXAHEDRON = 12


def _data_array(name, values):
    a = np.asarray(values, dtype=np.float64)
    comps = 1 if a.ndim == 1 else a.shape[1]
    body = " ".join(f"{v:.17g}" for v in a.ravel())
    return (f'<DataArray type="Float64" Name="{name}" NumberOfComponents="{comps}" format="ascii">'
            f"{body}</DataArray>")


def write_vtu(path, coords, conn, point_data=None, cell_data=None):
    """coords (n_nodes x 3), conn (n_elems x 8, Dune vertex order); point_data / cell_data: name -> array with
    one row per node / element (1 or more components, e.g. the displacement reshaped to n_nodes x 3 or the 6 Voigt
    stress values)."""
    X = np.asarray(coords, dtype=np.float64).reshape(-1, 3)
    E = np.asarray(conn, dtype=np.int64).reshape(-1, 8)[:, DUNE_TO_VTK_HEX]
    nn, ne = len(X), len(E)
    parts = ['<?xml version="1.0"?>',
             '<VTKFile type="UnstructuredGrid" version="0.1" byte_order="LittleEndian">',
             "<UnstructuredGrid>", f'<Piece NumberOfPoints="{nn}" NumberOfCells="{ne}">', "<Points>",
             _data_array("Coordinates", X), "</Points>", "<Cells>",
             '<DataArray type="Int64" Name="connectivity" format="ascii">' + " ".join(map(str, E.ravel())) +
             "</DataArray>",
             '<DataArray type="Int64" Name="offsets" format="ascii">' +
             " ".join(str(8 * (k + 1)) for k in range(ne)) + "</DataArray>",
             '<DataArray type="UInt8" Name="types" format="ascii">' + " ".join([str(VTK_HEXAHEDRON)] * ne) +
             "</DataArray>", "</Cells>"]
    for tag, data, count in (("PointData", point_data, nn), ("CellData", cell_data, ne)):
        parts.append(f"<{tag}>")
        for name, arr in (data or {}).items():
            a = np.asarray(arr, dtype=np.float64)
            if a.shape[0] != count:
                raise ValueError(f"{tag} '{name}' has {a.shape[0]} rows, expected {count}")
            parts.append(_data_array(name, a))
        parts.append(f"</{tag}>")
    parts += ["</Piece>", "</UnstructuredGrid>", "</VTKFile>"]
    with open(path, "w") as f:
        f.write("\n".join(parts) + "\n")
