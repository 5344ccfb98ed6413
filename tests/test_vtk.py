"""Mesh.toVTK (Mesh.hpp:357-424): the VTK XML files of a refined mesh parse, hold one quad per leaf
cell with the added mesh functions as cell data, and one quad per leaf patch in the quadtree file.
Host-only (the mesh is built by the library's host code; no GPU needed)."""
import xml.etree.ElementTree as ET

import numpy as np


def test_mesh_to_vtk(lib, tmp_path):
    import ellipticforest_gb300 as ef
    root = ef.FiniteVolumePatch(ef.FiniteVolumeGrid(4, 0.0, 1.0, 4, 0.0, 1.0))
    mesh = ef.Mesh().refineByFunction(lambda x, y: x + y > 1.4, 0.0, 1, 3, root)
    X, Y = mesh.cell_centres()
    mesh.addMeshFunction(np.sin(X) * Y, "u")
    mesh.addMeshFunction(lambda x, y: x - y, "x_minus_y")
    base = str(tmp_path / "out")
    mesh.toVTK(base, number=7)
    piece = ET.parse(base + "-mesh-0007-0.vtu").getroot().find("UnstructuredGrid/Piece")
    assert int(piece.get("NumberOfCells")) == X.size
    arrays = {a.get("Name"): np.array(a.text.split(), dtype=np.float64) for a in piece.iter("DataArray")}
    assert np.array_equal(arrays["u"], np.sin(X) * Y)
    assert np.array_equal(arrays["x_minus_y"], X - Y)
    pts = arrays["Points"].reshape(-1, 3)
    # each cell's quad surrounds its cell centre
    quad = pts.reshape(-1, 4, 3)
    assert np.allclose(quad[:, :, 0].mean(axis=1), X) and np.allclose(quad[:, :, 1].mean(axis=1), Y)
    pv = ET.parse(base + "-mesh-0007.pvtu").getroot()
    assert pv.find("PUnstructuredGrid/Piece").get("Source") == "out-mesh-0007-0.vtu"
    q = ET.parse(base + "-quadtree-0007.vtu").getroot().find("UnstructuredGrid/Piece")
    assert int(q.get("NumberOfCells")) == mesh.num_leaves()
    lv = [a for a in q.iter("DataArray") if a.get("Name") == "level"][0]
    levels = np.array(lv.text.split(), dtype=float).astype(int)
    assert levels.min() >= 1 and levels.max() == 3
    assert np.array_equal(levels, [mesh.leaf(k)[0] for k in range(mesh.num_leaves())])
