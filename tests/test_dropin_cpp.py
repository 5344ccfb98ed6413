"""The C++ drop-in (include/EllipticForest.hpp): a driver written against the reference's API
compiles against the headers and the shared library, and on the GPU reproduces the oracle's leaf
solutions to 1e-12 relative on config 1 (uniform level 3) and on an adaptive mesh."""
import json
import os
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from oracle import hps_oracle as O

ROOT = Path(__file__).resolve().parents[1]
SRC = ROOT / "tests" / "cpp" / "elliptic_single.cpp"
LIBDIR = ROOT / "ellipticforest_gb300"


@pytest.fixture(scope="module")
def driver(lib, tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    exe = tmp_path_factory.mktemp("dropin") / "elliptic_single"
    cmd = [cxx, "-std=c++17", "-O2", "-Wall", "-Wextra", "-Wno-unused-parameter", "-I", str(ROOT / "include"),
           str(SRC), "-o", str(exe), "-L", str(LIBDIR), "-lellipticforest_gb300", f"-Wl,-rpath,{LIBDIR}"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    assert "warning" not in res.stderr, res.stderr
    return exe


def test_dropin_driver_compiles(driver):
    assert os.access(driver, os.X_OK)


def _oracle(n, lo, hi, min_level, max_level):
    f = lambda x, y: -(np.sin(x) + np.sin(y))
    root = O.FiniteVolumePatch(O.FiniteVolumeGrid(n, lo, hi, n, lo, hi))
    mesh = O.Mesh().refineByFunction(lambda x, y: abs(f(x, y)) > 1.2, 1.2, min_level, max_level, root)
    hps = O.HPSAlgorithm(mesh, O.FiniteVolumeSolver(solver_type=O.FISHPACK90))
    hps.buildStage()
    hps.upwardsStage(f)
    hps.solveStage(lambda s, x, y: (np.sin(x) + np.sin(y), 1.0, 0.0))
    return O.leaf_solution(hps)


@pytest.mark.gpu
@pytest.mark.parametrize("n,lo,hi,min_level,max_level", [(16, -10.0, 10.0, 3, 3), (8, -10.0, 10.0, 0, 4)])
def test_dropin_driver_matches_oracle(driver, tmp_path, n, lo, hi, min_level, max_level):
    out = tmp_path / "u.bin"
    res = subprocess.run([str(driver), f"--nx={n}", f"--x-lower={lo}", f"--x-upper={hi}",
                          f"--min-level={min_level}", f"--max-level={max_level}", f"--out={out}"],
                         capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stderr
    info = json.loads(res.stdout.strip().splitlines()[-1])
    u = np.fromfile(out, dtype=np.float64)
    uo = _oracle(n, lo, hi, min_level, max_level)
    assert u.size == uo.size == info["dofs"]
    assert np.abs(u - uo).max() <= 1e-12 * np.abs(uo).max()
    # Mesh::toVTK: one quad per leaf cell with the solution as cell data, one quad per leaf patch
    import xml.etree.ElementTree as ET
    piece = ET.parse(f"{out}-vtk-mesh-0.vtu").getroot().find("UnstructuredGrid/Piece")
    assert int(piece.get("NumberOfCells")) == u.size
    arrays = {a.get("Name"): a for a in piece.iter("DataArray")}
    uv = np.array(arrays["u"].text.split(), dtype=np.float64)
    assert np.array_equal(uv, u)
    assert "u_exact" in arrays and arrays["types"].text.split()[0] == "9"
    assert ET.parse(f"{out}-vtk-mesh.pvtu").getroot().find("PUnstructuredGrid/Piece").get("Source").endswith("-0.vtu")
    quad = ET.parse(f"{out}-vtk-quadtree.vtu").getroot().find("UnstructuredGrid/Piece")
    assert int(quad.get("NumberOfCells")) == info["leaves"]


def test_overriding_a_per_node_hook_does_not_compile(tmp_path):
    """The reference's per-node hooks (merge4to1, upwards4to1, split1to4, leafSolve) are virtual
    customisation points; the drop-in runs whole tree levels as grouped kernels, so an override would
    never be called.  They are final: a subclass that overrides one is a compile error, not a
    silently ignored method."""
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    src = ROOT / "tests" / "cpp" / "override_hook.cpp"
    res = subprocess.run([cxx, "-std=c++17", "-fsyntax-only", "-I", str(ROOT / "include"), str(src)],
                         capture_output=True, text=True)
    assert res.returncode != 0
    assert "final" in res.stderr, res.stderr
    # the same driver without the override compiles
    ok = src.read_text().replace(" override {}", " {}").replace("void merge4to1", "void myMerge")
    tmp = tmp_path / "no_override.cpp"
    tmp.write_text(ok)
    res = subprocess.run([cxx, "-std=c++17", "-fsyntax-only", "-I", str(ROOT / "include"), str(tmp)],
                         capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
