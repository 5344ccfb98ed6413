"""C-ABI checks that need no GPU: the library loads, exports every symbol of
include/ellipticforest_gb300.h, rejects bad arguments with status codes, and its host-side quadtree
(Mesh::refineByFunction restated without p4est) matches the oracle's leaf for leaf."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from oracle import hps_oracle as O

HEADER = Path(__file__).resolve().parents[1] / "include" / "ellipticforest_gb300.h"


def header_functions():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\*?\s+\*?(ef_\w+)\s*\(", text, re.M)))


def test_header_declares_the_abi():
    names = header_functions()
    assert "ef_hps_build" in names and "ef_mesh_create_refined" in names
    assert len(names) >= 25


def test_library_exports_every_declared_symbol(lib):
    from ellipticforest_gb300 import _lib
    for name in header_functions():
        assert hasattr(lib, name), name
        assert name in _lib.SIGNATURES, f"{name} missing from the ctypes table"


def test_bad_arguments_return_status_codes(lib):
    from ellipticforest_gb300 import _lib
    h = C.c_void_p()
    assert lib.ef_mesh_create_uniform(1.0, 0.0, 0.0, 1.0, 8, 8, 2, C.byref(h)) == _lib.EF_ERR_INVALID
    assert b"domain" in lib.ef_last_error()
    assert lib.ef_mesh_create_uniform(0.0, 1.0, 0.0, 1.0, 0, 8, 2, C.byref(h)) == _lib.EF_ERR_INVALID
    assert lib.ef_mesh_num_leaves(None, None) == _lib.EF_ERR_INVALID
    assert lib.ef_hps_build(None) == _lib.EF_ERR_INVALID
    assert lib.ef_hps_set_option(None, b"cache-operators", 1) == _lib.EF_ERR_INVALID


def test_uniform_mesh(lib):
    import ellipticforest_gb300 as ef
    root = ef.FiniteVolumePatch(ef.FiniteVolumeGrid(8, -1, 1, 8, -1, 1))
    m = ef.Mesh().uniform(3, root)
    assert m.num_leaves() == 64 and m.num_nodes() == 1 + 4 + 16 + 64
    orot = O.FiniteVolumePatch(O.FiniteVolumeGrid(8, -1, 1, 8, -1, 1))
    om = O.Mesh().uniform(3, orot)
    for k, node in enumerate(om.quadtree.leaves()):
        lvl, ix, iy, box = m.leaf(k)
        assert O.leaf_path(lvl, ix, iy) == node.path
        g = node.data.grid()
        assert list(box) == [g.xLower(), g.xUpper(), g.yLower(), g.yUpper()]


@pytest.mark.parametrize("case", ["config2", "spot", "minlevel"])
def test_refine_by_function_matches_oracle(lib, case):
    import ellipticforest_gb300 as ef
    if case == "config2":
        fn, dom, n, lo, hi = (lambda x, y: abs(np.sin(x) + np.sin(y)) > 1.2), (-10, 10, -10, 10), 16, 0, 7
    elif case == "spot":
        fn, dom, n, lo, hi = (lambda x, y: (x - 0.3) ** 2 + (y + 0.2) ** 2 < 0.01), (0, 1, -1, 0), 4, 0, 8
    else:
        fn, dom, n, lo, hi = (lambda x, y: x * y > 0.5), (-1, 1, -1, 1), 8, 2, 6
    root = ef.FiniteVolumePatch(ef.FiniteVolumeGrid(n, dom[0], dom[1], n, dom[2], dom[3]))
    m = ef.Mesh().refineByFunction(fn, 0.0, lo, hi, root)
    orot = O.FiniteVolumePatch(O.FiniteVolumeGrid(n, *dom[:2], n, *dom[2:]))
    om = O.Mesh().refineByFunction(fn, 0.0, lo, hi, orot)
    ol = om.quadtree.leaves()
    assert m.num_leaves() == len(ol)
    assert m.num_nodes() == len(om.quadtree.map)
    for k, node in enumerate(ol):
        lvl, ix, iy, box = m.leaf(k)
        assert O.leaf_path(lvl, ix, iy) == node.path
        g = node.data.grid()
        assert list(box) == [g.xLower(), g.xUpper(), g.yLower(), g.yUpper()]
