"""Subtree split on the GPU: four gloo processes (one level-1 subtree each, all on this one GPU --
their kernels never wait on one another; T, h and g move between them through host memory) build
and solve one tree; rank 0 merges the top level.  The leaf solutions must equal a single-handle build
and solve bit for bit, on a uniform and an adaptive mesh, with Dirichlet and Robin root data."""
import os
import socket

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _problem(kind):
    import ellipticforest_gb300 as ef
    if kind == "uniform":
        root = ef.FiniteVolumePatch(ef.FiniteVolumeGrid(8, -1.0, 1.0, 8, -1.0, 1.0))
        mesh = ef.Mesh().uniform(4, root)
    else:
        root = ef.FiniteVolumePatch(ef.FiniteVolumeGrid(16, -10.0, 10.0, 16, -10.0, 10.0))
        mesh = ef.Mesh().refineByFunction(lambda x, y: abs(np.sin(x) + np.sin(y)) > 1.2, 0.0, 2, 6, root)
    solver = ef.FiniteVolumeSolver(solver_type=ef.FISHPACK90)
    f = lambda x, y: np.sin(1.3 * x + 0.2) * np.cos(0.7 * y) + 0.1 * x * y
    return mesh, solver, f


def _bc(robin):
    if robin:
        return lambda side, x, y: (np.cos(x - 2 * y), 1.0, 0.25)
    return lambda side, x, y: (np.sin(x) + np.cos(0.5 * y), 1.0, 0.0)


def _rank_main(rank, world, port, kind, robin, path):
    import sys
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch
    import torch.distributed as dist
    torch.cuda.set_device(0)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from ellipticforest_gb300.subtree import SubtreeSplit
        mesh, solver, f = _problem(kind)
        sp = SubtreeSplit(mesh, solver, 1)
        sp.buildStage()
        sp.upwardsStage(f)
        sp.solveStage(_bc(robin))
        u = sp.leaf_solution()
        if rank == 0:
            np.save(path, u)
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("kind,robin", [("uniform", False), ("adaptive", False), ("adaptive", True)])
def test_subtree_split_equals_single_handle_bit_for_bit(lib, tmp_path, kind, robin):
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    path = str(tmp_path / "u.npy")
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 4, port, kind, robin, path)) for r in range(4)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=600)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    u_split = np.load(path)

    import ellipticforest_gb300 as ef
    mesh, solver, f = _problem(kind)
    hps = ef.HPSAlgorithm(mesh, solver)
    hps.buildStage()
    hps.upwardsStage(f)
    hps.solveStage(_bc(robin))
    u = hps.leaf_solution()
    assert u_split.shape == u.shape
    assert np.array_equal(u_split, u)


def test_top_handle_refuses_the_single_handle_stages(lib):
    import ellipticforest_gb300 as ef
    from ellipticforest_gb300 import _lib
    mesh, solver, f = _problem("uniform")
    subs = [ef.HPSAlgorithm(mesh.subtree(1, p), solver) for p in range(4)]
    Ts = []
    for h in subs:
        h.buildStage()
        Ts.append(h.root_T())
    top = ef.HPSAlgorithm(mesh, solver)
    assert top.split_sizes(1) == [T.shape[0] for T in Ts]
    top.buildStageTop(1, Ts)
    X, Y = mesh.cell_centres()
    fv = np.ascontiguousarray(f(X, Y))
    assert _lib.load().ef_hps_upwards(top.handle, _lib.dptr(fv)) == _lib.EF_ERR_STATE
    with pytest.raises(RuntimeError):
        top.buildStageTop(4, Ts)  # leaves lie at level 4: no split there
