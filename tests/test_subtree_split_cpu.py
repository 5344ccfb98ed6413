"""Subtree split, host side, on CPU ranks (gloo, world size 2): the partition of a mesh into its
level-k subtrees and the exchange between processes, without a GPU.

Each rank extracts the subtrees it owns (round-robin over the 4^k level-k nodes), sends their leaf
quadrants and patch boxes to rank 0 over gloo with the same point-to-point transport the solver
uses, and rank 0 checks that, put back in z-order and shifted to the full tree's coordinates, they
are the full mesh's leaves with bit-identical patch boxes, and that every subtree's leaves are a
contiguous range of the full leaf order."""
import os
import socket

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _mesh(kind):
    import ellipticforest_gb300 as ef
    if kind == "uniform":
        root = ef.FiniteVolumePatch(ef.FiniteVolumeGrid(8, -1.0, 1.0, 8, -1.0, 1.0))
        return ef.Mesh().uniform(4, root)
    root = ef.FiniteVolumePatch(ef.FiniteVolumeGrid(16, -10.0, 10.0, 16, -10.0, 10.0))
    return ef.Mesh().refineByFunction(lambda x, y: abs(np.sin(x) + np.sin(y)) > 1.2, 0.0, 2, 6, root)


def _rank_main(rank, world, port, kind, level, out):
    import sys
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist
    from ellipticforest_gb300 import _lib
    from ellipticforest_gb300.subtree import _Transport, subtree_leaf_ranges, subtree_owners
    _lib.load()
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mesh = _mesh(kind)
        tr = _Transport()
        count = mesh.level_count(level)
        owners = subtree_owners(count, world)
        mine = {}
        for p in range(count):
            if owners[p] == rank:
                sub = mesh.subtree(level, p)
                rows = []
                for k in range(sub.num_leaves()):
                    lvl, ix, iy, box = sub.leaf(k)
                    rows.append([lvl, ix, iy, *box])
                mine[p] = np.array(rows, dtype=np.float64)
        # leaf counts first (so rank 0 knows the sizes), then the leaf tables
        counts = [0] * count
        for p, a in mine.items():
            counts[p] = a.shape[0]
        import torch
        t = torch.tensor(counts, dtype=torch.float64)
        dist.all_reduce(t)
        allc = [int(v) for v in t.tolist()]
        if rank != 0:
            for p, a in sorted(mine.items()):
                tr.send(a.ravel(), 0, p)
            ok = True
        else:
            tables = [mine[p] if owners[p] == 0 else tr.recv(allc[p] * 7, owners[p], p).reshape(-1, 7)
                      for p in range(count)]
            full = np.array([[*mesh.leaf(k)[:3], *mesh.leaf(k)[3]] for k in range(mesh.num_leaves())])
            # subtree quadrants back to the full tree's coordinates
            got = []
            ranges = subtree_leaf_ranges(mesh, level)
            for p, tab in enumerate(tables):
                b, e = ranges[p]
                ref = full[b:e]
                d = tab[:, 0]
                lvl_full = ref[:, 0]
                assert np.array_equal(d + level, lvl_full)
                sh = (lvl_full - level).astype(np.int64)
                px = (ref[:, 1].astype(np.int64) >> sh)
                py = (ref[:, 2].astype(np.int64) >> sh)
                assert len(set(px)) == 1 and len(set(py)) == 1
                assert np.array_equal(tab[:, 1].astype(np.int64) + (px << sh), ref[:, 1].astype(np.int64))
                assert np.array_equal(tab[:, 2].astype(np.int64) + (py << sh), ref[:, 2].astype(np.int64))
                assert np.array_equal(tab[:, 3:], ref[:, 3:])  # patch boxes bit for bit
                got.append(tab)
            assert sum(t.shape[0] for t in got) == mesh.num_leaves()
            ok = True
        flag = torch.tensor([1.0 if ok else 0.0])
        dist.all_reduce(flag, op=dist.ReduceOp.MIN)
        out.put((rank, bool(flag.item() == 1.0)))
    except Exception as e:  # reported to the parent
        out.put((rank, repr(e)))
        raise
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("kind,level", [("uniform", 2), ("adaptive", 1)])
def test_subtree_partition_and_exchange_on_two_gloo_ranks(lib, kind, level):
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, kind, level, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=300) for _ in procs]
    for p in procs:
        p.join(timeout=60)
    assert all(r[1] is True for r in res), res
    assert all(p.exitcode == 0 for p in procs)


def test_subtree_split_rejects_a_level_with_leaves_above_it(lib):
    from ellipticforest_gb300.subtree import subtree_leaf_ranges
    import ellipticforest_gb300 as ef
    root = ef.FiniteVolumePatch(ef.FiniteVolumeGrid(8, 0.0, 1.0, 8, 0.0, 1.0))
    mesh = ef.Mesh().refineByFunction(lambda x, y: x > 0.7 and y > 0.7, 0.0, 1, 4, root)
    with pytest.raises(ValueError):
        subtree_leaf_ranges(mesh, 3)  # leaves at level 2 lie above it
