"""One tree split across processes by subtrees (one process per GPU).

The reference runs one tree over MPI ranks with p4est's partition and, at the process boundary,
broadcasts whole child patches inside ``merge4to1`` (src/Quadtree.hpp:470-496, the patch broadcast
at :146-148) and sends them back down in ``split1to4``.  Here the tree splits at a level k: its
4^k level-k nodes are the roots of independent subtrees, dealt round-robin to the processes.
Each process builds, upward-passes and solves its subtrees as trees of their own (the kernels see
exactly the operands of a single-handle run), and rank 0 runs the top k levels on a handle of the
full mesh:

    build : every subtree's root T (4m x 4m)     --gather-->  rank 0 merges levels k-1 .. 0
    upward: every subtree's root h (4m)          --gather-->  rank 0 upward pass of levels k-1 .. 0
    solve : rank 0 root data + downward pass to k --scatter--> g (4m) of every subtree, which its
            owner solves with as Dirichlet root data

The exchange is point-to-point ``torch.distributed`` send/recv of float64 tensors: host tensors on
``gloo``, device tensors on ``nccl``.  There is no other collective on the data path.  The leaf
solutions equal a single-handle build and solve bit for bit.
"""
from __future__ import annotations

from typing import Callable, Dict, List, Optional, Tuple

import numpy as np

from . import _lib
from ._lib import check, dptr
from .hps import FiniteVolumeSolver, HPSAlgorithm, Mesh


def subtree_owners(count: int, world: int) -> List[int]:
    """Owner rank of each of the `count` level-k subtrees (z-order): dealt round-robin."""
    return [p % world for p in range(count)]


def subtree_leaf_ranges(mesh: Mesh, level: int) -> List[Tuple[int, int]]:
    """[begin, end) of each level-k subtree's leaves in the full mesh's leaf (pre-)order: a subtree's
    leaves are contiguous there and the subtrees follow each other in z-order."""
    out, k = [], 0
    for p in range(mesh.level_count(level)):
        cnt = mesh.subtree(level, p).num_leaves()
        out.append((k, k + cnt))
        k += cnt
    if k != mesh.num_leaves():
        raise ValueError(f"subtree split: level {level} does not partition the leaves (a leaf lies at or above it)")
    return out


class _Transport:
    """float64 arrays between ranks by point-to-point send/recv (host tensors on gloo, device
    tensors on nccl)."""

    def __init__(self, group=None):
        import torch
        import torch.distributed as dist
        self.torch, self.dist, self.group = torch, dist, group
        self.device = "cuda" if dist.get_backend(group) == "nccl" else "cpu"

    def send(self, arr: np.ndarray, dst: int, tag: int):
        t = self.torch.from_numpy(np.ascontiguousarray(arr, dtype=np.float64)).to(self.device)
        self.dist.send(t, dst, group=self.group, tag=tag)

    def recv(self, size: int, src: int, tag: int) -> np.ndarray:
        t = self.torch.empty(size, dtype=self.torch.float64, device=self.device)
        self.dist.recv(t, src, group=self.group, tag=tag)
        return t.cpu().numpy()

    def bcast_ints(self, values: Optional[List[int]], count: int, src: int = 0) -> List[int]:
        t = self.torch.zeros(count, dtype=self.torch.int64, device=self.device)
        if values is not None:
            t.copy_(self.torch.tensor(values, dtype=self.torch.int64))
        self.dist.broadcast(t, src, group=self.group)
        return [int(v) for v in t.cpu().tolist()]


class SubtreeSplit:
    """HPSAlgorithm over several processes: each builds and solves the level-k subtrees it owns;
    rank 0 also runs the top k levels.  Stages mirror HPSAlgorithm's (buildStage, upwardsStage,
    solveStage); call them on every rank in the same order."""

    def __init__(self, mesh: Mesh, patch_solver: FiniteVolumeSolver, level: int, group=None,
                 options: Optional[dict] = None):
        import torch.distributed as dist
        self.mesh, self.level = mesh, int(level)
        self.rank, self.world = dist.get_rank(group), dist.get_world_size(group)
        self.tr = _Transport(group)
        self.count = mesh.level_count(self.level)
        self.owner = subtree_owners(self.count, self.world)
        self.ranges = subtree_leaf_ranges(mesh, self.level)
        self.local: Dict[int, Tuple[Mesh, HPSAlgorithm]] = {}
        for p in range(self.count):
            if self.owner[p] == self.rank:
                sub = mesh.subtree(self.level, p)
                self.local[p] = (sub, HPSAlgorithm(sub, patch_solver, options))
        self.top = HPSAlgorithm(mesh, patch_solver, options) if self.rank == 0 else None
        sizes = self.top.split_sizes(self.level) if self.rank == 0 else None
        self.sizes = self.tr.bcast_ints(sizes, self.count)
        self.n = mesh.root_patch.grid().nx()

    def _gather(self, local_arrays: Dict[int, np.ndarray], sizes: List[int], tag0: int) -> Optional[List[np.ndarray]]:
        """Rank 0 receives the array of every subtree (its own ones directly); others send theirs."""
        if self.rank != 0:
            for p, a in sorted(local_arrays.items()):
                self.tr.send(a, 0, tag0 + p)
            return None
        out = []
        for p in range(self.count):
            out.append(local_arrays[p] if self.owner[p] == 0 else self.tr.recv(sizes[p], self.owner[p], tag0 + p))
        return out

    def buildStage(self):
        Ts = {}
        for p, (_, h) in self.local.items():
            h.buildStage()
            if 4 * h.M != self.sizes[p]:
                raise ValueError(f"subtree {p}: root side {h.M} does not match the full tree's node ({self.sizes[p] // 4})")
            Ts[p] = h.root_T().ravel()
        got = self._gather(Ts, [m * m for m in self.sizes], 0)
        if self.rank == 0:
            self.top.buildStageTop(self.level, [T.reshape(m, m) for T, m in zip(got, self.sizes)])

    def upwardsStage(self, rhs: Callable[[np.ndarray, np.ndarray], np.ndarray]):
        """rhs(x, y) vectorised, sampled at every owned subtree's leaf cell centres."""
        hs = {}
        for p, (_, h) in self.local.items():
            h.upwardsStage(rhs)
            hs[p] = h.root_h()
        got = self._gather(hs, self.sizes, 1 << 20)
        if self.rank == 0:
            self.top.upwardsStageTop(self.level, got)

    def solveStage(self, bc):
        """bc(side, x, y) -> (r, a, b) on the full domain's boundary (evaluated on rank 0)."""
        tag0 = 2 << 20
        if self.rank == 0:
            gs = self.top.solveStageTop(self.level, *self.top.root_data(bc))
            for p in range(self.count):
                if self.owner[p] != 0:
                    self.tr.send(gs[p], self.owner[p], tag0 + p)
        lib = _lib.load()
        for p, (_, h) in sorted(self.local.items()):
            g = gs[p] if self.rank == 0 else self.tr.recv(self.sizes[p], 0, tag0 + p)
            g = np.ascontiguousarray(g)
            check(lib.ef_hps_solve_root_dirichlet(h.handle, dptr(g)))

    def leaf_solution(self) -> Optional[np.ndarray]:
        """The full mesh's leaf solutions in its leaf order, assembled on rank 0 (None elsewhere)."""
        nn = self.n * self.n
        us = {p: h.leaf_solution() for p, (_, h) in self.local.items()}
        got = self._gather(us, [(e - b) * nn for b, e in self.ranges], 3 << 20)
        return np.concatenate(got) if self.rank == 0 else None
