"""Serving loop: requests over several resident trees arrive at random times, are batched per tree
while other blocks run, and every result equals the same request solved alone (bit for bit) and
the FP64 HPS solution to <= 1e-10 relative.  The HBM budget limits the lanes."""
import threading
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ef(lib):
    import ellipticforest_gb300
    return ellipticforest_gb300


def tree(ef, kind):
    if kind == "uniform":
        root = ef.FiniteVolumePatch(ef.FiniteVolumeGrid(16, -1.0, 1.0, 16, -1.0, 1.0))
        mesh = ef.Mesh().uniform(3, root)
    else:
        root = ef.FiniteVolumePatch(ef.FiniteVolumeGrid(8, 0.0, 1.0, 8, 0.0, 1.0))
        mesh = ef.Mesh().refineByFunction(lambda x, y: y > 0.45 and x > 0.45, 0.0, 0, 5, root)
    hps = ef.HPSAlgorithm(mesh, ef.FiniteVolumeSolver(solver_type=ef.FISHPACK90))
    hps.buildStage()
    return mesh, hps


def request(mesh, hps, seed):
    rng = np.random.default_rng(seed)
    X, Y = mesh.cell_centres()
    amp, cx, cy, wd = rng.uniform(-1, 1, 8), rng.uniform(-1, 1, 8), rng.uniform(-1, 1, 8), rng.uniform(0.05, 0.3, 8)
    f = sum(amp[k] * np.exp(-((X - cx[k]) ** 2 + (Y - cy[k]) ** 2) / wd[k] ** 2) for k in range(8))
    co = rng.standard_normal((4, 6))
    r = np.concatenate([sum(co[s, m] * np.sin((m + 1) * np.pi * ((y if s < 2 else x) + 1) / 2) for m in range(6))
                        for s, (x, y) in enumerate(hps.boundary_points())])
    return f, np.ones_like(r), r


def test_server_mix_equals_alone(ef):
    trees = [tree(ef, "uniform"), tree(ef, "adaptive")]
    rng = np.random.default_rng(3)
    N = 40
    plan = [(int(rng.integers(0, 2)), 100 + k) for k in range(N)]
    reqs = [request(*trees[t], seed) for t, seed in plan]
    sweeps = [1, 2]  # per tree: the adaptive tree gets a second refinement sweep
    srv = ef.Server([h for _, h in trees], bmax=[6, 5], lanes=2, sweeps=sweeps)
    assert srv.lanes(0) == 2 and srv.lanes(1) == 2
    ids = [None] * N

    def producer():  # Poisson-like arrivals from another thread
        for k, (t, _) in enumerate(plan):
            ids[k] = srv.submit(t, *reqs[k])
            time.sleep(float(rng.exponential(2e-4)))

    th = threading.Thread(target=producer)
    th.start()
    th.join()
    results = [srv.wait(ids[k]) for k in range(N)]
    st = srv.stats()
    srv.close()
    assert st["completed"] == N and st["blocks"] < N  # some requests shared a block
    # the same requests alone, each in a block of one, and the FP64 HPS solution
    for t, (mesh, hps) in enumerate(trees):
        hps.mixed_init(1)
    for k, (t, _) in enumerate(plan):
        mesh, hps = trees[t]
        f, a, r = reqs[k]
        alone = hps.mixed_solve(f[None], a[None], r[None], sweeps=sweeps[t])[0]
        assert np.array_equal(results[k][0], alone), k
        hps.upwards_array(f)
        hps.solve_arrays(a, np.zeros_like(a), r)
        ref = hps.leaf_solution()
        assert np.abs(results[k][0] - ref).max() / np.abs(ref).max() <= 1e-10
        assert results[k][1] > 0


def test_server_budget_limits_lanes(ef):
    mesh, hps = tree(ef, "uniform")
    probe = ef.Server([hps], bmax=4, lanes=1)
    one_lane = probe.device_bytes()
    probe.close()
    srv = ef.Server([hps], bmax=4, lanes=3, hbm_budget_bytes=one_lane + 1)
    assert srv.lanes(0) == 1  # a second lane would not fit
    f, a, r = request(mesh, hps, 9)
    ids = [srv.submit(0, f, a, r) for _ in range(6)]
    outs = [srv.wait(i)[0] for i in ids]
    srv.close()
    for o in outs[1:]:
        assert np.array_equal(o, outs[0])


def test_server_thermal_root_operator_mix_equals_alone(ef):
    """A tree served with fixed Neumann sides (a = 0, b = 1 on S/N, Dirichlet on W/E, as the
    reference's thermal driver solves its many right-hand sides): results within 1e-10 of the FP64
    HPS solution and bit-identical to the same request alone."""
    mesh, hps = tree(ef, "uniform")
    M = hps.M
    a = np.concatenate([np.ones(2 * M), np.zeros(2 * M)])
    b = np.concatenate([np.zeros(2 * M), np.ones(2 * M)])
    reqs = [request(mesh, hps, 300 + k) for k in range(12)]
    srv = ef.Server([hps], bmax=5, lanes=2, sweeps=1)
    srv.set_root(0, a, b)
    ids = [srv.submit(0, f, np.zeros_like(r), r) for f, _, r in reqs]
    results = [srv.wait(i)[0] for i in ids]
    srv.close()
    hps.mixed_init(1)
    hps.mixed_set_root(a, b)
    for k, (f, _, r) in enumerate(reqs):
        alone = hps.mixed_solve(f[None], np.zeros_like(r)[None], r[None], sweeps=1)[0]
        assert np.array_equal(results[k], alone), k
        hps.upwards_array(f)
        hps.solve_arrays(a, b, r)
        ref = hps.leaf_solution()
        assert np.abs(results[k] - ref).max() / np.abs(ref).max() <= 1e-10
