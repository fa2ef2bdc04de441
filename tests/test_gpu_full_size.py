"""Size-independent checks at the benchmark sizes: the 4,096-world mix (2.1 M bodies) stepped as one
batch gives each sampled world (the largest, the smallest and others) the bits it gets stepped
alone, every pose stays finite and the colouring has no conflicts; the 1 M-body mixed pile's pair
set from the tree equals the grid's (the reference's own tree check, tests/gpu-hploc.js:16-62),
step after step."""
import numpy as np
import pytest

from avbd_gb300 import createSolverPipeline, workloads

pytestmark = pytest.mark.gpu

KEYS = ("position", "rotation", "velocity", "angular", "prev_velocity")


@pytest.fixture(scope="module")
def pipe():
    p = createSolverPipeline("gb300", device=0)
    yield p
    p.destroy()


def test_world_mix_4096_batch_matches_worlds_alone(pipe):
    scenes, counts, _ = workloads.world_mix()
    assert len(scenes) == 4096 and int(counts.sum()) > 2_000_000
    steps = 4
    batch = pipe.createBatch(scenes)
    batch.step(steps)
    c = batch.readCounters()
    assert c["conflicts"] == 0 and c["overflow"] >= 0
    pick = sorted({0, 1, 2047, 4095, int(np.argmax(counts)), int(np.argmin(counts))})
    for i in pick:
        w = pipe.createSolver(scenes[i])
        w.step(steps)
        ref = w.readBodyState()
        w.destroy()
        got = batch.readBodyState(i)
        for k in KEYS:
            assert np.array_equal(got[k], ref[k]), (i, k)
    poses = batch.readPoses()
    assert poses.shape == (batch.bodyCount, 8) and np.all(np.isfinite(poses))
    batch.destroy()


def test_mixed_1m_tree_pairs_equal_grid_pairs(pipe):
    scene = workloads.mixed_pile(1_000_000, seed=0xA5BD0001)
    worlds = {}
    for bp in ("grid", "hploc"):
        scene.params.broadphase = bp
        worlds[bp] = pipe.createSolver(scene)
    for _ in range(3):
        pairs = {}
        for bp, w in worlds.items():
            w.step(1)
            pairs[bp] = w.readPairs()
        assert len(pairs["grid"]) > 1_000_000 and np.array_equal(pairs["grid"], pairs["hploc"])
        a, b = (worlds[k].readBodyState() for k in ("grid", "hploc"))
        for k in KEYS:
            assert np.array_equal(a[k], b[k]), k
    for w in worlds.values():
        w.destroy()
