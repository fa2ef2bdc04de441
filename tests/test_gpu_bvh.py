"""The tree broadphase (Morton order, radix sort, hierarchical PLOC treelets, escape links, refit)
must find exactly the grid's pair set: the reference's own check is "H-PLOC pair set == grid pair
set" (tests/gpu-hploc.js). With identical pairs every later stage sees identical inputs, so whole
trajectories must agree bit for bit across rebuilds and refits, in batches and across eviction.
"""
import numpy as np
import pytest

import parity
from avbd_gb300 import createSolverPipeline, workloads

pytestmark = pytest.mark.gpu

KEYS = ("position", "rotation", "velocity", "angular", "prev_velocity")


@pytest.fixture(scope="module")
def pipe():
    p = createSolverPipeline("gb300", device=0)
    yield p
    p.destroy()


def _same_state(a, b):
    for k in KEYS:
        assert np.array_equal(a[k], b[k]), k


@pytest.mark.parametrize("n,extent", [(3000, 10.0), (700, 4.0)])
def test_tree_pairs_equal_grid_pairs_over_rebuilds(pipe, n, extent):
    scene = workloads.mixed_pile(n, seed=4242 + n, extent=extent)
    grid = pipe.createSolver(scene, {"broadphase": "grid"})
    tree = pipe.createSolver(scene, {"broadphase": "hploc", "bvh": {"rebuildInterval": 7}})
    for step in range(36):  # builds at steps 0, 7, 14, ...; refits in between
        grid.step(1)
        tree.step(1)
        pg, pt = grid.readPairs(), tree.readPairs()
        assert pg.shape == pt.shape and np.array_equal(pg, pt), step
        if step % 5 == 0:
            _same_state(grid.readBodyState(), tree.readBodyState())
    assert tree.readCounters()["pairs"] > n  # the pile is in contact
    _same_state(grid.readBodyState(), tree.readBodyState())
    grid.destroy()
    tree.destroy()


def test_tree_world_one_step_parity_with_oracle(pipe):
    scene = workloads.mixed_pile(500, seed=99, extent=5.0)
    scene.params.broadphase = "hploc"
    w = pipe.createSolver(scene)
    rep = parity.compare_step(w, scene, 30)
    assert rep["pairs_equal"] and rep["contact_counts_equal"] and rep["colors_equal"], rep
    assert rep["max_err_fp32"] <= parity.TOL, rep
    w.destroy()


def test_auto_picks_the_tree_for_a_jointed_cloth_and_matches_the_grid(pipe):
    # 110 x 110 cloth (12,100 small boxes with ball joints) plus bricks: the grid cell follows the
    # bricks, far larger than the cloth boxes, so "auto" selects the tree
    scene = workloads.cloth_wall(grid=110, wall=(20, 2, 10))
    auto = pipe.createSolver(scene)
    grid = pipe.createSolver(scene, {"broadphase": "grid"})
    for _ in range(3):
        auto.step(10)
        grid.step(10)
        assert np.array_equal(auto.readPairs(), grid.readPairs())
    _same_state(auto.readBodyState(), grid.readBodyState())
    auto.destroy()
    grid.destroy()


def test_tree_worlds_in_a_batch_and_across_eviction(pipe):
    scenes = [workloads.mixed_pile(n, seed=7000 + n, extent=4.0 + n / 200) for n in (300, 900, 150)]
    for sc in scenes[:2]:
        sc.params.broadphase = "hploc"
        sc.params.bvh_rebuild = 5
    batch = pipe.createBatch(scenes)
    batch.step(23)
    alone = []
    for sc in scenes:
        w = pipe.createSolver(sc)
        w.step(23)
        alone.append(w.readBodyState())
        w.destroy()
    for i in range(3):
        _same_state(batch.readBodyState(i), alone[i])
    batch.destroy()
    server = pipe.createServer(budgetBytes=4 << 30)
    wid = server.admit(scenes[1])
    server.advance(wid, 11)
    for _ in range(11):
        server.tick()
    server.evict(wid)
    server.advance(wid, 12)
    for _ in range(12):
        server.tick()
    _same_state(server.readBodyState(wid), alone[1])
    server.destroy()
