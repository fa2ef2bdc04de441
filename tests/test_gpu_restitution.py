"""Restitution (addBox/addSphere `restitution`, the velocity bounce after the solve of
src/native/cpu/restitution.js in the GPU backend's arrangement, src/gpu/restitution.js) through
the C ABI: per manifold the contact centroids, the incoming normal speed from the step's starting
velocities, a 1 m/s impact threshold and 12 Jacobi rounds relaxed by the constraint-list length.
The engine must match the float32 oracle over a step with impacts, and a bouncy world must give
the same bits alone, in a batch beside worlds without restitution, and served across eviction.
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


def _bouncy(n, seed, share=0.7):
    scene = workloads.mixed_pile(n, seed=seed, extent=5.0)
    rng = np.random.default_rng(seed)
    e = rng.uniform(0.2, 0.95, scene.n_bodies)
    e[rng.random(scene.n_bodies) >= share] = 0.0
    scene.restitution = e
    return scene


@pytest.mark.parametrize("warm", [38, 55, 90])
def test_bounce_step_matches_the_oracle(pipe, warm):
    # bodies fall from 2..7 m: the first impacts (several m/s) come after about 35 steps
    scene = _bouncy(400, 71 + warm)
    w = pipe.createSolver(scene)
    rep = parity.compare_step(w, scene, warm)
    assert rep["pairs_equal"] and rep["contact_counts_equal"] and rep["colors_equal"], rep
    assert rep["max_err_fp32"] <= parity.TOL, rep
    got = w.readBodyState()
    w.destroy()
    # the same step without restitution differs: the pass did bounce something
    plain = workloads.mixed_pile(400, seed=71 + warm, extent=5.0)
    p = pipe.createSolver(plain)
    p.step(warm + 1)
    assert not np.array_equal(p.readBodyState()["velocity"], got["velocity"])
    p.destroy()


def test_sphere_dropped_on_the_ground_bounces_back_up(pipe):
    from avbd_gb300 import AvbdScene3D
    sc = AvbdScene3D(timeStep=1 / 60, iterations=10, gravity=-10)
    sc.addBox([20, 1, 20], position=[0, -0.5, 0], density=0)
    s = sc.addSphere(0.5, position=[0, 0.6, 0], velocity=[0, -6, 0], restitution=0.8)
    w = pipe.createSolver(sc)
    vmax = 0.0
    for _ in range(6):
        w.step(1)
        vmax = max(vmax, float(w.readBodyState()["velocity"][s][1]))
    assert vmax > 3.0  # about e x 6 m/s back up
    w.destroy()


def test_bouncy_world_alone_in_a_batch_and_served(pipe):
    scenes = [workloads.mixed_pile(150, seed=5, extent=4.0), _bouncy(300, 6), workloads.mixed_pile(90, seed=7, extent=4.0)]
    alone = pipe.createSolver(scenes[1])
    alone.step(70)
    ref = alone.readBodyState()
    alone.destroy()
    batch = pipe.createBatch(scenes)
    batch.step(70)
    for k in KEYS:
        assert np.array_equal(batch.readBodyState(1)[k], ref[k]), k
    batch.destroy()
    server = pipe.createServer(budgetBytes=2 << 30)
    ids = [server.admit(sc) for sc in scenes]
    for i in ids:
        server.advance(i, 40)
    for _ in range(40):
        server.tick()
    server.evict(ids[1])
    server.advance(ids[1], 30)
    for _ in range(30):
        server.tick()
    got = server.readBodyState(ids[1])
    for k in KEYS:
        assert np.array_equal(got[k], ref[k]), k
    server.destroy()
