"""Edge cases of the world, batch and server paths (the reference's tests include the empty and
ground-only scenes, tests/avbd3d-ref.test.ts): worlds with no bodies, only static bodies, one free
body; batches mixing them with ordinary worlds; a server admitting and stepping them; empty calls
(no indices, no records, no queries) that must succeed and change nothing.
"""
import numpy as np
import pytest

import parity
import ref_scenes
from avbd_gb300 import createSolverPipeline, workloads
from avbd_gb300.scene import SolverParams

pytestmark = pytest.mark.gpu

KEYS = ("position", "rotation", "velocity", "angular", "prev_velocity")


@pytest.fixture(scope="module")
def pipe():
    p = createSolverPipeline("gb300", device=0)
    yield p
    p.destroy()


def _scene(index):
    sc = ref_scenes.build(index)
    sc.params = SolverParams(dt=1 / 60, gravity=-10.0, up=(0.0, 0.0, 1.0), iterations=10)
    return sc


def test_empty_and_ground_only_worlds(pipe):
    empty, ground = _scene(0), _scene(1)
    assert empty.n_bodies == 0
    w = pipe.createSolver(empty)
    w.step(5)
    assert w.readBodyState()["position"].shape == (0, 3)
    assert w.readCounters()["pairs"] == 0
    assert w.readSelectedBodies([]).size == 0
    assert w.sphereCastAll([]) == [] and w.raycast([0, 0, 5], [0, 0, -1]) is None
    w.editBodies([])
    w.setVelocities([], [])
    assert w.readContactEvents()["events"] == []
    w.destroy()
    g = pipe.createSolver(ground)
    rep = parity.compare_step(g, ground, 10)
    assert rep["max_err_fp32"] <= parity.TOL and rep["pairs_equal"], rep
    g.destroy()


def test_batch_and_server_with_empty_worlds(pipe):
    scenes = [_scene(0), workloads.mixed_pile(50, seed=3, extent=4.0), _scene(1), _scene(0)]
    alone = pipe.createSolver(scenes[1])
    alone.step(12)
    ref = alone.readBodyState()
    alone.destroy()
    batch = pipe.createBatch(scenes)
    batch.step(12)
    got = batch.readBodyState(1)
    for k in KEYS:
        assert np.array_equal(got[k], ref[k]), k
    assert batch.readBodyState(0)["position"].shape == (0, 3)
    poses = batch.readPoses()
    assert poses.shape == (batch.bodyCount, 8)
    batch.destroy()
    server = pipe.createServer(budgetBytes=1 << 30)
    ids = [server.admit(sc) for sc in scenes]
    for i in ids:
        server.advance(i, 12)
    for _ in range(12):
        server.tick()
    for k in KEYS:
        assert np.array_equal(server.readBodyState(ids[1])[k], ref[k]), k
    assert server.readPoses([ids[0], ids[3]]).shape == (0, 8)
    t = server.advance(ids[0], 0)
    assert t in server.completed()
    server.destroy()


def test_one_free_body_falls_like_the_oracle(pipe):
    from avbd_gb300 import AvbdScene3D
    sc = AvbdScene3D(timeStep=1 / 60, iterations=10, gravity=-10)
    sc.addSphere(0.5, position=[0, 10, 0], velocity=[1, 0, 0], angularVelocity=[0, 2, 0])
    arr = sc.arrays()
    w = pipe.createSolver(sc)
    rep = parity.compare_step(w, arr, 20)
    assert rep["max_err_fp32"] <= parity.TOL and rep["pairs_gpu"] == 0, rep
    w.destroy()


@pytest.mark.parametrize("broadphase", ["grid", "hploc"])
def test_ground_created_last_owns_its_pairs(pipe, broadphase):
    # pairs belong to their higher-index body: a ground created after 2,000 bodies owns every
    # contact with it (its range is ordered by heapsort beyond 64 partners); same pairs, same step
    sc = workloads.mixed_pile(2000, seed=23, extent=8.0)
    perm = np.r_[np.arange(1, sc.n_bodies), 0]  # the ground (body 0) moves to the last slot
    for k in ("pos", "quat", "size", "vel", "angvel", "prev_vel", "mass", "moment", "friction", "radius",
              "shape", "group", "mask"):
        setattr(sc, k, np.asarray(getattr(sc, k))[perm])
    sc.params.broadphase = broadphase
    w = pipe.createSolver(sc)
    rep = parity.compare_step(w, sc, 60)
    assert rep["pairs_equal"] and rep["contact_counts_equal"] and rep["colors_equal"], rep
    assert rep["max_err_fp32"] <= parity.TOL, rep
    ground = sc.n_bodies - 1
    assert int(np.sum(w.readPairs()[:, 0] == ground)) > 64
    w.destroy()


def test_sphere_box_pairs_around_the_touching_distance(pipe):
    # spheres placed at distances from 2 cm inside to 2 cm outside rotated boxes (face, edge and
    # corner regions): contact counts, poses and velocities as the oracle's one step
    from avbd_gb300 import AvbdScene3D
    rng = np.random.default_rng(8)
    sc = AvbdScene3D(timeStep=1 / 60, iterations=10, gravity=0)
    for k in range(60):
        c = np.array([6.0 * (k % 10), 0.0, 6.0 * (k // 10)])
        q = rng.normal(size=4)
        q /= np.linalg.norm(q)
        h = rng.uniform(0.3, 1.0, 3)
        sc.addBox(list(2 * h), position=list(c), rotation=list(q), density=0)
        local = rng.normal(size=3) * h * 2.5  # a point around the box, in its frame
        nearest = np.clip(local, -h, h)
        d = local - nearest
        if np.linalg.norm(d) < 1e-3:
            d = np.array([1.0, 0.0, 0.0]) * h[0]
            nearest = np.array([h[0], 0.0, 0.0])
        r = 0.4
        gap = rng.uniform(-0.02, 0.02)
        p_local = nearest + d / np.linalg.norm(d) * (r + gap)
        x, y, z, w = q
        R = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                      [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                      [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])
        sc.addSphere(r, position=list(c + R @ p_local))
    arr = sc.arrays()
    w = pipe.createSolver(sc)
    rep = parity.compare_step(w, arr, 0)
    assert rep["pairs_equal"] and rep["contact_counts_equal"], rep
    assert rep["max_err_fp32"] <= parity.TOL, rep
    assert 10 < rep["contacts"] < 60, rep  # both touching and clearly separated pairs
    w.destroy()
