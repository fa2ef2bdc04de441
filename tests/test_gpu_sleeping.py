"""Island sleeping (src/native/cpu/sleeping.js; world API src/native/cpu/world.js:859-890)
through the C ABI: step by step the engine's sleep flags and quiet times equal the float32
oracle's from the same state (and its poses and velocities agree within the parity tolerance),
across islands falling asleep, a late impact waking the world, and commands waking it; a
sleeping world gives the same bits alone, in a batch and served across eviction; the sleep
controls (enable/disable, allowSleep, wakeAll, stats, effective mass 0 in the 40-float record).
"""
import numpy as np
import pytest

import oracle as O
import parity
import ref_scenes
from avbd_gb300 import AvbdScene3D, createSolverPipeline
from avbd_gb300.pipeline import stage_edits
from avbd_gb300.scene import SolverParams

pytestmark = pytest.mark.gpu

KEYS = ("position", "rotation", "velocity", "angular", "prev_velocity")


@pytest.fixture(scope="module")
def pipe():
    p = createSolverPipeline("gb300", device=0)
    yield p
    p.destroy()


def _scene(late=True, sleeping=True, restitution=0.0):
    """Three stacks of four boxes, four spheres, and (late) a box dropped from 60 m onto the
    middle stack at about 3.5 s."""
    sc = AvbdScene3D(timeStep=1 / 60, iterations=10, gravity=-10)
    sc.addBox([40, 1, 40], position=[0, -0.5, 0], density=0)
    rng = np.random.default_rng(3)
    for x in (-4.0, 0.0, 4.0):
        for k in range(4):
            sc.addBox([1, 1, 1], position=[x + rng.uniform(-0.05, 0.05), 0.5 + 1.02 * k, rng.uniform(-0.05, 0.05)])
    for k in range(4):
        sc.addSphere(0.4, position=[-8.0 + 2.2 * k, 0.45, 6.0], restitution=restitution)
    if late:
        sc.addBox([1, 1, 1], position=[0.2, 60.0, 0.1])
    arr = sc.arrays()
    arr.params.sleeping = sleeping
    return arr


def _same(a, b, what=""):
    for k in KEYS:
        assert np.array_equal(a[k], b[k]), (what, k)


def _lockstep(pipe, sc, steps, edit_at=None):
    """Each step: the engine's state (with sleep flags and times) loaded into a float32 oracle,
    one step of both, sleep state compared exactly and poses/velocities within tolerance.
    Returns the number of sleeping bodies after each step."""
    w = pipe.createSolver(sc)
    counts = []
    for step in range(steps):
        st = w.exportState()
        o = O.OracleWorld(sc, fp64=False, app=True, colored=True)
        o.import_state(st)
        o.set_sleep(st["asleep"], st["sleep_time"])
        if step == edit_at:  # a command wakes every body (queued before the step)
            rec = stage_edits([{"body": 2, "linearVelocity": [0.0, 0.5, 0.0]}], sc.n_bodies, sc.params.dt)
            w.editRecords(rec)
            o.edit(rec)
        w.step(1)
        o.step(1)
        ga, gt = w.readSleepState()
        oa, ot = o.sleep_state()
        assert np.array_equal(ga, oa), step
        assert np.array_equal(gt, ot.astype(np.float32)), step
        g, b = w.readBodyState(), o.bodies()
        err = max(parity._err(g["position"], b["pos"]), parity._err(g["rotation"], b["quat"]),
                  parity._err(g["velocity"], b["vel"]), parity._err(g["angular"], b["angvel"]))
        assert err <= parity.TOL, (step, err)
        counts.append(int(ga.sum()))
    w.destroy()
    return counts


def test_sleep_state_matches_the_oracle_step_by_step(pipe):
    counts = _lockstep(pipe, _scene(restitution=0.5), 400, edit_at=330)
    assert max(counts) > 0  # islands fell asleep
    assert any(a > 0 and b == 0 for a, b in zip(counts, counts[1:]))  # and were woken


@pytest.mark.parametrize("index", [4, 11, 13])
def test_sleep_with_joints_and_ignore_pairs_matches_the_oracle(pipe, index):
    # pyramid (contacts only), soft body (joints, springs, ignore pairs), breakable joints
    sc = ref_scenes.build(index)
    sc.params = SolverParams(dt=1 / 60, gravity=-10.0, up=(0.0, 0.0, 1.0), iterations=10, sleeping=True)
    counts = _lockstep(pipe, sc, 300)
    if index != 11:
        assert counts[-1] > 0


def test_sleeping_world_alone_batched_and_served(pipe):
    scenes = [_scene(late=False, sleeping=False), _scene(), _scene(late=False)]
    alone = pipe.createSolver(scenes[1])
    alone.step(300)
    ref, ref_sleep = alone.readBodyState(), alone.readSleepState()
    assert ref_sleep[0].any()
    alone.destroy()
    batch = pipe.createBatch(scenes)
    batch.step(300)
    _same(batch.readBodyState(1), ref, "batch")
    a, t = batch.readSleepState(1)
    assert np.array_equal(a, ref_sleep[0]) and np.array_equal(t, ref_sleep[1])
    assert not batch.readSleepState(0)[0].any()  # sleeping off in world 0
    batch.destroy()
    server = pipe.createServer(budgetBytes=2 << 30)
    ids = [server.admit(sc) for sc in scenes]
    for i in ids:
        server.advance(i, 170)
    for _ in range(170):
        server.tick()
    server.evict(ids[1])
    server.advance(ids[1], 130)
    for _ in range(130):
        server.tick()
    _same(server.readBodyState(ids[1]), ref, "server")
    a, t = server.readSleepState(ids[1])
    assert np.array_equal(a, ref_sleep[0]) and np.array_equal(t, ref_sleep[1])
    server.destroy()


def test_sleep_controls(pipe):
    sc = _scene(late=False, sleeping=False)
    w = pipe.createSolver(sc)
    w.step(200)
    assert w.readSleepStats()["sleeping"] == 0  # off
    w.enableSleeping({"speedThreshold": 0.08, "timeThreshold": 0.6})
    w.step(100)
    n = w.readSleepStats()["sleeping"]
    assert n == int(np.sum(sc.mass > 0))
    before = w.readBodyState()
    w.step(10)
    _same(before, w.readBodyState(), "asleep")  # sleeping bodies hold still, velocities 0
    assert np.all(before["velocity"][sc.mass > 0] == 0)
    rec = w.readSelectedBodies([1, 2]).reshape(-1, 40)
    assert np.all(rec[:, 19] == 0)  # effective mass of a sleeping body
    w.wakeAll()
    assert w.readSleepStats()["sleeping"] == 0
    assert np.all(w.readSelectedBodies([1, 2]).reshape(-1, 40)[:, 19] > 0)
    w.step(60)
    assert w.readSleepStats()["sleeping"] == n  # quiet again: asleep after 0.6 s
    w.setSleepEnabled(1, False)  # its stack stays awake, the others fall asleep again
    assert w.readSleepStats()["sleeping"] == 0
    w.step(60)
    a, _ = w.readSleepState()
    assert not a[1:5].any() and a[5:].all()
    w.setVelocities([8], [[0.0, 0.0, 0.0]])  # a velocity write wakes the world
    assert w.readSleepStats()["sleeping"] == 0
    w.disableSleeping()
    w.step(100)
    assert w.readSleepStats()["sleeping"] == 0
    with pytest.raises(ValueError):
        w.enableSleeping({"speedThreshold": -1})
    w.destroy()
