"""Trigger bodies (isTrigger; src/native/cpu/cpuPhysics3D.js:148-156, sleeping.js:54,
restitution.js:68, world.js:342-350, 530, 757-784, queries.js:229-233): their contacts exist and
are reported (events with isTrigger and no impulse, word 11 of the body record) but apply no
forces, bounce or sleep links; casts see them unless told not to. Engine steps equal the float
oracle's bit for bit, before and after setSensor."""
import numpy as np
import pytest

import oracle as O
import parity
from avbd_gb300 import AvbdScene3D, createSolverPipeline

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pipe():
    p = createSolverPipeline("gb300", device=0)
    yield p
    p.destroy()


def _scene():
    # Y up: a static trigger slab over the ground, boxes and a sphere falling through it, a
    # dynamic trigger box falling onto the ground, a normal box resting beside them
    rng = np.random.default_rng(11)
    sc = AvbdScene3D(timeStep=1 / 60, iterations=10, gravity=-10)
    sc.addBox([20, 1, 20], density=0, position=[0, -0.5, 0])
    zone = sc.addBox([6, 0.5, 6], density=0, position=[0, 2.0, 0], isTrigger=True)
    falling = [sc.addBox(list(rng.uniform(0.4, 0.9, 3)), position=[rng.uniform(-2, 2), 3.0 + 1.2 * k, rng.uniform(-2, 2)])
               for k in range(6)]
    ball = sc.addSphere(0.4, position=[0.5, 5.0, 0.5], restitution=0.8)
    ghost = sc.addBox([1, 1, 1], position=[5, 1.5, 0], isTrigger=True)
    rest = sc.addBox([1, 1, 1], position=[-5, 0.5, 0])
    return sc, zone, falling, ball, ghost, rest


@pytest.mark.parametrize("warm", [0, 20, 60])
def test_trigger_step_parity(pipe, warm):
    sc, *_ = _scene()
    arr = sc.arrays()
    w = pipe.createSolver(sc)
    rep = parity.compare_step(w, arr, warm)
    assert rep["pairs_equal"] and rep["contact_counts_equal"] and rep["colors_equal"], rep
    assert rep["coloring_valid"] and rep["max_err_fp32"] <= parity.TOL, rep
    w.destroy()


def test_triggers_pass_through_and_report(pipe):
    sc, zone, falling, ball, ghost, rest = _scene()
    w = pipe.createSolver(sc)
    w.watchContacts({"maxEvents": 4096})
    w.step(120)
    st = w.readBodyState()
    assert np.sum(st["position"][falling, 1] < 1.75) >= 5  # fell through the trigger slab
    assert st["position"][ghost, 1] < -1.0  # a dynamic trigger falls through the ground as well
    assert abs(st["position"][rest, 1] - 0.49) < 0.02
    ev = w.readContactEvents()["events"]
    trig = [e for e in ev if zone in (e["a"], e["b"]) or ghost in (e["a"], e["b"])]
    assert trig and all(e["isTrigger"] for e in trig)
    assert all(e["impulse"] == 0 for e in trig if e["type"] == "begin")
    assert not any(e["isTrigger"] for e in ev if e not in trig)
    rec = w.readSelectedBodies([zone, rest]).reshape(-1, 40)
    assert rec[0, 11] == 1 and rec[1, 11] == 0
    w.destroy()


def test_casts_skip_triggers_on_request(pipe):
    sc, zone, *_ = _scene()
    w = pipe.createSolver(sc)
    # a ray past every falling body (they start within 2.45 m of the axis) onto the slab's corner
    hit = w.raycast([2.9, 8, 2.9], [0, -1, 0])
    assert hit is not None and hit["index"] == zone
    hit = w.raycast([2.9, 8, 2.9], [0, -1, 0], {"includeTriggers": False})
    assert hit is not None and hit["index"] == 0  # the ground below it
    w.destroy()


def test_set_sensor_keeps_parity_and_drops_the_body(pipe):
    sc, zone, falling, ball, ghost, rest = _scene()
    arr = sc.arrays()
    w = pipe.createSolver(sc)
    w.step(30)
    w.setSensor(rest, True)
    w.editBodies([{"body": zone, "isTrigger": False}])  # the slab turns solid
    arr.is_trigger = arr.is_trigger.copy()
    arr.is_trigger[rest] = True
    arr.is_trigger[zone] = False
    rep = parity.compare_step(w, arr, 0)
    assert rep["pairs_equal"] and rep["max_err_fp32"] <= parity.TOL, rep
    rep = parity.compare_step(w, arr, 30)
    assert rep["pairs_equal"] and rep["max_err_fp32"] <= parity.TOL, rep
    assert w.readBodyState()["position"][rest, 1] < 0.0  # no longer held by the ground
    w.destroy()
