"""Constraint edits on the engine, each driven the same way on the float oracle, whose steps the
engine's must equal bit for bit: spring fracture (src/gpu/springMaterial.js limits at the step
start), setSpringMaterial, setWorldAnchor (a dragged grab handle), captureConstraintFrames (a weld's
rest rotation and a spring's rest length taken again), disableConstraint; the joint records they
leave (src/gpu/appGpuSolver3D.js:826-833 layout) and their argument errors."""
import math

import numpy as np
import pytest

import oracle as O
from avbd_gb300 import AvbdScene3D, createSolverPipeline
from avbd_gb300._lib import AvbdError

pytestmark = pytest.mark.gpu

DT = 1 / 60


@pytest.fixture(scope="module")
def pipe():
    p = createSolverPipeline("gb300", device=0)
    yield p
    p.destroy()


def _same(w, o):
    g, c = w.readBodyState(), o.bodies()
    for gk, ck in (("position", "pos"), ("rotation", "quat"), ("velocity", "vel"), ("angular", "angvel")):
        assert np.array_equal(g[gk].astype(np.float64), c[ck]), gk


def _pair(pipe, sc):
    return pipe.createSolver(sc), O.OracleWorld(sc.arrays(), fp64=False, app=True, colored=True)


def _hanging(**material):
    sc = AvbdScene3D(timeStep=DT, iterations=10, gravity=-10)
    top = sc.addBox([0.2, 0.2, 0.2], density=0, position=[0, 5, 0])
    box = sc.addBox([1, 1, 1], position=[0, 4, 0])
    s = sc.addSpring(top, box, stiffness=200.0, rest=1.0, **material)
    return sc, box, s


def test_spring_tear_is_bit_equal(pipe):
    sc, box, s = _hanging(breakForce=12.0)
    w, o = _pair(pipe, sc)
    torn = None
    for k in range(40):
        w.step(1)
        o.step(1)
        _same(w, o)
        rec = w.readJoints().reshape(-1, 32)[0]
        if torn is None and rec[3] == 0:
            torn = k
        assert (rec[3] == 0) == (o.counts()["springs"] == 0)
    assert torn is not None and torn < 30
    w.destroy()


def test_set_spring_material_is_bit_equal(pipe):
    sc, box, s = _hanging()
    w, o = _pair(pipe, sc)
    w.step(20)
    o.step(20)
    rec = w.readJoints().reshape(-1, 32)[0]
    assert rec[3] == 200.0 and rec[11] == 0 and rec[15] == 0
    w.setSpringMaterial(s, breakStrain=0.5, breakForce=1.0)
    o.set_spring_material(0, break_strain=0.5, break_force=1.0)
    rec = w.readJoints().reshape(-1, 32)[0]
    assert rec[11] == 0.5 and rec[15] == 1.0
    for _ in range(10):
        w.step(1)
        o.step(1)
        _same(w, o)
    assert w.readJoints().reshape(-1, 32)[0, 3] == 0 and o.counts()["springs"] == 0
    with pytest.raises(AvbdError):  # torn: no longer a live spring
        w.setSpringMaterial(s, breakForce=5.0)
    w.destroy()


def test_world_anchor_drag_is_bit_equal(pipe):
    sc = AvbdScene3D(timeStep=DT, iterations=10, gravity=-10)
    sc.addBox([20, 1, 20], density=0, position=[0, -0.5, 0])
    b = sc.addBox([1, 1, 1], position=[0, 2, 0])
    c = sc.addBox([1, 1, 1], position=[3, 0.5, 0])
    grab = sc.addJoint(None, b, anchorA=[0, 2.5, 0], anchorB=[0, 0.5, 0], linearStiffness=5000.0)
    w, o = _pair(pipe, sc)
    for k in range(60):
        p = [0.05 * k, 2.5 + 0.01 * k, 0.0]
        w.setWorldAnchor(grab, p)
        o.set_world_anchor(0, p)
        w.step(1)
        o.step(1)
        _same(w, o)
    assert w.readBodyState()["position"][b, 0] > 1.5  # dragged along (and into the other box)
    with pytest.raises(ValueError):
        w.setWorldAnchor(grab, [0, math.nan, 0])
    w.destroy()


def test_capture_frames_is_bit_equal(pipe):
    sc = AvbdScene3D(timeStep=DT, iterations=10, gravity=-10)
    post = sc.addBox([0.4, 0.4, 0.4], density=0, position=[0, 3, 0])
    arm = sc.addBox([2, 0.2, 0.2], position=[1.2, 3, 0])
    weld = sc.addJoint(post, arm, anchorA=[0.2, 0, 0], anchorB=[-1.0, 0, 0], angularStiffness=200.0)
    bob = sc.addBox([0.5, 0.5, 0.5], position=[2.2, 1.5, 0])
    spring = sc.addSpring(arm, bob, anchorA=[1.0, 0, 0], anchorB=[0, 0.25, 0], stiffness=300.0)
    w, o = _pair(pipe, sc)
    w.step(15)
    o.step(15)
    _same(w, o)
    w.captureConstraintFrames([weld, {"slot": spring, "spring": True}])
    o.capture_frames([(0, False), (1, True)])
    for _ in range(30):
        w.step(1)
        o.step(1)
        _same(w, o)
    with pytest.raises(AvbdError):
        w.captureConstraintFrames([{"slot": weld, "spring": True}])
    w.disableConstraint(spring)
    assert w.readJoints().reshape(-1, 32)[1, 3] == 0
    with pytest.raises(AvbdError):
        w.captureConstraintFrames([{"slot": spring, "spring": True}])  # released
    with pytest.raises(AvbdError):
        w.setWorldAnchor(weld, [0, 0, 0])  # not attached to the world
    with pytest.raises(ValueError):
        w.setSpringMaterial(weld, breakForce=1.0)
    w.destroy()


def test_batch_edits_match_the_world_alone(pipe):
    # the batch forms of the property and constraint edits give a batched world the bits of the
    # same world edited alone (the other batched world untouched)
    def scene():
        sc = AvbdScene3D(timeStep=DT, iterations=10, gravity=-10)
        sc.addBox([20, 1, 20], density=0, position=[0, -0.5, 0])
        top = sc.addBox([0.2, 0.2, 0.2], density=0, position=[0, 5, 0])
        box = sc.addBox([1, 1, 1], position=[0, 4, 0])
        s = sc.addSpring(top, box, stiffness=200.0, rest=1.0)
        ball = sc.addSphere(0.4, position=[3, 2, 0])
        grab = sc.addJoint(None, ball, anchorA=[3, 2.5, 0], anchorB=[0, 0.4, 0], linearStiffness=3000.0)
        other = sc.addBox([1, 1, 1], position=[-3, 0.5, 0])
        return sc, box, s, ball, grab, other

    def edits(obj, w, parts):
        sc, box, s, ball, grab, other = parts
        args = () if w is None else (w,)
        obj.setFilters(*args, [other], [2], [2])
        obj.setRestitution(*args, [ball], [0.5])
        obj.setSensor(*args, other, True)
        obj.setSpringMaterial(*args, s, breakForce=8.0)
        obj.setWorldAnchor(*args, grab, [3.5, 3.0, 0.0])
        obj.captureConstraintFrames(*args, [{"slot": s, "spring": True}])

    parts = scene()
    alone = pipe.createSolver(parts[0])
    alone.step(10)
    edits(alone, None, parts)
    alone.step(30)
    ref = alone.readBodyState()
    alone.destroy()
    batch = pipe.createBatch([scene()[0], parts[0]])
    batch.step(10)
    edits(batch, 1, parts)
    batch.step(30)
    got = batch.readBodyState(1)
    for k in ("position", "rotation", "velocity", "angular"):
        assert np.array_equal(got[k], ref[k]), k
    batch.destroy()


def test_batch_property_edits_match_the_world_alone(pipe):
    def scene():
        sc = AvbdScene3D(timeStep=DT, iterations=10, gravity=-10)
        sc.addBox([20, 1, 20], density=0, position=[0, -0.5, 0])
        a = sc.addSphere(0.4, position=[0, 3, 0])
        b = sc.addBox([1, 1, 1], position=[2, 0.5, 0])
        c = sc.addBox([1, 1, 1], position=[-2, 3, 0])
        return sc, a, b, c

    sc, a, b, c = scene()
    edits = [{"body": a, "restitution": 0.7}, {"body": b, "isTrigger": True},
             {"body": c, "group": 2, "collidesWith": 2, "allowSleep": False, "linearVelocity": [1, 0, 0]}]
    w = pipe.createSolver(sc)
    w.step(5)
    w.editBodies(edits)
    w.step(40)
    ref = w.readBodyState()
    w.destroy()
    batch = pipe.createBatch([scene()[0], sc])
    batch.step(5)
    batch.editBodies(1, edits)
    batch.step(40)
    got = batch.readBodyState(1)
    for k in ("position", "rotation", "velocity", "angular"):
        assert np.array_equal(got[k], ref[k]), k
    assert got["position"][b, 1] < 0  # the trigger box fell through the ground
    batch.destroy()
