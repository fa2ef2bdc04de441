"""The oracle's spring fracture (src/gpu/springMaterial.js limits, checked at the step start as
src/native/cpu/cpuPhysics3D.js:276-299 does) and the builder's spring material options
(src/native/scenes.js:541-569): a spring tears once its extension at the start of a step passes
breakStrain x rest or breakForce / stiffness, never under compression, and the torn spring stops
acting (its body falls freely); setSpringMaterial, setWorldAnchor and captureConstraintFrames by
joint slot."""
import math

import numpy as np
import pytest

import oracle as O
from avbd_gb300 import AvbdScene3D

G = -10.0
DT = 1 / 60


def _hanging(stiffness=200.0, **material):
    # Y up, no ground: a 1 kg box hangs from a static anchor on a spring of rest length 1
    sc = AvbdScene3D(timeStep=DT, iterations=10, gravity=G)
    top = sc.addBox([0.2, 0.2, 0.2], density=0, position=[0, 5, 0])
    box = sc.addBox([1, 1, 1], position=[0, 4, 0])
    s = sc.addSpring(top, box, anchorA=[0, 0, 0], anchorB=[0, 0, 0], stiffness=stiffness, rest=1.0, **material)
    return sc, box, s


def _trajectory(sc, steps):
    o = O.OracleWorld(sc.arrays(), fp64=True, app=True, colored=True)
    pos, vel = [], []
    for _ in range(steps):
        o.step(1)
        b = o.bodies()
        pos.append(b["pos"].copy())
        vel.append(b["vel"].copy())
    return o, np.array(pos), np.array(vel)


def _tear_step(pos, box, rest, limit_ext):
    """First step whose start extension (the previous step's end) passes limit_ext."""
    ext = np.maximum(0.0, 5.0 - pos[:, box, 1] - rest)  # anchor at y = 5, spring vertical
    over = np.nonzero(ext > limit_ext)[0]
    return int(over[0]) + 1 if over.size else None


@pytest.mark.parametrize("material, limit_ext", [({"breakForce": 12.0}, 12.0 / 200.0),
                                                 ({"breakStrain": 0.04}, 0.04 * 1.0)])
def test_spring_tears_past_its_limit_and_then_stops_acting(material, limit_ext):
    sc, box, _ = _hanging(**material)  # static stretch m g / k = 0.05
    o, pos, vel = _trajectory(sc, 60)
    k = _tear_step(pos, box, 1.0, limit_ext)
    assert k is not None and k < 30
    # from the step after the tear the box falls freely: dv = g dt per step
    dv = np.diff(vel[k:, box, 1])
    assert np.allclose(dv, G * DT, atol=1e-9), dv[:5]
    # before it, the spring still pulled
    assert vel[k - 1, box, 1] - vel[k - 2, box, 1] > G * DT + 1e-3


def test_spring_holds_below_its_limits_and_never_tears_in_compression():
    sc, box, _ = _hanging(breakForce=30.0, breakStrain=0.5)
    _, pos, vel = _trajectory(sc, 240)
    assert abs(vel[-1, box, 1]) < 0.05 and abs(5.0 - pos[-1, box, 1] - 1.05) < 0.02
    # a spring squeezed far below its rest length (a box pressed into the ground by a static
    # anchor above it) with tiny limits stays
    sc = AvbdScene3D(timeStep=DT, iterations=10, gravity=G)
    sc.addBox([20, 1, 20], density=0, position=[0, -0.5, 0])
    b = sc.addBox([1, 1, 1], position=[0, 0.5, 0])
    top = sc.addBox([1, 1, 1], density=0, position=[0, 1.6, 0])
    sc.addSpring(top, b, stiffness=500.0, rest=3.0, breakStrain=1e-6, breakForce=1e-6)
    o = O.OracleWorld(sc.arrays(), fp64=True, app=True, colored=True)
    o.step(30)
    assert o.counts()["springs"] == 1


def test_set_spring_material_world_anchor_and_frames_by_slot():
    sc, box, s = _hanging()
    o = O.OracleWorld(sc.arrays(), fp64=True, app=True, colored=True)
    o.step(20)
    o.set_spring_material(0, break_force=1.0)  # far below the load: tears at the next step start
    o.step(2)
    assert o.counts()["springs"] == 0
    with pytest.raises(ValueError):
        o.set_spring_material(0, break_force=1.0)  # torn: no longer a live spring
    # a grab handle: a world joint whose anchor moves drags the body along
    sc = AvbdScene3D(timeStep=DT, iterations=10, gravity=0)
    b = sc.addBox([1, 1, 1], position=[0, 0, 0])
    sc.addJoint(None, b, anchorA=[0, 0, 0], anchorB=[0, 0, 0], linearStiffness=5000.0)
    o = O.OracleWorld(sc.arrays(), fp64=True, app=True, colored=True)
    for k in range(120):
        o.set_world_anchor(0, [k * 0.02, 0, 0])
        o.step(1)
    assert abs(o.bodies()["pos"][b, 0] - 119 * 0.02) < 0.1
    with pytest.raises(ValueError):
        o.capture_frames([(0, True)])  # a joint is not a spring
    o.capture_frames([(0, False)])


def test_builder_spring_material_options():
    sc = AvbdScene3D()
    a = sc.addBox([1, 1, 1], density=0)
    b = sc.addBox([1, 1, 1], position=[0, 2, 0])
    s0 = sc.addSpring(a, b)
    s1 = sc.addSpring(a, b, breakStrain=0.5, breakForce=40.0)
    arr = sc.arrays()
    assert math.isinf(arr.p2[s0]) and math.isinf(arr.p3[s0])
    assert (arr.p2[s1], arr.p3[s1]) == (40.0, 0.5)
    for bad in ({"breakStrain": 0.0}, {"breakForce": -1.0}, {"breakStrain": float("nan")}):
        with pytest.raises(ValueError):
            sc.addSpring(a, b, **bad)
