"""The oracle's angular rows: hinge motors and angle limits (src/gpu/angularConstraints.js,
frames as src/gpu/angularFrames.wgsl, restated in oracle/avbd_oracle.hpp).

The rows measure the twist with an atan2 written from the half-angle identity and a Taylor series
(so that the engine and the float oracle share its bits); it is checked here against numpy's. The
rows are pinned on the reference's own hinge check (tests/gpu-package-features.js:518-589: the
motor's first impulse, both stops holding against the motor, the pivot and the other axes locked)
and checked by what they do on small scenes: a motor turns a free wheel at its speed, a motor whose
torque bound is below the load slips while a strong one holds, released rows stop acting.
"""
import math

import numpy as np
import pytest

import oracle as O
from avbd_gb300 import AvbdScene3D


def test_atan2_restatement_matches_numpy():
    rng = np.random.default_rng(4)
    ang = np.linspace(-math.pi, math.pi, 20001)
    r = rng.uniform(1e-3, 1e3, ang.size)
    y, x = r * np.sin(ang), r * np.cos(ang)
    y = np.r_[y, 0.0, 0.0, 1.0, -1.0, 0.0, 1e-30, 3.0]
    x = np.r_[x, 1.0, -1.0, 0.0, 0.0, 0.0, 1.0, 3.0]
    ref = np.arctan2(y, x)
    ref[-3] = 0.0  # atan2(0, 0) is 0 here as in WGSL/JS
    d64 = O.angle_atan2(y, x, fp64=True)
    assert np.max(np.abs(d64 - ref)) < 1e-8
    y32, x32 = y.astype(np.float32).astype(np.float64), x.astype(np.float32).astype(np.float64)
    d32 = O.angle_atan2(y32, x32, fp64=False)
    assert np.max(np.abs(d32 - np.arctan2(y32, x32) * (np.abs(y32) + np.abs(x32) > 0))) < 1e-6


def _twist(quat):
    """Rotation angle about z of planar rotations (x, y, z, w)."""
    return 2.0 * np.arctan2(quat[..., 2], quat[..., 3])


def _run(sc, steps, fp64=True):
    o = O.OracleWorld(sc.arrays(), fp64=fp64, app=True, colored=True)
    qs, ws = [], []
    for _ in range(steps):
        o.step(1)
        b = o.bodies()
        qs.append(b["quat"].copy())
        ws.append(b["angvel"].copy())
    return np.array(qs), np.array(ws)


def _wheel(speed, torque):
    sc = AvbdScene3D(timeStep=1 / 60, iterations=10, gravity=0)
    w = sc.addBox([1.0, 1.0, 0.2], position=[0, 0, 0])
    h = sc.addHinge(None, w, axisA=[0, 0, 1], axisB=[0, 0, 1], span=0.4,
                    motor={"speed": speed, "maxTorque": torque})
    return sc, w, h


@pytest.mark.parametrize("fp64", [True, False])
def test_motor_turns_a_free_wheel_at_its_speed(fp64):
    sc, w, _ = _wheel(2.0, 1000.0)
    q, om = _run(sc, 120, fp64)
    assert abs(om[-1, w, 2] - 2.0) < 0.02, om[-1, w]
    assert np.max(np.abs(om[-1, w, :2])) < 1e-3
    # over the last second the twist advanced by speed x time (wrapped)
    d = math.remainder(float(_twist(q[-1, w]) - _twist(q[59, w])), 2 * math.pi)
    assert abs(d - math.remainder(2.0 * 60 / 60, 2 * math.pi)) < 0.05, d


def _arm(motor=None, lo=None, hi=None):
    # a 2 m arm hinged at its left end to the world, horizontal at rest, gravity along -y
    sc = AvbdScene3D(timeStep=1 / 60, iterations=10, gravity=-10, up=[0, 1, 0])
    arm = sc.addBox([2.0, 0.2, 0.2], position=[1.0, 0, 0])
    h = sc.addHinge(None, arm, anchorA=[0, 0, 0], anchorB=[-1.0, 0, 0], axisA=[0, 0, 1], axisB=[0, 0, 1], span=0.4,
                    minAngle=lo, maxAngle=hi, motor=motor)
    return sc, arm, h


def test_motor_torque_bound_decides_whether_the_load_is_held():
    # gravity's torque about the pivot: m g L / 2 = (2 * 0.2 * 0.2) * 10 * 1 = 0.8 N m
    sc, arm, _ = _arm(motor={"speed": 0.0, "maxTorque": 100.0})
    q, _ = _run(sc, 90)
    assert np.max(np.abs(_twist(q[:, arm]))) < 0.02
    sc, arm, _ = _arm(motor={"speed": 0.0, "maxTorque": 0.2})
    q, _ = _run(sc, 90)
    assert _twist(q[-1, arm]) < -0.5


def _rotor(fp64):
    # the reference's hinge check (tests/gpu-package-features.js:518-589): a unit box on a world
    # hinge about z, stops at +-0.4 rad, a motor at 2 rad/s with 1 N m, no gravity, 20 iterations
    sc = AvbdScene3D(timeStep=1 / 60, iterations=20, gravity=0)
    b = sc.addBox([1, 1, 1], position=[0, 0, 0])
    h = sc.addHinge(None, b, axisA=[0, 0, 1], axisB=[0, 0, 1], minAngle=-0.4, maxAngle=0.4,
                    motor={"speed": 2, "maxTorque": 1})
    return sc, b, h, O.OracleWorld(sc.arrays(), fp64=fp64, app=True, colored=True)


@pytest.mark.parametrize("fp64", [True, False])
def test_reference_hinge_check_stops_hold_against_the_motor(fp64):
    sc, b, h, o = _rotor(fp64)
    o.step(1)
    st = o.bodies()
    assert abs(st["angvel"][b, 2] - 0.1) < 0.015  # the first impulse is torque / inertia x dt
    o.step(180)
    st = o.bodies()
    q = st["quat"][b]
    assert 0.35 < _twist(q) < 0.43, _twist(q)  # upper stop holds against the motor
    assert np.hypot.reduce(st["pos"][b]) < 0.01  # the world hinge holds its pivot
    assert np.hypot(q[0], q[1]) < 0.002  # the other rotation axes stay locked
    slots = np.cumsum(np.asarray(sc.arrays().kind) != 2) - 1
    o.set_motor(int(slots[h.motor]), speed=-2, max_torque=1)
    o.step(180)
    lower = _twist(o.bodies()["quat"][b])
    assert -0.43 < lower < -0.35, lower  # lower stop holds
    with pytest.raises(ValueError):
        o.set_motor(int(slots[h.limit]), speed=1.0)


def test_released_hinge_leaves_the_rotor_free():
    sc, b, h, o = _rotor(True)
    o.step(30)
    slots = np.cumsum(np.asarray(sc.arrays().kind) != 2) - 1
    o.release_joints(slots[[*h.joints, h.limit, h.motor]])
    w0 = o.bodies()["angvel"][b].copy()
    o.step(60)
    st = o.bodies()
    assert np.allclose(st["angvel"][b], w0) and np.allclose(st["vel"][b], 0.0)  # nothing acts on it any more


def test_frames_are_measured_from_the_creation_pose():
    # the rotor created already turned by 0.3 rad: the stops sit at +-0.4 about that pose
    th = 0.3
    sc = AvbdScene3D(timeStep=1 / 60, iterations=20, gravity=0)
    b = sc.addBox([1, 1, 1], position=[0, 0, 0], rotation=[0, 0, math.sin(th / 2), math.cos(th / 2)])
    sc.addHinge(None, b, axisA=[0, 0, 1], axisB=[0, 0, 1], minAngle=-0.4, maxAngle=0.4,
                motor={"speed": 2, "maxTorque": 1})
    q, _ = _run(sc, 181)
    assert 0.35 < _twist(q[-1, b]) - th < 0.43
