"""Hinge motors and angle limits on the engine (angular rows, src/gpu/angularConstraints.js):
the reference's own hinge check through the public API, step parity with the float oracle (the
engine's rows and the oracle's share every operation, so the steps agree bit for bit) before and
after setMotor and releaseJoints, batches, the joint record layout and the argument errors."""
import math

import numpy as np
import pytest

import oracle as O
import parity
from avbd_gb300 import AvbdScene3D, createSolverPipeline
from avbd_gb300._lib import AvbdError, lib

pytestmark = pytest.mark.gpu

KEYS = ("position", "rotation", "velocity", "angular", "prev_velocity")


@pytest.fixture(scope="module")
def pipe():
    p = createSolverPipeline("gb300", device=0)
    yield p
    p.destroy()


def _twist(q):
    return 2.0 * math.atan2(float(q[2]), float(q[3]))


def _rotor(**hinge):
    # tests/gpu-package-features.js:518-589: a unit box on a world hinge about z, stops at +-0.4,
    # a motor at 2 rad/s with 1 N m, no gravity, 20 iterations
    sc = AvbdScene3D(timeStep=1 / 60, iterations=20, gravity=0)
    b = sc.addBox([1, 1, 1], position=[0, 0, 0])
    opts = dict(axisA=[0, 0, 1], axisB=[0, 0, 1], minAngle=-0.4, maxAngle=0.4, motor={"speed": 2, "maxTorque": 1})
    opts.update(hinge)
    h = sc.addHinge(None, b, **opts)
    return sc, b, h


def test_reference_hinge_check(pipe):
    sc, b, h = _rotor()
    w = pipe.createSolver(sc)
    w.step(1)
    assert abs(w.readBodyState()["angular"][b, 2] - 0.1) < 0.015  # first impulse: torque / inertia x dt
    w.step(180)
    st = w.readBodyState()
    q = st["rotation"][b]
    assert 0.35 < _twist(q) < 0.43, _twist(q)  # the upper stop holds against the motor
    assert np.hypot.reduce(st["position"][b]) < 0.01  # the world hinge holds its pivot
    assert np.hypot(q[0], q[1]) < 0.002  # the other rotation axes stay locked
    w.setMotor(h.motor, speed=-2, maxTorque=1)
    w.step(180)
    assert -0.43 < _twist(w.readBodyState()["rotation"][b]) < -0.35  # the lower stop holds
    rows = [*h.joints, h.limit, h.motor]
    w.releaseJoints(rows)
    rec = w.readJoints().reshape(-1, 32)
    assert np.all(rec[rows, 3] == 0)  # all hinge rows released
    w.destroy()


def _door_scene():
    # Y up: a trapdoor on a post swinging down onto its lower stop with boxes dropped on it, a
    # wheel driven by a motor on a body-body hinge (its hub welded to the world), a spinning box
    # under a world motor with a zero torque bound, and a loose pile beside them
    rng = np.random.default_rng(5)
    sc = AvbdScene3D(timeStep=1 / 60, iterations=10, gravity=-10)
    sc.addBox([30, 1, 30], density=0, position=[0, -0.5, 0])
    for k in range(40):
        p = [rng.uniform(-3, 3), rng.uniform(0.5, 6), rng.uniform(-3, 3)]
        if k % 3 == 0:
            sc.addSphere(rng.uniform(0.25, 0.5), position=p)
        else:
            sc.addBox(list(rng.uniform(0.4, 1.0, 3)), position=p)
    post = sc.addBox([0.3, 3.0, 0.3], density=0, position=[4.0, 1.5, 0])
    door = sc.addBox([2.0, 0.1, 1.0], position=[5.1, 3.0, 0])
    d = sc.addHinge(post, door, anchorA=[0.2, 1.5, 0], anchorB=[-1.05, 0, 0], axisA=[0, 0, 1], axisB=[0, 0, 1],
                    span=0.8, minAngle=-0.6, maxAngle=0.3)
    for k in range(3):
        sc.addBox([0.4, 0.4, 0.4], position=[5.0 + 0.5 * k, 4.0 + k, 0.1 * k])
    hub = sc.addBox([0.4, 0.4, 0.4], position=[-4.0, 2.0, 0])
    wheel = sc.addBox([1.2, 1.2, 0.2], position=[-4.0, 2.0, 0.5])
    sc.addJoint(None, hub, anchorA=[-4.0, 2.0, 0], anchorB=[0, 0, 0], angularStiffness=math.inf)
    m = sc.addHinge(hub, wheel, anchorA=[0, 0, 0.25], anchorB=[0, 0, -0.15], axisA=[0, 0, 1], axisB=[0, 0, 1],
                    span=0.3, motor={"speed": 3.0, "maxTorque": 20.0})
    spinner = sc.addBox([0.5, 0.5, 0.5], position=[0, 0.25, -6.0], angularVelocity=[0, 1.5, 0])
    z = sc.addMotor(None, spinner, axisA=[0, 1, 0], axisB=[0, 1, 0], speed=1.0, maxTorque=0.0)
    return sc, d, m, z


@pytest.mark.parametrize("warm", [0, 1, 25, 90])
def test_step_parity_with_the_oracle(pipe, warm):
    sc, *_ = _door_scene()
    arr = sc.arrays()
    w = pipe.createSolver(sc)
    rep = parity.compare_step(w, arr, warm)
    assert rep["pairs_equal"] and rep["contact_counts_equal"] and rep["colors_equal"], rep
    assert rep["coloring_valid"] and rep["max_err_fp32"] <= parity.TOL, rep
    w.destroy()


def test_trajectory_bits_equal_the_oracle(pipe):
    sc, b, h = _rotor()
    arr = sc.arrays()
    w = pipe.createSolver(sc)
    o = O.OracleWorld(arr, fp64=False, app=True, colored=True)
    for _ in range(40):
        w.step(1)
        o.step(1)
        g, c = w.readBodyState(), o.bodies()
        assert np.array_equal(g["position"].astype(np.float64), c["pos"])
        assert np.array_equal(g["rotation"].astype(np.float64), c["quat"])
        assert np.array_equal(g["angular"].astype(np.float64), c["angvel"])
    w.destroy()


def test_set_motor_and_release_keep_parity(pipe):
    sc, d, m, z = _door_scene()
    arr = sc.arrays()
    w = pipe.createSolver(sc)
    w.step(20)
    w.setMotor(m.motor, speed=-1.5)
    w.setMotor(z, maxTorque=5.0)
    arr.p0[m.motor] = -1.5
    arr.p1[z] = 5.0
    rep = parity.compare_step(w, arr, 15)
    assert rep["pairs_equal"] and rep["max_err_fp32"] <= parity.TOL, rep
    w.releaseJoints([d.limit, *m.joints])
    rep = parity.compare_step(w, arr, 0)
    assert rep["max_err_fp32"] <= parity.TOL, rep
    rep = parity.compare_step(w, arr, 10)
    assert rep["pairs_equal"] and rep["max_err_fp32"] <= parity.TOL, rep
    w.destroy()


def test_batch_worlds_match_single_worlds(pipe):
    scenes = [_rotor()[0], _door_scene()[0], _rotor(minAngle=-1.0, maxAngle=0.2, motor=None)[0]]
    _, _, h = _rotor()
    ref = []
    for i, sc in enumerate(scenes):
        w = pipe.createSolver(sc)
        w.step(30)
        if i == 0:
            w.setMotor(h.motor, speed=-2)
        w.step(30)
        ref.append(w.readBodyState())
        w.destroy()
    batch = pipe.createBatch(scenes)
    batch.step(30)
    batch.setMotor(0, h.motor, speed=-2)
    batch.step(30)
    for i in range(len(scenes)):
        got = batch.readBodyState(i)
        for k in KEYS:
            assert np.array_equal(got[k], ref[i][k]), (i, k)
    batch.releaseJoints(0, [h.limit])
    assert batch.readJoints(0).reshape(-1, 32)[2, 3] == 0
    with pytest.raises(ValueError):
        batch.setMotor(2, 2, speed=1.0)  # world 2's constraint 2 is a limit
    batch.destroy()


def test_joint_records_of_angular_rows(pipe):
    sc, b, h = _rotor()
    w = pipe.createSolver(sc)
    w.step(3)
    rec = w.readJoints().reshape(-1, 32)
    lim, mot = rec[2], rec[3]
    assert lim[3] == 1 and mot[3] == 1
    assert np.allclose(lim[24:27], [0, 0, 1]) and np.allclose(lim[28:31], [0, 0, 1])
    assert np.isclose(lim[27], -0.4) and np.isclose(lim[31], 0.4)
    assert mot[27] == 2.0 and mot[31] == 1.0
    for r in (lim, mot):  # unit reference tangents orthogonal to the axes
        assert np.isclose(np.linalg.norm(r[16:19]), 1, atol=1e-6) and abs(r[18]) < 1e-6
        assert np.isclose(np.linalg.norm(r[20:23]), 1, atol=1e-6) and abs(r[22]) < 1e-6
    assert mot[0] >= 1.0 and mot[8] != 0.0  # the motor's row is live
    w.destroy()


def test_angular_argument_errors(pipe):
    sc, b, h = _rotor()
    w = pipe.createSolver(sc)
    with pytest.raises(ValueError):
        w.setMotor(h.limit, speed=1.0)
    with pytest.raises(ValueError):
        w.setMotor(h.motor, maxTorque=-1.0)
    with pytest.raises(ValueError):
        w.releaseJoints([99])
    with pytest.raises(AvbdError):  # the C ABI checks the slot's kind itself
        from avbd_gb300 import _lib as L
        L.check(lib().avbd_world_set_motor(w._h, 0, 1, 1.0, 0.0))
    with pytest.raises(AvbdError):
        L.check(lib().avbd_world_set_motor(w._h, 3, 2, 0.0, float("nan")))
    w.destroy()
    bad = _rotor()[0].arrays()
    bad.p0[2], bad.p1[2] = 0.5, 0.25  # limit stops out of order
    with pytest.raises(AvbdError):
        pipe.createSolver(bad)


def test_hinges_and_springs_survive_eviction(pipe):
    # a served world with motors, stops and tearable springs, evicted to host memory and restored
    # between its requests, steps to the same bits as the world stepped alone
    sc, d, m, z = _door_scene()
    a = sc.addBox([0.3, 0.3, 0.3], density=0, position=[-8, 4, 0])
    b = sc.addBox([0.5, 0.5, 0.5], position=[-8, 3, 0])
    sc.addSpring(a, b, stiffness=150.0, rest=1.0, breakForce=20.0)
    alone = pipe.createSolver(sc)
    alone.step(50)
    ref = alone.readBodyState()
    alone.destroy()
    server = pipe.createServer(budgetBytes=1 << 30)
    wid = server.admit(sc)
    other = server.admit(_rotor()[0])
    for chunk in (10, 15, 25):
        server.advance(wid, chunk)
        server.advance(other, chunk)
        for _ in range(chunk):
            server.tick()
        server.evict(wid)
    got = server.readBodyState(wid)
    for k in KEYS:
        assert np.array_equal(got[k], ref[k]), k
    server.destroy()


def test_motor_change_wakes_a_sleeping_hinge(pipe):
    # a rotor held by a motor at rest falls asleep; setMotor wakes the world and it turns
    sc, b, h = _rotor(minAngle=None, maxAngle=None, motor={"speed": 0.0, "maxTorque": 5.0})
    w = pipe.createSolver(sc, {"sleeping": True})
    w.step(90)
    assert w.readSleepState()[0][b]
    w.setMotor(h.motor, speed=1.0)
    assert not w.readSleepState()[0][b]
    w.step(30)
    assert w.readBodyState()["angular"][b, 2] > 0.5
    w.destroy()
