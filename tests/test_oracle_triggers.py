"""Trigger bodies on the oracle (cpuPhysics3D.js:148-156, sleeping.js:54, restitution.js:68,
queries.js:229-233, world.js:757-762): a trigger's contacts apply no forces and no bounce, a
constraint on a trigger body links no sleeping island, casts skip triggers on request and
events report no impulse for them."""
import numpy as np

import oracle as O
import contact_events as CE
import queries as Q
from avbd_gb300 import AvbdScene3D


def _world(sc, fp64=True):
    return O.OracleWorld(sc.arrays(), fp64=fp64, app=True, colored=True)


def test_triggers_apply_no_forces_and_no_bounce():
    sc = AvbdScene3D(timeStep=1 / 60, iterations=10, gravity=-10)
    sc.addBox([20, 1, 20], density=0, position=[0, -0.5, 0])
    slab = sc.addBox([4, 0.4, 4], density=0, position=[0, 2, 0], isTrigger=True)
    box = sc.addBox([1, 1, 1], position=[0, 4, 0])
    ball = sc.addSphere(0.4, position=[1, 4, 1], restitution=0.9)
    ghost = sc.addBox([1, 1, 1], position=[5, 1, 0], isTrigger=True)
    o = _world(sc)
    vmin = 0.0
    grounded = False
    for _ in range(90):
        o.step(1)
        b = o.bodies()
        grounded |= b["pos"][ball, 1] < 0.45
        if not grounded:  # until it reaches the ground (radius 0.4) it only falls: no bounce off the slab
            assert b["vel"][ball, 1] <= 1e-9
        vmin = min(vmin, b["vel"][box, 1])
    assert grounded
    b = o.bodies()
    assert abs(b["pos"][box, 1] - 0.49) < 0.02  # through the slab, resting on the ground
    assert b["pos"][ghost, 1] < -5  # a dynamic trigger falls through the ground
    assert vmin < -6  # the box fell freely through the slab (v = g t past 2 m)
    assert o.counts()["manifolds"] >= 1 and slab == 1


def test_a_joint_to_a_trigger_anchor_gives_no_support():
    def run(trigger):
        sc = AvbdScene3D(timeStep=1 / 60, iterations=10, gravity=0)
        anchor = sc.addBox([0.2, 0.2, 0.2], density=0, position=[0, 3, 0], isTrigger=trigger)
        body = sc.addBox([1, 1, 1], position=[0, 2, 0])
        sc.addJoint(anchor, body, anchorA=[0, 0, 0], anchorB=[0, 1, 0])
        arr = sc.arrays()
        arr.params.sleeping = True
        o = O.OracleWorld(arr, fp64=True, app=True, colored=True)
        o.step(60)
        return o.sleep_state()[0][body]
    assert run(False)  # the static anchor supports the island: it sleeps
    assert not run(True)  # a trigger anchor links nothing: unsupported, it stays awake


def test_restated_casts_and_events_honour_triggers():
    st = {"position": np.array([[0.0, 0.0, 0.0], [0.0, 2.0, 0.0]]),
          "rotation": np.array([[0.0, 0.0, 0.0, 1.0]] * 2)}
    shape, size = [0, 0], np.array([[4.0, 1.0, 4.0], [1.0, 1.0, 1.0]])
    group = mask = [0xFFFFFFFF] * 2
    trig = [False, True]
    hit = Q.cast(st, shape, size, group, mask, [0, 8, 0], [0, -1, 0], triggers=trig)
    assert hit[0] == 1
    hit = Q.cast(st, shape, size, group, mask, [0, 8, 0], [0, -1, 0], triggers=trig, include_triggers=False)
    assert hit[0] == 0
    state = {"mpairs": np.array([[1, 0]]), "mcount": np.array([1]), "pos": st["position"],
             "quat": st["rotation"], "cra": np.array([[0.0, -0.5, 0.0]]), "clam": np.array([[-5.0, 0, 0]])}
    ev, _ = CE.step_events(set(), [1, 1], state, [1, 1], 1, 1 / 60, lambda a, b: [0, 1, 0], triggers=trig)
    assert ev[0][5] == 0.0
    ev, _ = CE.step_events(set(), [1, 1], state, [1, 1], 1, 1 / 60, lambda a, b: [0, 1, 0])
    assert ev[0][5] > 0
