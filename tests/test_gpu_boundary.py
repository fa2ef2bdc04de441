"""The rest of the native world surface (src/native/scenes.d.ts:317-454) through the C ABI:
readJoints (the reference's 32-float joint record), setFilters (new collision filters take effect
at the next step, bit-exact against the oracle built with the same filters), and a hinge (two ball
joints, src/native/scenes.js:587-601) that lets its body turn about the hinge axis only.
"""
import numpy as np
import pytest

import parity
import ref_scenes
from avbd_gb300 import AvbdScene3D, createSolverPipeline, workloads
from avbd_gb300.scene import SolverParams

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pipe():
    p = createSolverPipeline("gb300", device=0)
    yield p
    p.destroy()


def test_read_joints_matches_the_exported_joint_state(pipe):
    sc = ref_scenes.build(13)  # breakable joints
    sc.params = SolverParams(dt=1 / 60, gravity=-10.0, up=(0.0, 0.0, 1.0), iterations=10)
    w = pipe.createSolver(sc)
    w.step(150)
    rec = w.readJoints().reshape(-1, 32)
    st = w.exportState()
    joints = sc.kind != 2
    assert rec.shape[0] == int(joints.sum())
    assert np.array_equal(rec[:, 0:3], st["jpen_lin"]) and np.array_equal(rec[:, 4:7], st["jpen_ang"])
    assert np.array_equal(rec[:, 8:11], st["jlam_lin"]) and np.array_equal(rec[:, 12:15], st["jlam_ang"])
    broken = st["jbroken"] != 0
    assert broken.any() and not broken.all()
    p0 = np.where(np.isinf(sc.p0[joints]), 3e38, sc.p0[joints]).astype(np.float32)
    assert np.all(rec[broken, 3] == 0) and np.array_equal(rec[~broken, 3], p0[~broken])
    assert np.allclose(rec[:, 24:27], sc.ra[joints]) and np.allclose(rec[:, 28:31], sc.rb[joints])
    w.destroy()


def test_set_filters_takes_effect_and_matches_the_oracle(pipe):
    sc = workloads.mixed_pile(300, seed=41, extent=4.0)
    w = pipe.createSolver(sc)
    w.step(40)
    pairs = w.readPairs()
    a, b = (int(x) for x in pairs[len(pairs) // 2])  # a touching pair: make them pass through
    groups = np.array([2, 4], dtype=np.uint32)
    w.setFilters([a, b], groups, np.array([0xFFFFFFFF & ~4, 0xFFFFFFFF & ~2], dtype=np.uint32))
    sc2 = workloads.mixed_pile(300, seed=41, extent=4.0)
    sc2.group[[a, b]] = groups
    sc2.mask[[a, b]] = [0xFFFFFFFF & ~4, 0xFFFFFFFF & ~2]
    rep = parity.compare_step(w, sc2, 0)
    assert rep["pairs_equal"] and rep["contact_counts_equal"] and rep["colors_equal"], rep
    assert rep["max_err_fp32"] <= parity.TOL, rep
    assert not any((int(p[0]), int(p[1])) == (a, b) for p in w.readPairs())
    w.destroy()


def test_hinge_turns_about_its_axis_only(pipe):
    sc = AvbdScene3D(timeStep=1 / 60, iterations=10, gravity=-10)
    post = sc.addBox([0.2, 0.2, 2.0], density=0, position=[0, 5, 0])
    door = sc.addBox([0.2, 2.0, 1.0], position=[0, 4, 0])
    # hinge along z through the post's centre and the door's top edge (jointed bodies do not
    # collide): the door swings in the x-y plane like a pendulum
    sc.addHinge(post, door, anchorA=[0, 0, 0], anchorB=[0, 1.0, 0], axisA=[0, 0, 1], axisB=[0, 0, 1], span=0.8)
    w = pipe.createSolver(sc)
    w.setVelocities([door], [[2.0, 0.0, 0.0]])
    for _ in range(60):
        w.step(1)
        q = w.readBodyState()["rotation"][door]
        assert abs(q[0]) < 2e-2 and abs(q[1]) < 2e-2  # rotation about z only
    assert abs(w.readBodyState()["rotation"][door][2]) > 0.05  # and it did swing
    w.destroy()


def test_spatial_sort_slots_and_parity(pipe):
    # createSolver(scene, {spatialSort: true}): bodies in Morton-ordered slots (statics first);
    # every call takes slots and gpuIndex maps creation indices to them
    sc = workloads.mixed_pile(400, seed=17, extent=5.0)
    w = pipe.createSolver(sc, {"spatialSort": True})
    st = w.readBodyState()
    for ref in (0, 5, 123, 399):
        assert np.array_equal(st["position"][w.gpuIndex(ref)], sc.pos[ref].astype(np.float32))
    from avbd_gb300.pipeline import spatial_sort
    sorted_scene = spatial_sort(sc)
    rep = parity.compare_step(w, sorted_scene, 30)
    assert rep["pairs_equal"] and rep["contact_counts_equal"] and rep["colors_equal"], rep
    assert rep["max_err_fp32"] <= parity.TOL, rep
    w.destroy()


def test_property_edits_apply_after_commands(pipe):
    # editBodies' property part (src/native/runtime.js:72-103,157-165): restitution turns the
    # bounce pass on for a world created without it; a group edit stops a pair colliding
    sc = AvbdScene3D(timeStep=1 / 60, iterations=10, gravity=-10)
    sc.addBox([20, 1, 20], position=[0, -0.5, 0], density=0)
    ball = sc.addSphere(0.5, position=[0, 0.6, 0])
    other = sc.addSphere(0.5, position=[3, 0.6, 0])
    w = pipe.createSolver(sc)
    w.editBodies([{"body": ball, "restitution": 0.8, "linearVelocity": [0, -6, 0]},
                  {"body": other, "group": 2, "collidesWith": 0}])
    vmax = 0.0
    for _ in range(6):
        w.step(1)
        vmax = max(vmax, float(w.readBodyState()["velocity"][ball][1]))
    assert vmax > 3.0  # bounced: about 0.8 x 6 m/s
    assert all(int(p[0]) != other and int(p[1]) != other for p in w.readPairs())  # falls through
    w.step(24)
    assert w.readBodyState()["position"][other][1] < 0.0
    with pytest.raises(ValueError):
        w.editBodies([{"body": ball, "restitution": 2.0}])
    w.destroy()


def test_body_handles_route_to_the_world_commands(pipe):
    # runtime.js:169-237: body(i) handles give the world's per-body commands on slot i
    from avbd_gb300 import AvbdScene3D
    sc = AvbdScene3D(timeStep=1 / 60, iterations=10, gravity=0)
    a = sc.addBox([1, 1, 1], position=[0, 0, 0])
    b = sc.addBox([1, 1, 1], position=[5, 0, 0])
    w = pipe.createSolver(sc)
    h = w.body(b)
    assert h.gpuIndex == b and h.setLinearVelocity([1, 0, 0]) is h
    h.setAngularVelocity([0, 2, 0]).setRestitution(0.5)
    w.step(1)
    st = h.readState()
    assert np.allclose(st["linearVelocity"], [1, 0, 0], atol=1e-3) and np.allclose(st["angularVelocity"], [0, 2, 0], atol=1e-3)
    assert np.allclose(w.body(a).readState()["linearVelocity"], 0)
    h.teleport([9, 0, 0])
    w.step(1)
    assert 9 - 1e-4 <= h.readState()["position"][0] <= 9 + 1 / 60 + 1e-4
    with pytest.raises(ValueError):
        w.body(5)
    w.destroy()


def test_read_body_state_of_one_body(pipe):
    # src/native/cpu/world.js:572-588: {position, rotation, linearVelocity, angularVelocity, mass,
    # effectiveMass, sleeping} of one body
    from avbd_gb300 import AvbdScene3D
    sc = AvbdScene3D(timeStep=1 / 60, iterations=10, gravity=0)
    b = sc.addBox([1, 2, 1], density=2, position=[1, 2, 3], velocity=[0.5, 0, 0])
    w = pipe.createSolver(sc)
    w.step(2)
    st = w.readBodyState(b)
    assert set(st) == {"position", "rotation", "linearVelocity", "angularVelocity", "mass", "effectiveMass",
                       "sleeping"}
    assert st["mass"] == 4.0 and st["effectiveMass"] == 4.0 and st["sleeping"] is False
    assert np.allclose(st["linearVelocity"], [0.5, 0, 0], atol=1e-4) and abs(st["position"][0] - (1 + 1 / 60)) < 1e-4
    with pytest.raises(ValueError):
        w.readBodyState(3)
    w.destroy()
