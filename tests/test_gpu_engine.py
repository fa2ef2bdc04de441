"""CUDA engine parity and behaviour (needs a GPU).

Parity is checked one step at a time from the engine's own state (the reference GPU solver's
seedFrom, src/vendor/three-avbd-lib/solver3D.ts:942-979, in reverse): after some warm-up steps the engine's state is loaded into the oracle and both take
one step in the same colour order (parity.compare_step). Bit-exact: candidate pair sets,
contacts per pair, colours. Float: poses and velocities within 1e-5 relative
(|gpu - cpu| <= 1e-5 (|cpu| + 1)) of the float32 oracle.
"""
import numpy as np
import pytest

import parity
import ref_scenes
from avbd_gb300 import createSolverPipeline, workloads
from avbd_gb300.scene import SolverParams

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pipe():
    p = createSolverPipeline("gb300", device=0)
    yield p
    p.destroy()


def _check(rep, tol=parity.TOL):
    assert rep["pairs_equal"], rep
    assert rep["contact_counts_equal"], rep
    assert rep["colors_equal"], rep
    assert rep["coloring_valid"], rep
    assert rep["max_err_fp32"] <= tol, rep


@pytest.mark.parametrize("warm", [0, 1, 30, 90])
def test_box_pile_small_one_step(pipe, warm):
    scene = workloads.box_pile_c0(nx=4, ny=4, nz=4)
    w = pipe.createSolver(scene)
    _check(parity.compare_step(w, scene, warm))
    w.destroy()


def test_box_pile_c0_one_step(pipe):
    scene = workloads.box_pile_c0()
    w = pipe.createSolver(scene)
    rep = parity.compare_step(w, scene, 75)
    print(rep)
    _check(rep)
    w.destroy()


@pytest.mark.parametrize("warm", [5, 60])
def test_mixed_boxes_spheres_one_step(pipe, warm):
    scene = workloads.mixed_pile(400, seed=1234, extent=6.0)
    w = pipe.createSolver(scene)
    rep = parity.compare_step(w, scene, warm)
    print(rep)
    _check(rep)
    w.destroy()


def test_cloth_joints_one_step(pipe):
    scene = workloads.cloth_wall(grid=10, wall=(4, 2, 3))
    w = pipe.createSolver(scene)
    rep = parity.compare_step(w, scene, 40)
    print(rep)
    _check(rep)
    w.destroy()


def _app_params(sc):
    # reference scene (Z up, gravity -10) on the app path
    p = SolverParams(dt=1 / 60, gravity=-10.0, up=(0.0, 0.0, 1.0), iterations=10)
    sc.params = p
    return sc


@pytest.mark.parametrize("index", [2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13])
def test_reference_scenes_one_step(pipe, index):
    """Joints (hard, soft, angular rest frames), springs, ignore pairs, fracture."""
    scene = _app_params(ref_scenes.build(index))
    w = pipe.createSolver(scene)
    rep = parity.compare_step(w, scene, 45)
    print(ref_scenes.SCENES[index][0], rep)
    _check(rep)
    w.destroy()


def test_pair_capacity_regrowth_is_exact(pipe):
    """A dense sphere cluster overflows the initial pair capacity: the step is re-run after
    the buffers grow and still matches the oracle exactly."""
    rng = np.random.default_rng(7)
    from avbd_gb300.scene import SceneBuilder
    b = SceneBuilder(SolverParams(dt=1 / 60, gravity=-9.81, up=(0, 1, 0), iterations=4))
    b.rigid([40, 1, 40], 0, 0.5, [0, -0.5, 0])
    for _ in range(300):
        b.sphere(0.5, 1000, 0.5, list(rng.uniform([-2, 0.5, -2], [2, 4.5, 2])))
    scene = b.arrays()
    w = pipe.createSolver(scene)
    rep = parity.compare_step(w, scene, 0)
    assert w.readCounters()["overflow"] >= 1
    _check(rep)
    w.destroy()


def test_batch_matches_each_world_alone(pipe):
    """Worlds stepped in one batch evolve bit for bit as they do alone."""
    scenes = [workloads.mixed_pile(n, seed=100 + n, extent=5.0) for n in (16, 40, 90, 7, 160)]
    scenes.append(workloads.box_pile_c0(nx=3, ny=5, nz=2))
    scenes.append(workloads.cloth_wall(grid=6, wall=(3, 2, 2)))
    batch = pipe.createBatch(scenes)
    batch.step(25)
    for k, sc in enumerate(scenes):
        w = pipe.createSolver(sc)
        w.step(25)
        a, b = batch.readBodyState(k), w.readBodyState()
        for key in ("position", "rotation", "velocity", "angular"):
            assert np.array_equal(a[key], b[key]), (k, key)
        w.destroy()
    batch.destroy()


def test_box_pile_c0_300_steps_stable(pipe):
    """300 steps of config 0: finite, no cube below the ground by more than a few cm, the
    lattice ends up stacked (top layer within the lattice height), low kinetic energy."""
    scene = workloads.box_pile_c0()
    w = pipe.createSolver(scene)
    w.step(300)
    s = w.readBodyState()
    pos, vel = s["position"][1:], s["velocity"][1:]
    assert np.isfinite(pos).all() and np.isfinite(s["rotation"]).all()
    assert pos[:, 1].min() > 0.5 - 0.05, pos[:, 1].min()   # cube centre above ground top - margin
    assert pos[:, 1].max() < 0.55 + 9 * 1.05 + 0.1
    ke = 0.5 * 1000.0 * float((vel.astype(np.float64) ** 2).sum())
    assert ke / len(vel) < 50.0, ke
    c = w.readCounters()
    assert c["conflicts"] == 0 and c["colors"] <= 64
    w.destroy()


def test_read_selected_and_set_poses(pipe):
    scene = workloads.box_pile_c0(nx=2, ny=2, nz=2)
    w = pipe.createSolver(scene)
    rec = w.readSelectedBodies([1, 3])
    assert rec.shape == (80,)
    np.testing.assert_allclose(rec[0:3], scene.pos[1], rtol=0, atol=1e-6)
    assert rec[19] == np.float32(scene.mass[1]) and rec[39] == 0
    poses = w.readSelectedBodies([2], posesOnly=True)
    assert poses.shape == (8,)
    w.setPoses([1], [[0.0, 5.0, 0.0]], [[0, 0, 0, 2.0]])
    st = w.readBodyState()
    np.testing.assert_array_equal(st["position"][1], [0.0, 5.0, 0.0])
    np.testing.assert_array_equal(st["rotation"][1], [0, 0, 0, 1])
    w.setVelocities([1], linear=[[1.0, 2.0, 3.0]])
    assert np.array_equal(w.readBodyState()["velocity"][1], [1, 2, 3])
    with pytest.raises(ValueError):
        w.readSelectedBodies([99])
    w.destroy()


def test_free_fall_analytic(pipe):
    """A body with no contacts falls as y(t) = y0 + g t^2 / 2 up to the adaptive warm start
    (reference tests/gpu.js:148 checks 5 - 8/120^2 within 1e-5 for its setup)."""
    from avbd_gb300 import AvbdScene3D
    sc = AvbdScene3D(timeStep=1 / 60, iterations=10, gravity=-10)
    sc.addBox([1, 1, 1], position=[0, 5, 0])
    w = pipe.createSolver(sc)
    w.step(2)
    y = w.readBodyState()["position"][0, 1]
    # step 1: inertial target y0 - g dt^2, warm start weight 0 at rest; BDF1 with no constraints
    # lands exactly on the inertial target each step: y_n = y0 - g dt^2 (1 + 2 + ... + n)
    assert abs(y - (5 - 10 * (1 / 60) ** 2 * 3)) < 1e-5, y
    w.destroy()


def test_resting_contact_respects_the_floor_margin(pipe):
    """The reference's canonical check (tests/gpu-canonical.js:38-64): a unit box dropped from
    z = 4 onto a 100 x 100 x 1 floor rests after 240 steps with its centre at
    1 - COLLISION_MARGIN within 0.01, on at least four contacts."""
    from avbd_gb300 import AvbdScene3D
    sc = AvbdScene3D(timeStep=1 / 60, iterations=10, gravity=-10, up=[0, 0, 1])
    sc.addBox([100, 100, 1], density=0, friction=0.5, position=[0, 0, 0])
    box = sc.addBox([1, 1, 1], density=1, friction=0.5, position=[0, 0, 4])
    w = pipe.createSolver(sc)
    w.step(240)
    z = float(w.readBodyState()["position"][box][2])
    assert abs(z - (1 - 0.01)) < 0.01, z
    c = w.readCounters()
    assert c["contacts"] >= 4 and c["conflicts"] == 0
    w.destroy()
