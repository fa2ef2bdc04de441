"""Engine against the oracle at the benchmark configurations' own sizes (needs a GPU).

One-step parity (parity.compare_step: the engine's state after the warm-up steps loaded into the
oracle, one step on both, in the engine's colour order) on
* the full joint-heavy scene (75,538 bodies, 130,562 ball joints, 15 iterations) after 40 steps,
  when the cloth drapes over the sphere and the ball hits the wall;
* the largest world of the 4,096-world mix (8,192 bodies) and two worlds of the median size;
* a 16,384-body slice of the 1 M-body mixed pile on the tree broadphase.
Bit-exact: the candidate pair set, the contacts of every pair, the colours and their validity.
Float: poses and velocities within |gpu - cpu| <= 1e-5 (|cpu| + 1) of the float32 oracle. The
float64 errors (same colour order, and the reference's sequential order) are reported.

Over 300 steps, which are chaotic, the engine's run is compared with the float64 oracle's run of
the same steps in the reference's sequential order through size-independent quantities
(parity.stability_metrics): stack height, penetration into the ground and the sphere, and
kinetic energy, each within the tolerance written beside it.
"""
import numpy as np
import pytest

import oracle as O
import parity
from avbd_gb300 import createSolverPipeline, workloads

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pipe():
    p = createSolverPipeline("gb300", device=0)
    yield p
    p.destroy()


def _check(rep):
    assert rep["pairs_equal"], rep
    assert rep["contact_counts_equal"], rep
    assert rep["colors_equal"], rep
    assert rep["coloring_valid"], rep
    assert rep["max_err_fp32"] <= parity.TOL, rep
    assert np.isfinite(rep["max_err_fp64"]) and np.isfinite(rep["max_err_fp64_sequential"]), rep


def test_joint_heavy_scene_full_size_one_step(pipe):
    scene = workloads.cloth_wall()
    assert scene.n_bodies == 75_539 and scene.n_cons == 130_562
    w = pipe.createSolver(scene)
    rep = parity.compare_step(w, scene, 40)
    print(rep)
    _check(rep)
    assert rep["colors"] >= 4 and rep["contacts"] > 100_000
    w.destroy()


def test_world_mix_largest_and_median_worlds_one_step(pipe):
    counts, _ = workloads.world_counts()
    order = np.argsort(counts, kind="stable")
    picks = [int(np.argmax(counts)), int(order[len(order) // 2]), int(order[len(order) // 2 + 1])]
    assert counts[picks[0]] == 8192 and 200 <= counts[picks[1]] <= 320 and 200 <= counts[picks[2]] <= 320
    for i in picks:
        scene = workloads.world_mix_world(i)
        w = pipe.createSolver(scene)
        rep = parity.compare_step(w, scene, 30)
        print(i, int(counts[i]), rep)
        _check(rep)
        w.destroy()


def test_mixed_pile_slice_on_the_tree_one_step(pipe):
    scene = workloads.mixed_pile(16_384, seed=0xA5BD0001)
    scene.params.broadphase = "hploc"
    w = pipe.createSolver(scene)
    rep = parity.compare_step(w, scene, 90)
    print(rep)
    _check(rep)
    assert rep["contacts"] > 1000
    w.destroy()


def _state(world):
    s = world.readBodyState()
    return s["position"], s["rotation"], s["velocity"], s["angular"]


def _oracle_run(scene, steps):
    o = O.OracleWorld(scene, fp64=True, app=True, colored=False)
    o.step(steps)
    b = o.bodies()
    return b["pos"], b["quat"], b["vel"], b["angvel"]


def test_box_pile_300_steps_against_the_fp64_oracle(pipe):
    """Config 0 for its full 300 steps. Measured (float64 oracle, sequential order vs colour
    order vs float32 colour order, i.e. the engine): top 9.3962 / 9.3967 / 9.3969 m, mean height
    4.9392 / 4.9401 / 4.9399 m, ground penetration 13.7 / 12.1 / 12.4 mm, kinetic energy
    45.1 / 48.9 / 43.4 J."""
    scene = workloads.box_pile_c0()
    w = pipe.createSolver(scene)
    w.step(300)
    g = parity.stability_metrics(scene, *_state(w))
    w.destroy()
    c = parity.stability_metrics(scene, *_oracle_run(scene, 300))
    print("engine", g, "fp64 oracle", c)
    assert abs(g["top"] - c["top"]) <= 0.02           # stack height within 2 cm
    assert abs(g["mean_y"] - c["mean_y"]) <= 0.01     # mean height within 1 cm
    assert g["ground_pen"] <= 0.03 and abs(g["ground_pen"] - c["ground_pen"]) <= 0.01  # 3 cm bound, 1 cm apart
    assert abs(g["ke"] - c["ke"]) <= 0.35 * c["ke"] + 5.0  # kinetic energy within 35 % + 5 J


def test_joint_heavy_scene_300_steps_against_the_fp64_oracle(pipe):
    """Config 2's scene at reduced size (a 48 x 48 cloth, a 20 x 2 x 10 wall; the float64 oracle
    needs ~80 s for the 300 steps) for its full 300 steps; the cloth drapes over the sphere and
    the ball breaks through the wall. The 2 m ball then rolls on at 20-35 m/s and, after about
    2.5 s, sinks through the ground box, in the float64 oracle's sequential order as in the
    engine (the algorithm's single warm-started sphere contact), so the ground penetration is
    taken over the cloth and the bricks. Measured (float64 sequential vs the engine's float32
    colour order): top 10.4835 / 10.4835 m, mean height 8.4837 / 8.4842 m, sphere penetration
    110 / 109 mm, ground penetration 64 / 118 mm (bricks driven into the ground by the ball),
    kinetic energy 21.57 / 21.51 MJ (the ball)."""
    scene = workloads.cloth_wall(grid=48, wall=(20, 2, 10))
    sphere = ((0.0, 5.0, 0.0), 5.0)
    w = pipe.createSolver(scene)
    w.step(300)
    g = parity.stability_metrics(scene, *_state(w), sphere=sphere, footprint=150.0, max_radius=1.0)
    w.destroy()
    c = parity.stability_metrics(scene, *_oracle_run(scene, 300), sphere=sphere, footprint=150.0, max_radius=1.0)
    print("engine", g, "fp64 oracle", c)
    assert abs(g["top"] - c["top"]) <= 0.05
    assert abs(g["mean_y"] - c["mean_y"]) <= 0.05
    assert g["sphere_pen"] <= 0.2 and abs(g["sphere_pen"] - c["sphere_pen"]) <= 0.02
    assert g["ground_pen"] <= 0.2 and abs(g["ground_pen"] - c["ground_pen"]) <= 0.1
    assert abs(g["ke"] - c["ke"]) <= 0.05 * c["ke"]   # within 5 %


def test_joint_heavy_scene_full_size_300_steps_stable(pipe):
    """The full config 2 for its 300 steps on the engine alone (the oracle would need ~40 min):
    finite, the cloth on the sphere within 0.2 m, no cloth box or brick through the ground, no
    colouring conflict."""
    scene = workloads.cloth_wall()
    w = pipe.createSolver(scene)
    w.step(300)
    pos, quat, vel, ang = _state(w)
    assert np.isfinite(pos).all() and np.isfinite(quat).all() and np.isfinite(vel).all()
    m = parity.stability_metrics(scene, pos, quat, vel, ang, sphere=((0.0, 5.0, 0.0), 5.0), footprint=150.0,
                                 max_radius=1.0)
    print(m)
    assert m["sphere_pen"] <= 0.2 and m["ground_pen"] <= 0.2
    c = w.readCounters()
    assert c["conflicts"] == 0
    w.destroy()
