"""Body commands (editBodies / flushEdits, src/native/runtime.js:46-167) through the C ABI: the
engine must apply the 12-word records exactly as the CPU world does (src/native/cpu/world.js:
229-300) — bit-exact against the float32 oracle over the next step, including teleports that drop
the warm start of the teleported bodies' contacts — and the same way for worlds, batches and
servers.
"""
import numpy as np
import pytest

import parity
from avbd_gb300 import createSolverPipeline, workloads
from avbd_gb300.pipeline import stage_edits

pytestmark = pytest.mark.gpu

KEYS = ("position", "rotation", "velocity", "angular", "prev_velocity")


@pytest.fixture(scope="module")
def pipe():
    p = createSolverPipeline("gb300", device=0)
    yield p
    p.destroy()


def _edits(scene, rng, n_edits=60):
    dyn = np.nonzero(scene.mass > 0)[0]
    out = []
    for _ in range(n_edits):
        b = int(rng.choice(dyn))
        kind = int(rng.integers(0, 8))
        v = rng.normal(size=3) * 3
        e = {"body": b}
        if kind == 0:
            e["linearVelocity"] = v
        elif kind == 1:
            e["angularVelocity"] = v
        elif kind == 2:
            e["impulse"] = v * scene.mass[b]
            if rng.random() < 0.5:
                e["worldPoint"] = scene.pos[b] + rng.normal(size=3) * 0.3
        elif kind == 3:
            e["force"] = v * scene.mass[b] * 60
            e["worldPoint"] = scene.pos[b] + rng.normal(size=3) * 0.3
        elif kind == 4:
            e["angularImpulse"] = v
        elif kind == 5:
            e["torque"] = v * 100
        elif kind == 6:
            e["position"] = scene.pos[b] + np.array([0.0, 0.05, 0.0])
            e["rotation"] = rng.normal(size=4)
        else:  # several fields in one record group
            e.update(linearVelocity=v, impulse=v, angularImpulse=-v)
        out.append(e)
    return out


@pytest.mark.parametrize("warm", [3, 40])
def test_edits_then_one_step_match_the_oracle(pipe, warm):
    scene = workloads.mixed_pile(300, seed=55 + warm, extent=4.0)
    w = pipe.createSolver(scene)
    rng = np.random.default_rng(warm)
    w.step(warm)
    rec = stage_edits(_edits(scene, rng), scene.n_bodies, float(scene.params.dt))
    rep = parity.compare_step(w, scene, 0, edits=rec)
    assert rep["pairs_equal"] and rep["contact_counts_equal"] and rep["colors_equal"], rep
    assert rep["max_err_fp32"] <= parity.TOL, rep
    w.destroy()


def test_edits_wait_for_the_step_and_agree_across_apis(pipe):
    scene = workloads.mixed_pile(200, seed=77, extent=4.0)
    edits = [{"body": 5, "linearVelocity": [0, 4, 0]}, {"body": 9, "position": [0, 30, 0]},
             {"body": 5, "impulse": [1000, 0, 0], "worldPoint": [0, 5, 0]}, {"body": 12, "torque": [0, 500, 0]}]
    w = pipe.createSolver(scene)
    w.step(10)
    before = w.readBodyState()
    w.editBodies(edits)
    # a read applies the queued commands first (the reference's reads call flushEdits,
    # src/native/solver3D.js:223-227, src/native/cpu/world.js:566-575)
    after = w.readBodyState()
    assert not np.array_equal(after["velocity"][5], before["velocity"][5])
    assert after["position"][9][1] == 30.0
    w.flushEdits()  # nothing left to apply
    assert np.array_equal(w.readBodyState()["velocity"], after["velocity"])
    w.step(5)
    ref = w.readBodyState()
    w.destroy()
    batch = pipe.createBatch([workloads.mixed_pile(50, seed=1, extent=4.0), scene])
    batch.step(10)
    batch.editBodies(1, edits)
    batch.step(5)
    got = batch.readBodyState(1)
    for k in KEYS:
        assert np.array_equal(got[k], ref[k]), k
    batch.destroy()
    server = pipe.createServer(budgetBytes=2 << 30)
    wid = server.admit(scene)
    server.advance(wid, 10)
    for _ in range(10):
        server.tick()
    server.editBodies(wid, edits)
    server.evict(wid)  # edits wait across eviction
    server.advance(wid, 5)
    for _ in range(5):
        server.tick()
    got = server.readBodyState(wid)
    for k in KEYS:
        assert np.array_equal(got[k], ref[k]), k
    server.destroy()
