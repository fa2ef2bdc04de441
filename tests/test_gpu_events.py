"""Contact begin/end events (watchContacts / readContactEvents / resetContactHistory,
src/native/solver3D.js:256-310 over src/vendor/three-avbd-lib/contacts.ts) through the C ABI.

Step by step the engine's events equal the restatement of the reference's ContactWatch in
oracle/contact_events.py, computed from the engine's own exported states before and after the
step: the same begins and ends (kind, bodies, step) exactly, points, impulses and normals within
1e-5 relative; across a change of the watched bodies and a history reset. Capacity overflow
reports dropped events; a world's events are the same alone, batched and served across eviction.
"""
import numpy as np
import pytest

import contact_events as CE
import oracle as O
from avbd_gb300 import createSolverPipeline, workloads

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pipe():
    p = createSolverPipeline("gb300", device=0)
    yield p
    p.destroy()


def _scene(n=150, seed=21):
    sc = workloads.mixed_pile(n, seed=seed, extent=4.0)
    rng = np.random.default_rng(seed)
    sc.restitution = np.where(rng.random(sc.n_bodies) < 0.5, 0.7, 0.0)  # bouncing: contacts come and go
    return sc


def _records(raw):
    """(kind, a, b, step) tuples and float payloads of an (n, 12) record array."""
    r = raw["records"]
    f = r.view(np.float32)
    keys = [tuple(int(x) for x in row[:4]) for row in r]
    return keys, f[:, 4:7].astype(np.float64), f[:, 7].astype(np.float64), f[:, 8:11].astype(np.float64)


def _close(x, y, tol=1e-5):
    x, y = np.asarray(x, dtype=np.float64), np.asarray(y, dtype=np.float64)
    return np.all(np.abs(x - y) <= tol * (np.abs(y) + 1.0))


def test_events_match_the_reference_restatement_step_by_step(pipe):
    sc = _scene()
    n = sc.n_bodies
    w = pipe.createSolver(sc)
    w.step(20)
    watch = np.zeros(n, dtype=np.int64)  # the host's copy of the watch words
    prev_watch = watch.copy()
    prev_set = set()
    w.watchContacts({"maxEvents": 100000})
    watch[:] = 1
    counts = {1: 0, 2: 0}
    for k in range(60):
        step = 20 + k + 1
        if k == 25:  # watch only the first half of the bodies: the others' pairs start over
            sel = list(range(n // 2))
            w.watchContacts({"indices": sel})
            watch = (watch & ~1) | np.isin(np.arange(n), sel).astype(np.int64)
        if k == 40:  # new lifetimes for a few bodies: their contacts begin again
            ids = np.array([3, 7, 11, 40], dtype=np.uint32)
            w.resetContactHistory(ids)
            watch[ids] += 2
        before = w.exportState()
        o_prev = O.OracleWorld(sc, fp64=False, app=True, colored=True)
        o_prev.import_state(before)
        w.step(1)
        after = w.exportState()
        want, now = CE.step_events(prev_set, prev_watch, after, watch, step, sc.params.dt,
                                   lambda a, b: o_prev.collide(a, b)["basis"][0])
        prev_set, prev_watch = now, watch.copy()
        got = w.readContactEventsRaw()
        assert got["dropped"] == 0 and not got["full"]
        keys, point, impulse, normal = _records(got)
        assert keys == [(e[0], e[1], e[2], e[3]) for e in want], step
        for i, e in enumerate(want):
            counts[e[0]] += 1
            if e[0] == CE.BEGIN:
                assert _close(point[i], e[4]) and _close(impulse[i], e[5]) and _close(normal[i], e[6]), (step, e)
    assert counts[1] > 20 and counts[2] > 20  # contacts both began and ended
    w.destroy()


def test_first_read_and_capacity(pipe):
    sc = _scene(80, seed=5)
    w = pipe.createSolver(sc)
    w.step(40)
    ev = w.readContactEvents()  # turns events on: nothing yet
    assert ev["events"] == [] and ev["dropped"] == 0
    w.step(1)
    ev = w.readContactEvents()
    assert ev["events"] and all(e["type"] == "begin" and e["step"] == 41 for e in ev["events"])
    assert all(e["a"] > e["b"] for e in ev["events"])
    w.destroy()
    w = pipe.createSolver(sc)
    w.watchContacts({"maxEvents": 5})
    w.step(41)
    ev = w.readContactEvents()
    assert len(ev["events"]) == 5 and ev["dropped"] > 0 and ev["full"]
    assert w.readContactEvents()["dropped"] == 0  # cleared by the read
    with pytest.raises(ValueError):
        w.watchContacts({"maxEvents": 0})
    with pytest.raises(ValueError):
        w.resetContactHistory(np.array([5, 3], dtype=np.uint32))
    w.destroy()


def test_events_alone_batched_and_served(pipe):
    scenes = [_scene(60, seed=1), _scene(120, seed=2), _scene(90, seed=3)]

    def run_alone():
        w = pipe.createSolver(scenes[1])
        w.watchContacts()
        w.step(30)
        a = w.readContactEventsRaw()["records"]
        w.step(30)
        b = w.readContactEventsRaw()["records"]
        w.destroy()
        return np.concatenate([a, b])

    ref = run_alone()
    assert len(ref) > 10
    batch = pipe.createBatch(scenes)
    batch.watchContacts(1)
    batch.step(60)
    assert np.array_equal(batch.readContactEventsRaw(1)["records"], ref)
    batch.destroy()
    server = pipe.createServer(budgetBytes=2 << 30)
    ids = [server.admit(sc) for sc in scenes]
    server.watchContacts(ids[1])
    for i in ids:
        server.advance(i, 30)
    for _ in range(30):
        server.tick()
    server.evict(ids[1])  # pending events wait on the host
    server.advance(ids[1], 30)
    for _ in range(30):
        server.tick()
    assert np.array_equal(server.readContactEventsRaw(ids[1])["records"], ref)
    server.destroy()
