"""Ray and sphere casts (raycast / sphereCast / raycastAll / sphereCastAll,
src/native/solver3D.js:244-251 over src/gpu/shapeQueries.wgsl) through the C ABI against the
float64 restatement in oracle/queries.py on the engine's own poses: the same body (except where
the two nearest distances are within 1e-4), distance within 1e-4 (|t| + 1), normal within 1e-3;
filters (group mask, membership, ignore list), maximum distance, queued commands applied first,
and the same answers for a world in a batch and in a server.
"""
import numpy as np
import pytest

import queries as Q
from avbd_gb300 import createSolverPipeline, workloads

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pipe():
    p = createSolverPipeline("gb300", device=0)
    yield p
    p.destroy()


def _casts(rng, n, extent):
    out = []
    for k in range(n):
        o = rng.uniform(-extent, extent, 3) + np.array([0.0, extent + 1.0, 0.0])
        target = rng.uniform(-extent, extent, 3) + np.array([0.0, 2.0, 0.0])
        d = target - o
        r = 0.0 if k % 2 == 0 else float(rng.uniform(0.05, 0.8))
        c = {"origin": o.tolist(), "direction": d.tolist(), "radius": r}
        if k % 7 == 3:
            c["maxDistance"] = float(rng.uniform(0.5, 6.0))
        out.append(c)
    return out


def _check(got, scene, st, casts, **filt):
    mism = 0
    for g, c in zip(got, casts):
        want = Q.cast(st, scene.shape, scene.size, scene.group, scene.mask, c["origin"], c["direction"],
                      radius=c["radius"], max_distance=c.get("maxDistance", 3e38), **filt)
        if want is None:
            assert g is None, (c, g)
            continue
        i, t, n, second = want
        assert g is not None, (c, want)
        assert abs(g["distance"] - t) <= 1e-4 * (abs(t) + 1), (c, g, want)
        if g["index"] != i:
            assert second - t < 1e-4, (c, g, want)
            continue
        if np.linalg.norm(np.asarray(g["normal"]) - np.asarray(n)) > 1e-3:
            mism += 1
    assert mism <= len(casts) // 100, mism


def test_casts_match_the_restatement(pipe):
    scene = workloads.mixed_pile(150, seed=77, extent=4.0)
    w = pipe.createSolver(scene)
    w.step(45)
    st = w.readBodyState()
    rng = np.random.default_rng(3)
    casts = _casts(rng, 400, 5.0)
    got = w.sphereCastAll(casts)
    assert sum(g is not None for g in got) > 200
    _check(got, scene, st, casts)
    # the single-query forms
    c = casts[1]
    one = w.sphereCast(c["origin"], c["radius"], c["direction"])
    assert one == got[1]
    ray = w.raycast(casts[0]["origin"], casts[0]["direction"])
    assert ray == got[0]
    # filters
    scene.group = np.where(np.arange(scene.n_bodies) % 3 == 0, 1, 2).astype(np.uint32)
    scene.mask = np.where(np.arange(scene.n_bodies) % 2 == 0, 4, 8).astype(np.uint32)
    w2 = pipe.createSolver(scene)
    w2.step(45)
    st2 = w2.readBodyState()
    sub = casts[:120]
    _check(w2.sphereCastAll(sub, {"collidesWith": 2}), scene, st2, sub, collides_with=2)
    _check(w2.sphereCastAll(sub, {"membership": 8}), scene, st2, sub, membership=8)
    ign = [int(g["index"]) for g in w2.sphereCastAll(sub[:16]) if g is not None][:16]
    _check(w2.sphereCastAll(sub, {"ignore": ign}), scene, st2, sub, ignore=tuple(ign))
    assert all(g is None for g in w2.sphereCastAll(sub[:10], {"membership": 0}))
    with pytest.raises(ValueError):
        w2.sphereCastAll(sub[:1], {"ignore": list(range(17))})
    w.destroy()
    w2.destroy()


def test_casts_see_queued_commands_and_agree_across_apis(pipe):
    scenes = [workloads.mixed_pile(80, seed=1, extent=4.0), workloads.mixed_pile(120, seed=2, extent=4.0)]
    w = pipe.createSolver(scenes[1])
    w.step(20)
    w.editBodies([{"body": 5, "position": [0.0, 50.0, 0.0]}])  # queued: applied before the cast
    hit = w.raycast([0.0, 60.0, 0.0], [0.0, -1.0, 0.0])
    assert hit is not None and hit["index"] == 5
    casts = _casts(np.random.default_rng(9), 100, 5.0)
    ref = w.sphereCastAll(casts)
    w.destroy()
    batch = pipe.createBatch(scenes)
    batch.step(20)
    batch.editBodies(1, [{"body": 5, "position": [0.0, 50.0, 0.0]}])
    assert batch.sphereCastAll(1, [{"origin": [0.0, 60.0, 0.0], "direction": [0.0, -1.0, 0.0]}])[0]["index"] == 5
    assert batch.sphereCastAll(1, casts) == ref
    batch.destroy()
    server = pipe.createServer(budgetBytes=2 << 30)
    ids = [server.admit(sc) for sc in scenes]
    for i in ids:
        server.advance(i, 20)
    for _ in range(20):
        server.tick()
    server.editBodies(ids[1], [{"body": 5, "position": [0.0, 50.0, 0.0]}])
    server.sphereCastAll(ids[1], casts[:1])
    assert server.sphereCastAll(ids[1], casts) == ref
    server.destroy()
