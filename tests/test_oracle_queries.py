"""The cast restatement (oracle/queries.py, after src/gpu/shapeQueries.wgsl) on known answers and
against an independent check: the first distance at which the swept sphere touches a rotated box
equals the root of (distance from the center to the box) = radius, found by bisection."""
import math

import numpy as np

import queries as Q


def _state(pos, quat):
    return {"position": np.array(pos, dtype=np.float64), "rotation": np.array(quat, dtype=np.float64)}


def test_known_answers():
    st = _state([[0, 0, 0], [10, 0, 0]], [[0, 0, 0, 1], [0, 0, 0, 1]])
    shape, size = [0, 1], np.array([[2, 2, 2], [2, 2, 2]])
    group = mask = [0xFFFFFFFF, 0xFFFFFFFF]
    i, t, n, _ = Q.cast(st, shape, size, group, mask, (-5, 0, 0), (1, 0, 0))
    assert i == 0 and abs(t - 4) < 1e-12 and np.allclose(n, (-1, 0, 0))
    i, t, n, _ = Q.cast(st, shape, size, group, mask, (-5, 0, 0), (2, 0, 0), radius=0.5)
    assert i == 0 and abs(t - 3.5) < 1e-12 and np.allclose(n, (-1, 0, 0))
    i, t, n, _ = Q.cast(st, shape, size, group, mask, (10, 5, 0), (0, -1, 0), radius=0.5)
    assert i == 1 and abs(t - 3.5) < 1e-12 and np.allclose(n, (0, 1, 0))
    i, t, n, _ = Q.cast(st, shape, size, group, mask, (0.2, 0.1, 0), (0, 0, 1))  # inside: t = 0, n = -d
    assert i == 0 and t == 0 and np.allclose(n, (0, 0, -1))
    assert Q.cast(st, shape, size, group, mask, (-5, 0, 0), (1, 0, 0), max_distance=3.9) is None
    assert Q.cast(st, shape, size, group, mask, (-5, 3, 0), (1, 0, 0)) is None
    # filters: the box ignored, masked by group, or by membership -> the sphere behind it
    assert Q.cast(st, shape, size, group, mask, (-5, 0, 0), (1, 0, 0), ignore=(0,))[0] == 1
    assert Q.cast(st, shape, size, [1, 2], mask, (-5, 0, 0), (1, 0, 0), collides_with=2)[0] == 1
    assert Q.cast(st, shape, size, group, [1, 2], (-5, 0, 0), (1, 0, 0), membership=2)[0] == 1
    assert Q.cast(st, shape, size, group, mask, (-5, 0, 0), (1, 0, 0), membership=0) is None
    # an edge of the rounded box: the normal points from the edge to the sphere's center
    i, t, n, _ = Q.cast(st, shape, size, group, mask, (-5, 1.2, 0), (1, 0, 0), radius=0.5)
    assert i == 0 and np.allclose(np.linalg.norm(n), 1) and n[0] < 0 and n[1] > 0


def _box_distance(p, h):
    q = np.abs(p) - h
    return np.linalg.norm(np.maximum(q, 0)) + min(max(q[0], q[1], q[2]), 0)


def test_sphere_sweeps_touch_rotated_boxes_where_the_distance_reaches_the_radius():
    rng = np.random.default_rng(7)
    checked = 0
    for _ in range(120):
        h = rng.uniform(0.2, 1.5, 3)
        q = rng.normal(size=4)
        q /= np.linalg.norm(q)
        pos = rng.uniform(-1, 1, 3)
        o = pos + rng.normal(size=3) * 4
        d = pos + rng.normal(size=3) * 0.5 - o
        d /= np.linalg.norm(d)
        r = float(rng.uniform(0, 0.6))
        st = _state([pos], [q])
        hit = Q.cast(st, [0], np.array([2 * h]), [1], [1], o, d, radius=r)
        inv = np.array([-q[0], -q[1], -q[2], q[3]])

        def dist(t):
            c = np.array(Q._turn(tuple(inv), tuple(o + t * d - pos)))
            return _box_distance(c, h) - r

        if dist(0.0) <= 0:
            assert hit is not None and hit[1] == 0
            continue
        ts = np.linspace(0, 12, 1201)
        vals = np.array([dist(t) for t in ts])
        below = np.nonzero(vals <= 0)[0]
        if not len(below):
            assert hit is None or dist(hit[1]) < 1e-6  # grazing contacts between samples
            continue
        k = below[0]
        lo, hi = ts[k - 1], ts[k]
        for _ in range(60):
            mid = 0.5 * (lo + hi)
            lo, hi = (lo, mid) if dist(mid) <= 0 else (mid, hi)
        assert hit is not None and abs(hit[1] - hi) < 1e-6, (hit, hi)
        checked += 1
    assert checked > 40
