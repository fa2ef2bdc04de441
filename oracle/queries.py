"""AVBD CPU ORACLE -- test infrastructure only.

Ray and sphere casts restated from the reference GPU backend's shape queries
(src/gpu/shapeQueries.wgsl: raySphere, rayCapsule, roundedPoly for boxes, trace, ignored,
nearest/owner/finish; host side src/gpu/shapeQueries.js:97-259), in float64 on a world's poses:
the nearest hit per query over every body that passes the filter, ties to the lowest index.
"""
from __future__ import annotations

import math

MISS = (-1.0, (0.0, 0.0, 0.0))


def _sub(a, b):
    return (a[0] - b[0], a[1] - b[1], a[2] - b[2])


def _add(a, b):
    return (a[0] + b[0], a[1] + b[1], a[2] + b[2])


def _mul(a, s):
    return (a[0] * s, a[1] * s, a[2] * s)


def _dot(a, b):
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]


def _cross(a, b):
    return (a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0])


def _neg(a):
    return (-a[0], -a[1], -a[2])


def _turn(q, v):
    u = (q[0], q[1], q[2])
    t = _mul(_cross(u, v), 2.0)
    return _add(_add(v, _mul(t, q[3])), _cross(u, t))


def _closest(a, b, p):
    e = _sub(b, a)
    s = min(1.0, max(0.0, _dot(_sub(p, a), e) / max(_dot(e, e), 1e-20)))
    return _add(a, _mul(e, s))


def ray_sphere(o, d, c, r):
    v = _sub(o, c)
    b = _dot(v, d)
    disc = b * b - _dot(v, v) + r * r
    if disc < 0:
        return MISS
    t = -b - math.sqrt(disc)
    if t < 0:
        return MISS
    p = _sub(_add(o, _mul(d, t)), c)
    ln = math.sqrt(_dot(p, p))
    return (t, _mul(p, 1.0 / max(ln, 1e-20)) if ln > 1e-10 else _neg(d))


def ray_capsule(o, d, a, b, r):
    ba, oa = _sub(b, a), _sub(o, a)
    bb = _dot(ba, ba)
    if bb < 1e-16:
        return ray_sphere(o, d, a, r)
    bd, bo, od = _dot(ba, d), _dot(ba, oa), _dot(oa, d)
    A = bb - bd * bd
    B = bb * od - bo * bd
    Cc = bb * _dot(oa, oa) - bo * bo - r * r * bb
    hit = MISS
    disc = B * B - A * Cc
    if A > 1e-12 * bb and disc >= 0:
        t = (-B - math.sqrt(disc)) / A
        y = bo + t * bd
        if t >= 0 and 0 <= y <= bb:
            q = _sub(_add(o, _mul(d, t)), _add(a, _mul(ba, y / bb)))
            hit = (t, _mul(q, 1.0 / math.sqrt(_dot(q, q))))
    for c in (a, b):
        h = ray_sphere(o, d, c, r)
        if h[0] >= 0 and (hit[0] < 0 or h[0] < hit[0]):
            hit = h
    return hit


def _corner(v, h):
    return (h[0] if v & 1 else -h[0], h[1] if v & 2 else -h[1], h[2] if v & 4 else -h[2])


# the box's faces: outward normal, offset axis, corners (shapeQueries.wgsl FACE_VERTS order)
_FACES = [((1.0, 0.0, 0.0), 0, (1, 3, 7, 5)), ((-1.0, 0.0, 0.0), 0, (0, 2, 6, 4)),
          ((0.0, 1.0, 0.0), 1, (2, 3, 7, 6)), ((0.0, -1.0, 0.0), 1, (0, 1, 5, 4)),
          ((0.0, 0.0, 1.0), 2, (4, 5, 7, 6)), ((0.0, 0.0, -1.0), 2, (0, 1, 3, 2))]
_EDGES = [(0, 1), (2, 3), (4, 5), (6, 7), (0, 2), (1, 3), (4, 6), (5, 7), (0, 4), (1, 5), (2, 6), (3, 7)]


def _on_face(p, face, h):
    n, _, vs = face
    pts = [_corner(v, h) for v in vs]
    c = _mul(_add(_add(pts[0], pts[1]), _add(pts[2], pts[3])), 0.25)
    for j in range(4):
        a, b = pts[j], pts[(j + 1) % 4]
        side = _cross(_sub(b, a), n)
        sg = 1.0 if _dot(side, _sub(c, a)) >= 0 else -1.0
        if _dot(side, _sub(p, a)) * sg < -1e-6:
            return False
    return True


def ray_box(o, d, h, r):
    if r == 0:
        enter, exit_, normal = -3.4e38, 3.4e38, _neg(d)
        for n, k, _ in _FACES:
            denom = _dot(n, d)
            gap = h[k] - _dot(n, o)
            if abs(denom) < 1e-12:
                if gap < 0:
                    return MISS
            else:
                t = gap / denom
                if denom < 0:
                    if t > enter:
                        enter, normal = t, n
                else:
                    exit_ = min(exit_, t)
            if enter > exit_:
                return MISS
        if exit_ < 0:
            return MISS
        return (0.0, _neg(d)) if enter <= 0 else (enter, normal)
    inside, distance, hit = True, 3.4e38, MISS
    for face in _FACES:
        n, k, _ = face
        signed = _dot(n, o) - h[k]
        if signed > 0:
            inside = False
        if _on_face(_sub(o, _mul(n, signed)), face, h):
            distance = min(distance, signed * signed)
        denom = _dot(n, d)
        if denom < -1e-12:
            t = (h[k] + r - _dot(n, o)) / denom
            if t >= 0 and (hit[0] < 0 or t < hit[0]) and _on_face(_sub(_add(o, _mul(d, t)), _mul(n, r)), face, h):
                hit = (t, n)
    for ea, eb in _EDGES:
        a, b = _corner(ea, h), _corner(eb, h)
        q = _sub(o, _closest(a, b, o))
        distance = min(distance, _dot(q, q))
        c = ray_capsule(o, d, a, b, r)
        if c[0] >= 0 and (hit[0] < 0 or c[0] < hit[0]):
            hit = c
    if inside or distance <= r * r:
        return (0.0, _neg(d))
    return hit


def trace(pos, quat, size, shape, origin, direction, radius, max_distance):
    """One body: (t, world normal) or (-1, 0)."""
    inv = (-quat[0], -quat[1], -quat[2], quat[3])
    o = _turn(inv, _sub(origin, pos))
    d = _turn(inv, direction)
    if shape == 1:
        rad = size[0] * 0.5 + radius
        hit = (0.0, _neg(d)) if _dot(o, o) <= rad * rad else ray_sphere(o, d, (0.0, 0.0, 0.0), rad)
    elif shape == 2:  # capsule along local Y (shapeQueries.wgsl trace, shape -1)
        half = max(0.0, size[1] * 0.5 - size[0] * 0.5)
        a, b = (0.0, -half, 0.0), (0.0, half, 0.0)
        rad = size[0] * 0.5 + radius
        delta = _sub(o, _closest(a, b, o))
        hit = (0.0, _neg(d)) if _dot(delta, delta) <= rad * rad else ray_capsule(o, d, a, b, rad)
    else:
        hit = ray_box(o, d, (size[0] * 0.5, size[1] * 0.5, size[2] * 0.5), radius)
    if hit[0] > max_distance or hit[0] < 0:
        return MISS
    return (hit[0], _turn(quat, hit[1]))


def cast(state, shape, size, group, mask, origin, direction, radius=0.0, max_distance=3e38,
         collides_with=0xFFFFFFFF, membership=None, ignore=(), triggers=None, include_triggers=True):
    """Nearest hit: (index, t, normal, second-best t) or None; state: position, rotation arrays.
    Trigger bodies (`triggers[i]`) are skipped unless include_triggers (queries.js:229-233)."""
    ln = math.sqrt(sum(float(x) ** 2 for x in direction))
    dvec = tuple(float(x) / ln for x in direction)
    o = tuple(float(x) for x in origin)
    best = None
    second = math.inf
    for i in range(len(shape)):
        if not (int(group[i]) & collides_with):
            continue
        if membership is not None and (membership == 0 or not (int(mask[i]) & membership)):
            continue
        if i in ignore:
            continue
        if triggers is not None and triggers[i] and not include_triggers:
            continue
        t, n = trace(tuple(map(float, state["position"][i])), tuple(map(float, state["rotation"][i])),
                     tuple(map(float, size[i])), int(shape[i]), o, dvec, float(radius), float(max_distance))
        if t < 0:
            continue
        t = max(0.0, t)
        if best is None or t < best[1]:
            if best is not None:
                second = min(second, best[1])
            best = (i, t, n)
        else:
            second = min(second, t)
    return None if best is None else (best[0], best[1], best[2], second)
