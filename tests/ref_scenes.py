"""The 14 avbd-demo3d scenes of ``reference/three-avbd/src/avbd3d/ref/scenes.ts``, restated
for the oracle's golden-trajectory tests (Z up, gravity -10, the pinned solver's defaults).

Each builder follows its reference function line for line (same creation order of bodies and
constraints, same float64 arithmetic), since creation order fixes the reference's force-list
order and so its summation order.
"""
from __future__ import annotations

import math
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "babylon-avbd_gb300"))

from avbd_gb300.scene import INF, SceneBuilder, SolverParams  # noqa: E402


def _params():
    return SolverParams(dt=1 / 60, gravity=-10.0, up=(0.0, 0.0, 1.0), iterations=10)


# math.ts helpers used by the scenes
def _rotate(q, v):
    ux, uy, uz, w = q
    tx = (uy * v[2] - uz * v[1]) * 2
    ty = (uz * v[0] - ux * v[2]) * 2
    tz = (ux * v[1] - uy * v[0]) * 2
    return [v[0] + tx * w + (uy * tz - uz * ty), v[1] + ty * w + (uz * tx - ux * tz),
            v[2] + tz * w + (ux * ty - uy * tx)]


def _normalize(v):
    ln = math.sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2])
    return [v[0] / ln, v[1] / ln, v[2] / ln]


def _add_scaled(a, b, s):
    return [a[0] + b[0] * s, a[1] + b[1] * s, a[2] + b[2] * s]


def _ground(s, z=0.0):
    return s.rigid([100, 100, 1], 0, 0.5, [0, 0, z])


def empty(s):
    pass


def ground(s):
    _ground(s)
    s.rigid([1, 1, 1], 1, 0.5, [0, 0, 4])


def dynamic_friction(s):
    _ground(s)
    for x in range(11):
        s.rigid([1, 1, 0.5], 1, 5 - (x / 10) * 5, [0, -30 + x * 2, 0.75], [10, 0, 0])


def static_friction(s):
    _ground(s)
    angle = 30 * 0.017453292519943295
    ramp = s.rigid([40, 24, 1], 0, 1, [0, 0, 3])
    q = [0.0, math.sin(angle * 0.5), 0.0, math.cos(angle * 0.5)]
    s.bodies[ramp].quat = q
    tangent = _normalize(_rotate(q, [1, 0, 0]))
    normal = _normalize(_rotate(q, [0, 0, 1]))
    for i in range(11):
        friction = (i / 10) * 0.25 + 0.25
        y = -10 + i * 2
        pos = _add_scaled(s.bodies[ramp].pos, tangent, -12)
        pos[1] += y
        pos = _add_scaled(pos, normal, 1.05)
        s.rigid([1, 1, 1], 1, friction, pos)


def pyramid(s, size=16):
    _ground(s, -0.5)
    for y in range(size):
        for x in range(size - y):
            s.rigid([1, 0.5, 0.5], 1, 0.5, [x * 1.01 + y * 0.5 - size / 2, 0, y * 0.85 + 0.5])


def rope(s):
    _ground(s, -20)
    prev = None
    for i in range(20):
        curr = s.rigid([1, 0.5, 0.5], 0 if i == 0 else 1, 0.5, [i, 0, 10])
        if prev is not None:
            s.joint(prev, curr, [0.5, 0, 0], [-0.5, 0, 0])
        prev = curr


def heavy_rope(s):
    N, SIZE = 20, 5
    _ground(s, -20)
    prev = None
    for i in range(N):
        last = i == N - 1
        curr = s.rigid([SIZE, SIZE, SIZE] if last else [1, 0.5, 0.5], 0 if i == 0 else 1, 0.5,
                       [i + (SIZE / 2 if last else 0), 0, 10])
        if prev is not None:
            s.joint(prev, curr, [0.5, 0, 0], [-SIZE / 2, 0, 0] if last else [-0.5, 0, 0])
        prev = curr


def spring(s):
    _ground(s)
    anchor = s.rigid([1, 1, 1], 0, 0.5, [0, 0, 14])
    block = s.rigid([2, 2, 2], 1, 0.5, [0, 0, 8])
    s.spring(anchor, block, [0, 0, 0], [0, 0, 0], 100, 4)


def springs_ratio(s):
    N = 8
    _ground(s, -10)
    prev = None
    for i in range(N):
        x = (i - (N - 1) * 0.5) * 3
        curr = s.rigid([1, 0.75, 0.75], 0 if (i == 0 or i == N - 1) else 1, 0.5, [x, 0, 12])
        if prev is not None:
            s.spring(prev, curr, [0.5, 0, 0], [-0.5, 0, 0], 10 if i % 2 == 0 else 10000, 3)
        prev = curr


def stack(s):
    _ground(s)
    for i in range(10):
        s.rigid([1, 1, 1], 1, 0.5, [0, 0, i * 1.5 + 1])


def stack_ratio(s):
    thick = 1
    s.rigid([100, 100, thick], 0, 0.5, [0, 0, 0])
    top = thick * 0.5
    sz = 1
    for _ in range(4):
        half = sz * 0.5
        cz = top + half
        s.rigid([sz, sz, sz], 1, 0.5, [0, 0, cz])
        top = cz + half
        sz *= 2


def soft_body(s):
    _ground(s)
    Klin, Kang = 1000, 250
    W = D = H = 4
    N = 3
    size = 0.8
    half = size * 0.5
    baseZ, gap = 8, 2
    for i in range(N):
        stackZ = i * (H * size + gap)
        grid = [[[None] * H for _ in range(D)] for _ in range(W)]
        for x in range(W):
            for y in range(D):
                for z in range(H):
                    px = (x - (W - 1) * 0.5) * size
                    py = (y - (D - 1) * 0.5) * size
                    pz = baseZ + stackZ + z * size
                    grid[x][y][z] = s.rigid([size, size, size], 1, 0.5, [px, py, pz])
        for x in range(1, W):
            for y in range(D):
                for z in range(H):
                    s.joint(grid[x - 1][y][z], grid[x][y][z], [half, 0, 0], [-half, 0, 0], Klin, Kang)
        for x in range(W):
            for y in range(1, D):
                for z in range(H):
                    s.joint(grid[x][y - 1][z], grid[x][y][z], [0, half, 0], [0, -half, 0], Klin, Kang)
        for x in range(W):
            for y in range(D):
                for z in range(1, H):
                    s.joint(grid[x][y][z - 1], grid[x][y][z], [0, 0, half], [0, 0, -half], Klin, Kang)
        for x in range(1, W):
            for y in range(D):
                for z in range(1, H):
                    s.ignore(grid[x - 1][y][z - 1], grid[x][y][z])
                    s.ignore(grid[x][y][z - 1], grid[x - 1][y][z])
        for x in range(W):
            for y in range(1, D):
                for z in range(1, H):
                    s.ignore(grid[x][y - 1][z - 1], grid[x][y][z])
                    s.ignore(grid[x][y][z - 1], grid[x][y - 1][z])
        for x in range(1, W):
            for y in range(1, D):
                for z in range(H):
                    s.ignore(grid[x - 1][y - 1][z], grid[x][y][z])
                    s.ignore(grid[x][y - 1][z], grid[x - 1][y][z])


def bridge(s):
    N, L, Wd, Ht = 40, 1, 4, 0.5
    hl, hw = L * 0.5, Wd * 0.5
    _ground(s)
    prev = None
    for i in range(N):
        curr = s.rigid([L, Wd, Ht], 0 if (i == 0 or i == N - 1) else 1, 0.5, [i - N / 2, 0, 10])
        if prev is not None:
            s.joint(prev, curr, [hl, hw, 0], [-hl, hw, 0], INF, 0)
            s.joint(prev, curr, [hl, -hw, 0], [-hl, -hw, 0], INF, 0)
        prev = curr
    for x in range(N // 4):
        for y in range(N // 8):
            s.rigid([1, 1, 1], 1, 0.5, [x - N / 8, 0, y + 12])


def breakable(s):
    N, M, brk = 10, 5, 90
    _ground(s)
    prev = None
    for i in range(N + 1):
        curr = s.rigid([1, 1, 0.5], 1, 0.5, [i - N / 2, 0, 6])
        if prev is not None:
            s.joint(prev, curr, [0.5, 0, 0], [-0.5, 0, 0], INF, INF, brk)
        prev = curr
    s.rigid([1, 1, 5], 0, 0.5, [-N / 2, 0, 2.5])
    s.rigid([1, 1, 5], 0, 0.5, [N / 2, 0, 2.5])
    for i in range(M):
        s.rigid([2, 1, 1], 1, 0.5, [0, 0, i * 2 + 8])


SCENES = [
    ("Empty", empty), ("Ground", ground), ("Dynamic Friction", dynamic_friction),
    ("Static Friction", static_friction), ("Pyramid", pyramid), ("Rope", rope),
    ("Heavy Rope", heavy_rope), ("Spring", spring), ("Spring Ratio", springs_ratio),
    ("Stack", stack), ("Stack Ratio", stack_ratio), ("Soft Body", soft_body),
    ("Bridge", bridge), ("Breakable", breakable),
]


def build(name_or_index, iterations=10):
    if isinstance(name_or_index, int):
        name, fn = SCENES[name_or_index]
    else:
        name, fn = next(x for x in SCENES if x[0] == name_or_index)
    p = _params()
    p.iterations = iterations
    s = SceneBuilder(p)
    fn(s)
    return s.arrays()
