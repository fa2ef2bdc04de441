"""Seeded synthetic scenes of the benchmark configurations.

No dataset is involved: every scene is generated from a NumPy PCG64 stream seeded with
``0xA5BD0000 + config_index``. Mass properties use the builder's formulas
(``reference/three-avbd/src/avbd3d/ref/body.ts:47-51``, ``shapes.ts:28-36``) in float64.
Y is up, gravity -9.81 m/s^2, dt 1/60 s, friction 0.5, density 1000 kg/m^3, solver parameters
at the reference defaults (alpha 0.99, beta 1e4 / 100, gamma 0.999, massPenalty and faceBias
on).

* box_pile_c0   1,000 unit cubes in a 10x10x10 lattice (1.05 m spacing, +-0.01 m jitter,
                +-2 deg yaw) over a static 50x1x50 m ground; grid broadphase, 10 iterations.
* mixed_pile    N bodies, 70 % boxes (half-extents U[0.25, 1] m per axis), 30 % spheres
                (r U[0.25, 0.75] m), uniform random orientation, centres uniform in a
                2L x L x 2L volume (L = 200 m for 1,000,000 bodies, scaled with N^(1/3)),
                over a static ground box 1.1 x the footprint, 2 m thick, top at y = 0.
* lattice_pile  N config-1 bodies (same shape, size and orientation distributions) stacked in
                a jittered cubic lattice (1.9 m spacing, +-0.05 m jitter) starting just above a
                static ground box: a pile that is in contact from the first steps.
* world_mix     4,096 lattice piles with log-normal body counts (median 256, clipped to
                [16, 8,192]); sigma is chosen by bisection so the total is ~2.1 M bodies.
* cloth_wall    a 256x256 grid of 0.1 m cubes with 4-neighbour ball joints, two corners pinned,
                over a static 5 m sphere, beside a 100x2x50 wall of 1x0.5x0.5 m bricks hit by
                a 2 m sphere at 40 m/s; 15 iterations.
"""
from __future__ import annotations

import math

import numpy as np

from .scene import (INF, KIND_JOINT, MASK_ALL, SHAPE_BOX, SHAPE_SPHERE, SceneArrays,
                    SolverParams)

SEED_BASE = 0xA5BD0000
DENSITY = 1000.0
FRICTION = 0.5
GRAVITY = -9.81


def params(iterations=10) -> SolverParams:
    return SolverParams(dt=1.0 / 60.0, gravity=GRAVITY, up=(0.0, 1.0, 0.0), iterations=iterations)


def _bodies(size, density, friction, pos, quat, shape, radius_sphere=None):
    """Vectorised Rigid constructor (+ sphere overrides); float64, reference operation order."""
    n = size.shape[0]
    sx, sy, sz = size[:, 0], size[:, 1], size[:, 2]
    mass = sx * sy * sz * density
    moment = np.stack([((sy * sy + sz * sz) / 12) * mass, ((sx * sx + sz * sz) / 12) * mass,
                       ((sx * sx + sy * sy) / 12) * mass], axis=1)
    a, b, c = sx * 0.5, sy * 0.5, sz * 0.5
    radius = np.sqrt(a * a + b * b + c * c)
    sph = shape == SHAPE_SPHERE
    if sph.any():
        r = radius_sphere[sph]
        d = density[sph]
        m = np.where(d > 0, (4 / 3) * math.pi * r * r * r * d, 0.0)
        mass[sph] = m
        inertia = 0.4 * m * r * r
        moment[sph] = inertia[:, None]
        radius[sph] = r
    z3 = np.zeros((n, 3))
    return dict(pos=pos.astype(np.float64), quat=quat.astype(np.float64), size=size.astype(np.float64),
                vel=z3.copy(), angvel=z3.copy(), prev_vel=z3.copy(), mass=mass, moment=moment,
                friction=np.full(n, friction, dtype=np.float64) if np.isscalar(friction) else friction,
                radius=radius, shape=shape.astype(np.int32), group=np.full(n, MASK_ALL, dtype=np.uint32),
                mask=np.full(n, MASK_ALL, dtype=np.uint32))


def _concat(parts):
    return {k: np.concatenate([p[k] for p in parts]) for k in parts[0]}


def _arrays(b, p, cons=None) -> SceneArrays:
    cons = cons or dict(kind=np.zeros(0, np.int32), ca=np.zeros(0, np.int32), cb=np.zeros(0, np.int32),
                        ra=np.zeros((0, 3)), rb=np.zeros((0, 3)), p0=np.zeros(0), p1=np.zeros(0), p2=np.zeros(0))
    return SceneArrays(params=p, **b, **cons)


def _static_box(size, pos):
    return _bodies(np.array([size], dtype=np.float64), np.array([0.0]), FRICTION, np.array([pos], dtype=np.float64),
                   np.array([[0.0, 0.0, 0.0, 1.0]]), np.array([SHAPE_BOX]))


def _uniform_quats(rng, n):
    q = rng.standard_normal((n, 4))
    return q / np.linalg.norm(q, axis=1, keepdims=True)


def box_pile_c0(seed=SEED_BASE + 0, nx=10, ny=10, nz=10) -> SceneArrays:
    rng = np.random.Generator(np.random.PCG64(seed))
    ground = _static_box((50.0, 1.0, 50.0), (0.0, -0.5, 0.0))
    n = nx * ny * nz
    i, j, k = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    i, j, k = i.reshape(-1), j.reshape(-1), k.reshape(-1)
    pos = np.stack([(i - (nx - 1) / 2) * 1.05, 0.55 + j * 1.05, (k - (nz - 1) / 2) * 1.05], axis=1)
    pos = pos + rng.uniform(-0.01, 0.01, size=(n, 3))
    yaw = np.deg2rad(rng.uniform(-2.0, 2.0, size=n))
    quat = np.stack([np.zeros(n), np.sin(yaw / 2), np.zeros(n), np.cos(yaw / 2)], axis=1)
    cubes = _bodies(np.ones((n, 3)), np.full(n, DENSITY), FRICTION, pos, quat, np.full(n, SHAPE_BOX))
    return _arrays(_concat([ground, cubes]), params(10))


def mixed_pile(n, seed, extent=None) -> SceneArrays:
    """Boxes and spheres as config 1; `extent` = L (height), default scaled to 200 m at 1 M."""
    rng = np.random.Generator(np.random.PCG64(seed))
    L = extent if extent is not None else 200.0 * (n / 1_000_000) ** (1.0 / 3.0)
    L = max(L, 4.0)
    ground = _static_box((2.2 * L, 2.0, 2.2 * L), (0.0, -1.0, 0.0))
    is_sphere = rng.random(n) < 0.3
    half = rng.uniform(0.25, 1.0, size=(n, 3))
    r = rng.uniform(0.25, 0.75, size=n)
    size = np.where(is_sphere[:, None], (2 * r)[:, None] * np.ones((1, 3)), 2 * half)
    pos = np.stack([rng.uniform(-L, L, n), rng.uniform(2.0, 2.0 + L, n), rng.uniform(-L, L, n)], axis=1)
    quat = _uniform_quats(rng, n)
    shape = np.where(is_sphere, SHAPE_SPHERE, SHAPE_BOX)
    bodies = _bodies(size, np.full(n, DENSITY), FRICTION, pos, quat, shape, radius_sphere=r)
    return _arrays(_concat([ground, bodies]), params(10))


def lattice_pile(n, seed, spacing=1.9) -> SceneArrays:
    rng = np.random.Generator(np.random.PCG64(seed))
    ny = max(1, int(round(n ** (1.0 / 3.0) / 1.6)))
    nxz = int(math.ceil(math.sqrt(n / ny)))
    k = np.arange(n)
    layer, rem = k // (nxz * nxz), k % (nxz * nxz)
    ix, iz = rem // nxz, rem % nxz
    pos = np.stack([(ix - (nxz - 1) / 2) * spacing, 1.05 + layer * spacing, (iz - (nxz - 1) / 2) * spacing], axis=1)
    pos = pos + rng.uniform(-0.05, 0.05, size=(n, 3))
    is_sphere = rng.random(n) < 0.3
    half = rng.uniform(0.25, 1.0, size=(n, 3))
    r = rng.uniform(0.25, 0.75, size=n)
    size = np.where(is_sphere[:, None], (2 * r)[:, None] * np.ones((1, 3)), 2 * half)
    quat = _uniform_quats(rng, n)
    shape = np.where(is_sphere, SHAPE_SPHERE, SHAPE_BOX)
    bodies = _bodies(size, np.full(n, DENSITY), FRICTION, pos, quat, shape, radius_sphere=r)
    foot = 1.2 * nxz * spacing + 4.0
    ground = _static_box((foot, 2.0, foot), (0.0, -1.0, 0.0))
    return _arrays(_concat([ground, bodies]), params(10))


def world_counts(n_worlds=4096, target=2_100_000, seed=SEED_BASE + 3, median=256, lo=16, hi=8192):
    """Log-normal world sizes; returns (counts, sigma) with sigma fitted to the target total."""
    rng = np.random.Generator(np.random.PCG64(seed))
    z = rng.standard_normal(n_worlds)

    def counts(sig):
        return np.clip(np.rint(median * np.exp(sig * z)), lo, hi).astype(np.int64)

    a, b = 0.0, 3.0
    for _ in range(60):
        m = 0.5 * (a + b)
        if counts(m).sum() < target:
            a = m
        else:
            b = m
    sig = 0.5 * (a + b)
    return counts(sig), sig


def world_mix(n_worlds=4096, target=2_100_000, seed=SEED_BASE + 3):
    counts, sigma = world_counts(n_worlds, target, seed)
    worlds = [lattice_pile(int(c), (seed * 7919 + w) & 0xFFFFFFFFFFFF) for w, c in enumerate(counts)]
    return worlds, counts, sigma


def world_mix_world(index, n_worlds=4096, target=2_100_000, seed=SEED_BASE + 3) -> SceneArrays:
    """World `index` of world_mix(...) alone (the same scene, without building the others)."""
    counts, _ = world_counts(n_worlds, target, seed)
    return lattice_pile(int(counts[index]), (seed * 7919 + index) & 0xFFFFFFFFFFFF)


def cloth_wall(seed=SEED_BASE + 2, grid=256, wall=(100, 2, 50)) -> SceneArrays:
    parts = []
    ground = _static_box((300.0, 2.0, 300.0), (0.0, -1.0, 0.0))
    parts.append(ground)
    big = _bodies(np.full((1, 3), 10.0), np.array([0.0]), FRICTION, np.array([[0.0, 5.0, 0.0]]),
                  np.array([[0.0, 0.0, 0.0, 1.0]]), np.array([SHAPE_SPHERE]), radius_sphere=np.array([5.0]))
    parts.append(big)
    g = grid
    i, k = np.meshgrid(np.arange(g), np.arange(g), indexing="ij")
    i, k = i.reshape(-1), k.reshape(-1)
    s = 0.1
    pos = np.stack([(i - (g - 1) / 2) * s, np.full(g * g, 10.5), (k - (g - 1) / 2) * s], axis=1)
    cloth = _bodies(np.full((g * g, 3), s), np.full(g * g, DENSITY), FRICTION, pos,
                    np.tile([0.0, 0.0, 0.0, 1.0], (g * g, 1)), np.full(g * g, SHAPE_BOX))
    parts.append(cloth)
    wx, wz, wy = wall
    a, c, b = np.meshgrid(np.arange(wx), np.arange(wz), np.arange(wy), indexing="ij")
    a, b, c = a.reshape(-1), b.reshape(-1), c.reshape(-1)
    nb = a.size
    wpos = np.stack([(a - (wx - 1) / 2) * 1.0 + 0.25 * (b % 2), 0.25 + b * 0.5, 40.0 + c * 0.5], axis=1)
    bricks = _bodies(np.tile([1.0, 0.5, 0.5], (nb, 1)), np.full(nb, DENSITY), FRICTION, wpos,
                     np.tile([0.0, 0.0, 0.0, 1.0], (nb, 1)), np.full(nb, SHAPE_BOX))
    parts.append(bricks)
    ball = _bodies(np.full((1, 3), 4.0), np.array([DENSITY]), FRICTION, np.array([[0.0, 2.0, 25.0]]),
                   np.array([[0.0, 0.0, 0.0, 1.0]]), np.array([SHAPE_SPHERE]), radius_sphere=np.array([2.0]))
    ball["vel"][0] = [0.0, 0.0, 40.0]
    parts.append(ball)
    b = _concat(parts)
    off = 2  # cloth starts after ground and static sphere
    idx = lambda x, z: off + x * g + z  # noqa: E731
    ka, kb, ra, rb = [], [], [], []
    for x in range(g):
        for z in range(g):
            if x + 1 < g:
                ka.append(idx(x, z)); kb.append(idx(x + 1, z)); ra.append([s / 2, 0, 0]); rb.append([-s / 2, 0, 0])
            if z + 1 < g:
                ka.append(idx(x, z)); kb.append(idx(x, z + 1)); ra.append([0, 0, s / 2]); rb.append([0, 0, -s / 2])
    for x, z in ((0, 0), (g - 1, 0)):
        p = b["pos"][idx(x, z)]
        ka.append(-1); kb.append(idx(x, z)); ra.append(list(p)); rb.append([0, 0, 0])
    m = len(ka)
    cons = dict(kind=np.full(m, KIND_JOINT, np.int32), ca=np.array(ka, np.int32), cb=np.array(kb, np.int32),
                ra=np.array(ra, np.float64), rb=np.array(rb, np.float64), p0=np.full(m, INF),
                p1=np.zeros(m), p2=np.full(m, INF))
    return _arrays(b, params(15), cons)


def request_stream(n_requests=20_000, rate=10_000.0, seed=SEED_BASE + 4, warm_creates=256, create_share=0.1,
                   median=256, lo=16, hi=65_536, sigma=1.2078):
    """A serving request stream: Poisson arrivals at `rate` per second; each request creates a
    world (log-normal body count with the given median and sigma, clipped to [lo, hi]; a box and
    sphere pile as in the world mix) or advances a uniformly chosen earlier world by K in
    {1, 4, 16} steps. The first `warm_creates` requests are creates, then creates make up
    `create_share` of the requests. Returns a dict of arrays in arrival order."""
    rng = np.random.Generator(np.random.PCG64(seed))
    arrival = np.cumsum(rng.exponential(1.0 / rate, n_requests))
    create = rng.random(n_requests) < create_share
    create[:warm_creates] = True
    z = rng.standard_normal(n_requests)
    counts = np.clip(np.rint(median * np.exp(sigma * z)), lo, hi).astype(np.int64)
    steps = rng.choice(np.array([1, 4, 16]), size=n_requests)
    u = rng.random(n_requests)
    made = np.cumsum(create) - create  # worlds created before each request
    target = np.where(create, -1, np.minimum((u * made).astype(np.int64), np.maximum(made - 1, 0)))
    counts = np.where(create, counts, 0)
    steps = np.where(create, 0, steps)
    world_seed = (seed * 7919 + np.arange(n_requests)) & 0xFFFFFFFFFFFF
    return {"arrival": arrival, "create": create, "count": counts, "steps": steps, "target": target,
            "world_seed": world_seed, "sigma": sigma, "rate": rate, "seed": seed}
