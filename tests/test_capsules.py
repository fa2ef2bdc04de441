"""Capsules (src/native/scenes.js:180-193 addCapsule, src/gpu/capsuleShape.js, the CPU path's
spine geometry src/native/cpu/cpuContacts3D.js:43-88,188-296).

CPU: the builder's mass properties (the cylinder-plus-caps formulas), its validation, and the
oracle's generic narrowphase on capsules (a capsule lying on a box touches along its spine's
nearest end; two crossed capsules touch at their segments' closest points). GPU (marked): a pile
of capsules, spheres and boxes stepped by the engine against the oracle -- candidate pairs and the
contacts of every capsule-box, capsule-sphere and capsule-capsule pair bit-exact, poses within the
float32 tolerance -- and capsule casts against the float64 restatement of shapeQueries.wgsl.
"""
import math

import numpy as np
import pytest

import oracle as O
import parity
from avbd_gb300 import AvbdScene3D, createSolverPipeline
from avbd_gb300.scene import SHAPE_BOX, SHAPE_CAPSULE, SHAPE_SPHERE, SolverParams


def test_capsule_mass_properties():
    sc = AvbdScene3D(timeStep=1 / 60, iterations=10, gravity=-9.81)
    r, h, rho = 0.3, 1.6, 800.0
    i = sc.addCapsule(r, h, density=rho, position=[0, 2, 0])
    a = sc.arrays()
    L = h - 2 * r
    cyl = math.pi * r * r * L * rho
    caps = 4 / 3 * math.pi * r ** 3 * rho
    assert a.mass[i] == pytest.approx(cyl + caps, rel=1e-15)
    axial = cyl * r * r / 2 + caps * 2 * r * r / 5
    radial = cyl * (L * L / 12 + r * r / 4) + caps * (2 * r * r / 5 + L * L / 4 + 3 * L * r / 8)
    np.testing.assert_allclose(a.moment[i], [radial, axial, radial], rtol=1e-15)
    assert a.radius[i] == pytest.approx(h / 2) and a.shape[i] == SHAPE_CAPSULE
    np.testing.assert_array_equal(a.size[i], [2 * r, h, 2 * r])
    with pytest.raises(ValueError):
        sc.addCapsule(0.5, 0.9)  # height below twice the radius
    with pytest.raises(ValueError):
        sc.addCapsule(-1.0, 3.0)


def _scene(kind):
    sc = AvbdScene3D(timeStep=1 / 60, iterations=10, gravity=-9.81)
    sc.addBox([20, 1, 20], density=0, friction=0.5, position=[0, -0.5, 0])
    if kind == "lying":
        sc.addCapsule(0.25, 1.5, density=1000, friction=0.5, position=[0, 0.24, 0],
                      rotation=[0, 0, math.sin(math.pi / 4), math.cos(math.pi / 4)])
    else:
        sc.addCapsule(0.25, 1.5, density=1000, friction=0.5, position=[0, 0.3, 0],
                      rotation=[0, 0, math.sin(math.pi / 4), math.cos(math.pi / 4)])
        sc.addCapsule(0.25, 1.5, density=1000, friction=0.5, position=[0, 0.78, 0],
                      rotation=[math.sin(math.pi / 4), 0, 0, math.cos(math.pi / 4)])
    return sc.arrays()


def test_oracle_capsule_on_box_and_crossed_capsules():
    a = _scene("lying")
    o = O.OracleWorld(a, fp64=True, app=True)
    c = o.collide(1, 0)
    assert c["count"] == 1
    n = np.asarray(c["basis"])[0]
    assert abs(abs(n[1]) - 1.0) < 1e-12  # the box's top face normal
    b = _scene("crossed")
    o = O.OracleWorld(b, fp64=True, app=True)
    c = o.collide(2, 1)
    assert c["count"] == 1
    n = np.asarray(c["basis"])[0]
    assert abs(abs(n[1]) - 1.0) < 1e-9  # crossed segments: the normal joins their closest points


def capsule_pile(n, seed):
    rng = np.random.default_rng(seed)
    sc = AvbdScene3D(timeStep=1 / 60, iterations=10, gravity=-9.81)
    sc.addBox([30, 1, 30], density=0, friction=0.5, position=[0, -0.5, 0])
    side = int(math.ceil(n ** (1 / 3)))
    for k in range(n):
        x, y, z = k % side, (k // side) % side, k // (side * side)
        pos = [(x - side / 2) * 1.3 + rng.uniform(-0.1, 0.1), 0.9 + 1.3 * z + rng.uniform(0, 0.1),
               (y - side / 2) * 1.3 + rng.uniform(-0.1, 0.1)]
        q = rng.normal(size=4)
        q = list(q / np.linalg.norm(q))
        kind = k % 3
        if kind == 0:
            sc.addCapsule(rng.uniform(0.15, 0.35), rng.uniform(0.8, 1.2), density=1000, friction=0.5, position=pos, rotation=q)
        elif kind == 1:
            sc.addSphere(rng.uniform(0.2, 0.45), density=1000, friction=0.5, position=pos)
        else:
            sc.addBox(list(rng.uniform(0.4, 0.9, size=3)), density=1000, friction=0.5, position=pos, rotation=q)
    return sc.arrays()


@pytest.mark.gpu
@pytest.mark.parametrize("warm", [10, 60])
def test_capsule_pile_matches_the_oracle(warm):
    scene = capsule_pile(120, seed=9)
    pipe = createSolverPipeline("gb300", device=0)
    w = pipe.createSolver(scene)
    rep = parity.compare_step(w, scene, warm)
    pairs = w.readPairs().astype(np.int64)
    counts = w.readPairContacts()
    shapes = scene.shape[pairs]
    kinds = {"capsule-box": ((shapes == SHAPE_CAPSULE) & (shapes[:, ::-1] == SHAPE_BOX)).any(axis=1),
             "capsule-sphere": ((shapes == SHAPE_CAPSULE) & (shapes[:, ::-1] == SHAPE_SPHERE)).any(axis=1),
             "capsule-capsule": (shapes == SHAPE_CAPSULE).all(axis=1)}
    touching = {k: int(((counts > 0) & m).sum()) for k, m in kinds.items()}
    print(warm, touching, rep)
    pipe.destroy()
    assert rep["pairs_equal"] and rep["contact_counts_equal"] and rep["colors_equal"] and rep["coloring_valid"], rep
    assert rep["max_err_fp32"] <= parity.TOL, rep
    if warm == 60:
        assert all(v > 0 for v in touching.values()), touching


@pytest.mark.gpu
def test_capsule_casts_match_the_restatement():
    """Rays and sphere casts at a pile with capsules: the same body as the float64 restatement of
    shapeQueries.wgsl (except where its two nearest distances are within 1e-4), distance within
    1e-4 (|t| + 1)."""
    import queries as Q
    scene = capsule_pile(60, seed=4)
    pipe = createSolverPipeline("gb300", device=0)
    w = pipe.createSolver(scene)
    w.step(20)
    st = w.readBodyState()
    rng = np.random.default_rng(5)
    casts = []
    for k in range(300):
        o = rng.uniform([-5, 4, -5], [5, 8, 5])
        target = rng.uniform([-4, 0, -4], [4, 3, 4])
        casts.append({"origin": o.tolist(), "direction": (target - o).tolist(),
                      "radius": 0.0 if k % 2 == 0 else float(rng.uniform(0.05, 0.5))})
    got = w.sphereCastAll(casts)
    hits = capsule_hits = 0
    for g, c in zip(got, casts):
        want = Q.cast(st, scene.shape, scene.size, scene.group, scene.mask, c["origin"], c["direction"],
                      radius=c["radius"])
        if want is None:
            assert g is None, (c, g)
            continue
        i, t, n, second = want
        assert g is not None, (c, want)
        assert abs(g["distance"] - t) <= 1e-4 * (abs(t) + 1), (c, g, want)
        if g["index"] != i:
            assert second - t < 1e-4, (c, g, want)
        hits += 1
        capsule_hits += int(scene.shape[i] == SHAPE_CAPSULE)
    pipe.destroy()
    assert hits > 100 and capsule_hits > 10, (hits, capsule_hits)
