"""The oracle's restitution pass against an independent float64 restatement of the reference's
bounce (src/native/cpu/restitution.js captureIncoming / bounceContacts, and the GPU backend's
src/gpu/restitution.js): per manifold the centroid of the rotated anchors, the incoming normal
speed n . ((v - r x w)_a - (v - r x w)_b) from the step's starting velocities, a 1 m/s impact
threshold, k = 1/ma + 1/mb + ta.Ia^-1 ta + tb.Ib^-1 tb, target -e vn, and 12 Jacobi rounds of
max(0, impulse + (target - vn) / (k max(1, deg a, deg b))) whose velocity changes are summed per
round. The degree is the length of a body's constraint list. The two reference backends differ
there: the GPU backend's adjacency holds dynamic bodies only (a static body's degree is 0,
avbd2d/gpu/wgsl-topology.ts countEndpoints), the CPU world counts every force of a static body
too. The oracle, like the engine, follows the GPU backend; the restatement below takes the
degree as a parameter and checks both readings against the oracle and each other.

Every contact here is fresh (no manifold from an earlier step), so the oracle's manifolds are
exactly what its narrowphase returns for the start-of-step poses.
"""
import numpy as np
import pytest

from avbd_gb300 import AvbdScene3D


def _turn(q, v):
    x, y, z, w = q
    u = np.array([x, y, z])
    t = 2.0 * np.cross(u, v)
    return v + w * t + np.cross(u, t)


def _reference_bounce(o_start, inc_v, inc_w, v, w, quat, mass, moment, e, static_degree=False):
    """bounceContacts of restitution.js (3D, no sleeping bodies or triggers); `static_degree`:
    static bodies count their manifolds in the relaxation degree (the CPU world's reading)."""
    n = len(mass)
    inv_mass = np.where(mass > 0, 1.0 / np.where(mass > 0, mass, 1.0), 0.0)

    def inv_inertia(i, t):
        if not inv_mass[i]:
            return np.zeros(3)
        q = quat[i]
        local = _turn(np.array([-q[0], -q[1], -q[2], q[3]]), t)
        local = np.array([local[k] / moment[i][k] if moment[i][k] > 0 else 0.0 for k in range(3)])
        return _turn(q, local)

    def point_velocity(vv, ww, i, r):
        return vv[i] - np.cross(r, ww[i])

    manifolds = []
    for a, b in o_start.candidate_pairs():
        m = o_start.collide(int(a), int(b))
        if m["count"] == 0:
            continue
        ra = np.zeros(3)
        rb = np.zeros(3)
        for c in range(m["count"]):
            ra += _turn(quat[a], m["ra"][c]) / m["count"]
            rb += _turn(quat[b], m["rb"][c]) / m["count"]
        manifolds.append(dict(a=int(a), b=int(b), n=m["basis"][0].copy(), ra=ra, rb=rb, e=max(e[a], e[b])))
    degree = np.zeros(n, dtype=np.int64)
    for m in manifolds:  # the body's constraint list (no joints in these scenes)
        for i in (m["a"], m["b"]):
            if mass[i] > 0 or static_degree:
                degree[i] += 1
    pairs = []
    for p in manifolds:
        if p["e"] <= 0:
            continue
        vn = p["n"] @ (point_velocity(inc_v, inc_w, p["a"], p["ra"]) - point_velocity(inc_v, inc_w, p["b"], p["rb"]))
        if vn >= -1:
            continue
        ta, tb = np.cross(p["ra"], p["n"]), np.cross(p["rb"], p["n"])
        ia, ib = inv_inertia(p["a"], ta), inv_inertia(p["b"], tb)
        k = inv_mass[p["a"]] + inv_mass[p["b"]] + ta @ ia + tb @ ib
        if k > 0:
            pairs.append(dict(p, ia=ia, ib=ib, k=k, target=-p["e"] * vn, impulse=0.0))
    v, w = v.copy(), w.copy()
    for _ in range(12):
        if not pairs:
            break
        dv, dw = np.zeros_like(v), np.zeros_like(w)
        for p in pairs:
            vn = p["n"] @ (point_velocity(v, w, p["a"], p["ra"]) - point_velocity(v, w, p["b"], p["rb"]))
            imp = max(0.0, p["impulse"] + (p["target"] - vn) / (p["k"] * max(1, degree[p["a"]], degree[p["b"]])))
            change = imp - p["impulse"]
            p["impulse"] = imp
            for i, sign, inertia in ((p["a"], 1, p["ia"]), (p["b"], -1, p["ib"])):
                dv[i] += sign * change * inv_mass[i] * p["n"]
                dw[i] += sign * change * inertia
        v += dv
        w += dw
    return v, w, len(pairs)


def _scene(bouncy=True):
    sc = AvbdScene3D(timeStep=1 / 60, iterations=10, gravity=-10)
    sc.addBox([40, 1, 40], position=[0, -0.5, 0], density=0)
    r = (lambda x: x) if bouncy else (lambda x: 0.0)
    # onto the ground (top at y = 0), touching at the start of the step
    sc.addSphere(0.5, position=[-12, 0.49, 0], velocity=[0, -5, 0], restitution=r(0.8))
    sc.addSphere(0.4, position=[-9, 0.39, 1], velocity=[1.5, -7, 0.5], angularVelocity=[0, 0, 3], restitution=r(0.5))
    sc.addBox([1, 1, 1], position=[-6, 0.495, 0], velocity=[0, -4, 0], restitution=r(0.6))
    sc.addBox([2, 0.5, 1], position=[-2, 0.24, 3], velocity=[0.5, -6, 0], angularVelocity=[0.3, 0, 0.2],
              rotation=[0.02, 0.0, 0.01, 1.0], restitution=r(0.9))
    sc.addSphere(0.5, position=[2, 0.49, 0], velocity=[0, -0.6, 0], restitution=r(0.9))  # below the threshold
    sc.addSphere(0.5, position=[4, 0.49, 0], velocity=[0, -5, 0], restitution=0.0)  # e = 0
    # head-on in the air: the larger restitution of the two applies
    sc.addSphere(0.5, position=[9.5, 4, 0], velocity=[5, 0, 0], restitution=r(1.0))
    sc.addSphere(0.5, position=[10.49, 4, 0], velocity=[-5, 0, 0], restitution=r(0.3))
    sc.addBox([1, 1, 1], position=[14, 4, 0], velocity=[3, 0, 0], restitution=r(0.7))
    sc.addBox([1, 1, 1], position=[14.99, 4, 0], velocity=[-3, 0.2, 0], density=3, restitution=r(0.2))
    return sc.arrays()


def test_oracle_bounce_matches_the_reference_restatement(oracle_mod):
    bouncy, plain = _scene(True), _scene(False)
    start = oracle_mod.OracleWorld(bouncy, fp64=True, app=True, colored=True)
    o_bounce = oracle_mod.OracleWorld(bouncy, fp64=True, app=True, colored=True)
    o_plain = oracle_mod.OracleWorld(plain, fp64=True, app=True, colored=True)
    s0 = start.bodies()
    o_bounce.step(1)
    o_plain.step(1)
    b, p = o_bounce.bodies(), o_plain.bodies()
    # the pass only changes velocities
    assert np.array_equal(b["pos"], p["pos"]) and np.array_equal(b["quat"], p["quat"])
    v, w, active = _reference_bounce(start, s0["vel"], s0["angvel"], p["vel"], p["angvel"], b["quat"],
                                     bouncy.mass, bouncy.moment, bouncy.restitution)
    assert active == 6  # four ground impacts and two head-on pairs
    assert np.abs(b["vel"] - v).max() < 1e-9
    assert np.abs(b["angvel"] - w).max() < 1e-9
    # bodies without a qualifying impact are untouched
    for i in (5, 6):
        assert np.array_equal(b["vel"][i], p["vel"][i])
    assert abs(b["vel"][1][1] - 4.0) < 1e-9  # the e = 0.8 sphere leaves at 0.8 x 5 m/s
    # the CPU world's reading relaxes the six ground contacts by the ground's degree: weaker
    # bounces, the head-on pairs (no static body) unchanged
    vc, _, _ = _reference_bounce(start, s0["vel"], s0["angvel"], p["vel"], p["angvel"], b["quat"],
                                 bouncy.mass, bouncy.moment, bouncy.restitution, static_degree=True)
    assert 3.0 < vc[1][1] < 4.0
    assert np.abs(vc[7:] - v[7:]).max() < 1e-12


@pytest.mark.parametrize("fp64", [False, True])
def test_zero_restitution_is_the_plain_step(oracle_mod, fp64):
    plain = _scene(False)
    zeros = _scene(False)
    zeros.restitution = np.zeros(zeros.n_bodies)
    a = oracle_mod.OracleWorld(plain, fp64=fp64, app=True, colored=True)
    b = oracle_mod.OracleWorld(zeros, fp64=fp64, app=True, colored=True)
    a.step(20)
    b.step(20)
    for k, x in a.bodies().items():
        assert np.array_equal(x, b.bodies()[k]), k
