"""CPU-side checks: the C-ABI library loads and exports every declared symbol, the scene
builder validates like the reference, workloads have the configured shapes, and the oracle's
app path behaves (no GPU needed)."""
import ctypes
import math
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib_path():
    import importlib.util
    spec = importlib.util.spec_from_file_location("avbd_build", os.path.join(ROOT, "babylon-avbd_gb300", "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build()


def declared_symbols():
    names = []
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            text = open(os.path.join(ROOT, "include", h)).read()
            names += re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\*?\s+\**(avbd_[a-z_0-9]+)\s*\(", text, re.M)
    return sorted(set(names))


def test_library_exports_every_declared_symbol(lib_path):
    lib = ctypes.CDLL(lib_path)
    names = declared_symbols()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n


def test_ctypes_signatures_cover_header():
    from avbd_gb300 import _lib
    bound = {n for n, _, _ in _lib.SIGNATURES}
    assert set(declared_symbols()) <= bound | set()


def test_builder_validation_and_mass():
    from avbd_gb300 import AvbdScene3D
    s = AvbdScene3D(gravity=-9.81)
    b = s.addBox([1, 2, 3], density=2)
    arr = s.arrays()
    assert arr.mass[b] == 12 and list(arr.moment[b]) == [13, 10, 5]
    sp = s.addSphere(0.5, density=1000, position=[0, 3, 0], velocity=[1, 0, 0])
    arr = s.arrays()
    assert arr.shape[sp] == 1 and arr.radius[sp] == 0.5
    assert abs(arr.mass[sp] - 4 / 3 * math.pi * 0.125 * 1000) < 1e-9
    assert list(arr.prev_vel[sp]) == [0, 0, 0] and list(arr.vel[sp]) == [1, 0, 0]
    with pytest.raises(ValueError):
        s.addBox([1, -1, 1])
    with pytest.raises(ValueError):
        s.addBox([1, 1, 1], rotation=[0, 0, 0, 0])
    with pytest.raises(ValueError):
        s.addJoint(b, b)
    with pytest.raises(ValueError):
        AvbdScene3D(up=[0, 2, 0])
    with pytest.raises(ValueError):
        s.addSpring(None, b)
    j = s.addJoint(None, b, [0, 5, 0], [0, 0, 0])
    assert s.arrays().ca[j] == -1
    m = s.addBox([1, 1, 1], density=1, mass=3)
    a = s.arrays()
    assert a.mass[m] == 3 and abs(a.moment[m][0] - 0.5) < 1e-12


def test_world_mix_counts():
    from avbd_gb300 import workloads
    counts, sigma = workloads.world_counts()
    assert len(counts) == 4096
    assert counts.min() >= 16 and counts.max() <= 8192
    assert abs(counts.sum() - 2_100_000) < 2000
    assert 0.9 < sigma < 1.4
    assert int(np.median(counts)) in range(240, 272)


def test_box_pile_c0_layout():
    from avbd_gb300 import workloads
    s = workloads.box_pile_c0()
    assert s.n_bodies == 1001 and s.mass[0] == 0 and np.all(s.mass[1:] == 1000)
    assert np.all(np.abs(s.pos[1:, 1] - np.round((s.pos[1:, 1] - 0.55) / 1.05) * 1.05 - 0.55) <= 0.0100001)


def test_oracle_app_stack_rests_on_ground():
    """App path (Y up): a 5-box stack settles within the collision margin per contact."""
    import oracle
    from avbd_gb300.scene import SceneBuilder, SolverParams
    b = SceneBuilder(SolverParams(dt=1 / 60, gravity=-10, up=(0, 1, 0), iterations=10))
    b.rigid([100, 1, 100], 0, 0.5, [0, -0.5, 0])
    for i in range(5):
        b.rigid([1, 1, 1], 1, 0.5, [0, 0.5 + 1.2 * i, 0])
    w = oracle.OracleWorld(b.arrays(), fp64=True, app=True)
    w.step(600)
    y = w.bodies()["pos"][1:, 1]
    for i in range(5):
        assert abs(y[i] - (0.5 + i)) < 0.011 * (i + 1), y


def test_oracle_colored_equals_sequential_without_contacts():
    """With no constraints the colour order cannot matter: bit-identical free fall."""
    import oracle
    from avbd_gb300 import workloads
    s = workloads.mixed_pile(50, seed=3, extent=400.0)
    a = oracle.OracleWorld(s, fp64=True, app=True, colored=False)
    b = oracle.OracleWorld(s, fp64=True, app=True, colored=True)
    a.step(3)
    b.step(3)
    assert np.array_equal(a.bodies()["pos"], b.bodies()["pos"])


def test_oracle_fp32_narrowphase_box_box_kat():
    """300 seeded rotated box pairs (reference tests/helpers/reference-contacts.js:20-57 LCG,
    seed 0x51a7b0d): the float32 narrowphase agrees with float64 on hit/miss outside a 1 cm
    skin, and the normal is unit length to 1e-4 (reference tests/gpu-stress.js:200-240)."""
    import oracle
    from avbd_gb300.scene import SceneBuilder, SolverParams
    seed = 0x51A7B0D

    def rnd():
        nonlocal seed
        seed = (seed * 1664525 + 1013904223) & 0xFFFFFFFF
        return seed / 4294967296

    hits = misses = 0
    for _ in range(300):
        b = SceneBuilder(SolverParams(up=(0, 1, 0)))
        for k in range(2):
            size = [0.2 + 1.8 * rnd() for _ in range(3)]
            pos = [(rnd() - 0.5) * 2.0 for _ in range(3)]
            q = [rnd() - 0.5 for _ in range(4)]
            n = math.sqrt(sum(v * v for v in q))
            i = b.rigid(size, 1, 0.5, pos)
            b.bodies[i].quat = [v / n for v in q]
        s = b.arrays()
        s.pos = s.pos.astype(np.float32).astype(np.float64)
        s.quat = s.quat.astype(np.float32).astype(np.float64)
        s.size = s.size.astype(np.float32).astype(np.float64)
        r32 = oracle.OracleWorld(s, fp64=False, app=True).collide(1, 0)
        r64 = oracle.OracleWorld(s, fp64=True, app=True).collide(1, 0)
        if (r32["count"] > 0) != (r64["count"] > 0):
            continue  # grazing case inside the skin
        if r64["count"]:
            hits += 1
            assert abs(np.linalg.norm(r32["basis"][0]) - 1) < 1e-4
        else:
            misses += 1
    assert hits > 20 and misses > 20


def test_stage_edits_layout_and_validation():
    import numpy as np
    import pytest as _pt
    from avbd_gb300.pipeline import stage_edits
    rec = stage_edits([{"body": 2, "position": [1, 2, 3], "rotation": [0, 0, 0, 2], "linearVelocity": [4, 5, 6],
                        "force": [1, 0, 0], "worldPoint": [0, 1, 0], "torque": [0, 0, 3]}], 5, 0.5)
    assert rec.shape == (4, 12)
    f = rec.view(np.float32)
    assert list(rec[:, 1]) == [4, 0, 3, 6]  # teleport first, then kinds in order
    assert list(rec[:, 0]) == [2, 2, 2, 2]
    assert rec[0, 2] == 1 and list(f[0, 4:7]) == [1, 2, 3] and list(f[0, 8:12]) == [0, 0, 0, 1]
    assert rec[1, 2] == 0 and rec[2, 2] == 1 and f[2, 7] == 0.5 and f[3, 7] == 0.5
    assert list(f[2, 8:11]) == [0, 1, 0]
    for bad in ({"body": 5, "linearVelocity": [0, 0, 0]}, {"body": 0, "rotation": [0, 0, 0, 1]},
                {"body": 0, "impulse": [0, float("nan"), 0]}, {"body": 0, "position": [0, 0, 0], "rotation": [0, 0, 0, 0]},
                {"body": 0, "restitution": 0.5}):
        with _pt.raises(ValueError):
            stage_edits([bad], 5, 0.5)


def test_hinge_is_two_ball_joints_along_the_axis():
    # scenes.js:587-601: joints at anchor -+ span/2 along each body's axis
    from avbd_gb300 import AvbdScene3D
    sc = AvbdScene3D()
    a = sc.addBox([1, 1, 1], density=0, position=[0, 2, 0])
    b = sc.addBox([1, 1, 1], position=[0, 3.2, 0])
    h = sc.addHinge(a, b, anchorA=[0, 0.6, 0], anchorB=[0, -0.6, 0], axisA=[2, 0, 0], axisB=[1, 0, 0], span=0.8)
    arr = sc.arrays()
    assert h.joints == (0, 1) and h.limit is None and h.motor is None and list(arr.kind) == [0, 0]
    assert np.allclose(arr.ra, [[-0.4, 0.6, 0], [0.4, 0.6, 0]]) and np.allclose(arr.rb, [[-0.4, -0.6, 0], [0.4, -0.6, 0]])
    assert np.isinf(arr.p0).all() and np.all(arr.p1 == 0)
    with pytest.raises(ValueError):
        sc.addHinge(a, b, axisA=[0, 0, 0])


def test_hinge_limit_and_motor_records():
    # scenes.js:587-630 and angularConstraintOptions (src/gpu/angularConstraints.js:87-120): the
    # limit row (kind 4) carries the unit axes and the stops, the motor (kind 3) speed and torque
    from avbd_gb300 import AvbdScene3D
    sc = AvbdScene3D()
    a = sc.addBox([1, 1, 1], density=0, position=[0, 2, 0])
    b = sc.addBox([1, 1, 1], position=[0, 3.2, 0])
    sc.ignoreCollision(a, b)
    h = sc.addHinge(a, b, axisA=[0, 0, 3], axisB=[0, 0, 1], minAngle=-0.5, maxAngle=0.25,
                    motor={"speed": 2.0, "maxTorque": 40.0})
    m = sc.addMotor(None, b, axisA=[1, 0, 0], axisB=[1, 0, 0], speed=-1.0, maxTorque=0.0)
    arr = sc.arrays()
    assert h.joints == (1, 2) and h.limit == 3 and h.motor == 4 and m == 5
    assert list(arr.kind) == [2, 0, 0, 4, 3, 3]
    assert np.allclose(arr.ra[3], [0, 0, 1]) and np.allclose(arr.rb[3], [0, 0, 1])
    assert (arr.p0[3], arr.p1[3]) == (-0.5, 0.25) and (arr.p0[4], arr.p1[4]) == (2.0, 40.0)
    assert arr.ca[5] == -1 and (arr.p0[5], arr.p1[5]) == (-1.0, 0.0)
    for bad in ({"minAngle": 0.5, "maxAngle": 0.25}, {"minAngle": -4.0}, {"maxAngle": 3.2},
                {"motor": {"maxTorque": -1.0}}, {"motor": {"speed": float("inf")}}, {"motor": {"torque": 1.0}},
                {"minAngle": float("nan")}):
        with pytest.raises(ValueError):
            sc.addHinge(a, b, **bad)
    with pytest.raises(ValueError):
        sc.addMotor(a, b, axisA=[0, 0, 0])
    from avbd_gb300.pipeline import _motor_args, _motor_slot
    assert _motor_slot(arr.kind, 4) == 3 and _motor_slot(arr.kind, 5) == 4
    for c in (0, 1, 3, 6):
        with pytest.raises(ValueError):
            _motor_slot(arr.kind, c)
    assert _motor_args(None, 5.0) == (2, 0.0, 5.0) and _motor_args(1.5, None) == (1, 1.5, 0.0)
    with pytest.raises(ValueError):
        _motor_args(None, -1.0)


def test_spatial_sort_keeps_statics_first_and_remaps_constraints():
    import ref_scenes
    from avbd_gb300.pipeline import morton_order, spatial_sort
    sc = ref_scenes.build(13)  # boxes, a static ground, breakable joints
    ss = spatial_sort(sc)
    n = sc.n_bodies
    assert sorted(ss.order.tolist()) == list(range(n))
    assert np.array_equal(ss.pos, sc.pos[ss.order]) and np.array_equal(ss.mass, sc.mass[ss.order])
    nstatic = int(np.sum(sc.mass <= 0))
    assert np.all(ss.mass[:nstatic] <= 0) and np.all(ss.mass[nstatic:] > 0)
    slot = np.empty(n, dtype=np.int64)
    slot[ss.order] = np.arange(n)
    ca = np.where(sc.ca >= 0, slot[np.maximum(sc.ca, 0)], -1)
    assert np.array_equal(ss.ca, ca) and np.array_equal(ss.cb, slot[sc.cb])
    # the Morton key: 10 bits per axis over the bounds, ties by index
    pts = np.array([[0.0, 0, 0], [1, 1, 1], [1, 0, 0], [0, 1, 0], [0, 0, 1], [1, 0, 0]])
    assert morton_order(pts).tolist() == [0, 2, 5, 3, 4, 1]


def test_stage_properties_validation():
    from avbd_gb300.pipeline import stage_edits, stage_properties
    edits = [{"body": 1, "restitution": 0.5, "linearVelocity": [0, 1, 0]},
             {"body": 2, "group": 4, "collidesWith": 3}, {"body": 3, "allowSleep": False}]
    props = stage_properties(edits, 5)
    assert [p["index"] for p in props] == [1, 2, 3]
    assert props[0]["restitution"] == 0.5 and props[1]["group"] == 4 and props[2]["allowSleep"] is False
    assert stage_edits(edits, 5, 0.5, allow_properties=True).shape == (1, 12)
    assert stage_properties([{"body": 4, "isTrigger": True}], 5)[0]["isTrigger"] is True
    for bad in ({"body": 0, "restitution": 1.5}, {"body": 0, "collidesWith": 3}, {"body": 0, "allowSleep": 1},
                {"body": 0, "isTrigger": 1}, {"body": 7, "group": 1}):
        with pytest.raises(ValueError):
            stage_properties([bad], 5)


def test_advance_accumulator_matches_runtime_js():
    # runtime.js:238-272: at most maxSubSteps (6) steps, elapsed clamped to maxFrameTime (0.05 s)
    from avbd_gb300.pipeline import World
    taken = []

    class Fake:
        dt = 1 / 60
        timeAccumulator = 0.0
        _live = lambda self: None  # noqa: E731
        step = lambda self, n: taken.append(n)  # noqa: E731

    f = Fake()
    assert World.advance(f, 1.0) == 3 and taken == [3]  # 0.05 s -> 3 steps of 1/60
    assert World.advance(f, 0.01) == 0 and abs(f.timeAccumulator - 0.01) < 1e-12
    assert World.advance(f, 0.01) == 1
    import pytest as _pt
    with _pt.raises(ValueError):
        World.advance(f, -1.0)


def test_node_addon_compiles_against_the_node_api_declarations():
    # the addon (babylon-avbd_gb300/node/avbd_addon.cc) cannot be built without Node; its C++ is
    # checked here against declarations of the Node-API functions it calls and the real C ABI
    import shutil
    import subprocess
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([gxx, "-std=c++17", "-fsyntax-only", "-Wall", "-Wextra", "-Werror",
                        "-I", os.path.join(root, "tests", "napi_decl"), "-I", os.path.join(root, "include"),
                        "-DNODE_GYP_MODULE_NAME=avbd_gb300", os.path.join(root, "babylon-avbd_gb300", "node", "avbd_addon.cc")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
