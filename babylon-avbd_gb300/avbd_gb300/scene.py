"""Scene description: the reference's ``AvbdScene3D`` builder, restated.

Follows ``src/native/scenes.js:107-698`` (builder API, validation, defaults: density 1,
friction 0.6, Y up, mass override, rotation normalisation) and the mass properties of
``reference/three-avbd/src/avbd3d/ref/body.ts:32-54`` (box) and
``reference/three-avbd/src/avbd3d/shapes.ts:28-36`` (solid sphere). Arithmetic is done in
float64 in the same operation order as the JavaScript, so the numbers handed to the engine
are the ones the reference would compute; the engine stores them as float32.

A built scene is a set of flat structure-of-arrays (``SceneArrays``) that the C ABI
(``avbd_world_create``) consumes directly.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

SHAPE_BOX = 0
SHAPE_SPHERE = 1
SHAPE_CAPSULE = 2

KIND_JOINT = 0
KIND_SPRING = 1
KIND_IGNORE = 2
KIND_MOTOR = 3  # angular rows (src/gpu/angularConstraints.js info types 3 and 4)
KIND_LIMIT = 4

INF = math.inf
MASK_ALL = 0xFFFFFFFF


@dataclass
class SolverParams:
    """Solver settings (``reference/three-avbd/src/avbd3d/ref/solver.ts:347-359``,
    ``src/native/cpu/cpuSolver3D.ts:46-79``)."""

    dt: float = 1.0 / 60.0
    gravity: float = -10.0
    up: tuple = (0.0, 1.0, 0.0)
    iterations: int = 10
    alpha: float = 0.99
    beta_lin: float = 10000.0
    beta_ang: float = 100.0
    gamma: float = 0.999
    mass_penalty: bool = True
    face_bias: bool = True
    color_rounds: int = 64
    broadphase: str = "auto"  # "grid", "hploc" (the tree of gpuHploc.js) or "auto"; same pairs
    bvh_rebuild: int = 16     # steps between tree rebuilds; refit in between
    # island sleeping (src/native/cpu/sleeping.js:3-16): off unless enabled by the solver
    # options ({sleeping: true | {speedThreshold, timeThreshold}}) or a body's allowSleep: true
    sleeping: bool = False
    sleep_speed: float = 0.08  # m/s, |(v, w)|
    sleep_time: float = 0.6    # seconds of quiet before a body sleeps


@dataclass
class SceneArrays:
    """Flat per-body and per-constraint arrays, in creation order."""

    pos: np.ndarray
    quat: np.ndarray
    size: np.ndarray
    vel: np.ndarray
    angvel: np.ndarray
    prev_vel: np.ndarray
    mass: np.ndarray
    moment: np.ndarray
    friction: np.ndarray
    radius: np.ndarray
    shape: np.ndarray
    group: np.ndarray
    mask: np.ndarray
    kind: np.ndarray
    ca: np.ndarray
    cb: np.ndarray
    ra: np.ndarray
    rb: np.ndarray
    p0: np.ndarray
    p1: np.ndarray
    p2: np.ndarray
    params: SolverParams = field(default_factory=SolverParams)
    restitution: np.ndarray | None = None  # per body, 0..1 (None: all zero)
    allow_sleep: np.ndarray | None = None  # per body, bool (None: all may sleep)
    order: np.ndarray | None = None  # after a spatial sort: creation index of each body slot
    p3: np.ndarray | None = None  # per constraint: a spring's breakStrain (None: none anywhere)
    is_trigger: np.ndarray | None = None  # per body, bool (None: no triggers)

    def is_trigger_or_zero(self) -> np.ndarray:
        if self.is_trigger is None:
            return np.zeros(self.n_bodies, dtype=np.int32)
        return np.asarray(self.is_trigger).astype(np.int32)

    def p3_or_none(self) -> np.ndarray:
        """Spring strain limits (0: none), one per constraint."""
        return self.p3 if self.p3 is not None else np.zeros(self.n_cons, dtype=np.float64)

    def restitution_or_zero(self) -> np.ndarray:
        return self.restitution if self.restitution is not None else np.zeros(self.n_bodies, dtype=np.float64)

    def allow_sleep_or_one(self) -> np.ndarray:
        if self.allow_sleep is None:
            return np.ones(self.n_bodies, dtype=np.int32)
        return np.asarray(self.allow_sleep).astype(np.int32)

    @property
    def n_bodies(self) -> int:
        return int(self.pos.shape[0])

    @property
    def n_cons(self) -> int:
        return int(self.kind.shape[0])


class _Body:
    __slots__ = ("pos", "quat", "size", "vel", "angvel", "prev_vel", "mass", "moment",
                 "friction", "radius", "shape", "group", "mask", "restitution", "allow_sleep", "is_trigger")

    def __init__(self, size, density, friction, position, velocity=(0.0, 0.0, 0.0)):
        # body.ts:32-54
        sx, sy, sz = (float(v) for v in size)
        self.size = [sx, sy, sz]
        self.friction = float(friction)
        self.pos = [float(v) for v in position]
        self.quat = [0.0, 0.0, 0.0, 1.0]
        self.vel = [float(v) for v in velocity]
        self.prev_vel = [float(v) for v in velocity]
        self.angvel = [0.0, 0.0, 0.0]
        self.mass = sx * sy * sz * float(density)
        self.moment = [((sy * sy + sz * sz) / 12) * self.mass,
                       ((sx * sx + sz * sz) / 12) * self.mass,
                       ((sx * sx + sy * sy) / 12) * self.mass]
        a, b, c = sx * 0.5, sy * 0.5, sz * 0.5
        self.radius = math.sqrt(a * a + b * b + c * c)
        self.shape = SHAPE_BOX
        self.group = MASK_ALL
        self.mask = MASK_ALL
        self.restitution = 0.0
        self.allow_sleep = True
        self.is_trigger = False


class SceneBuilder:
    """Low-level creation-order builder shared by ``AvbdScene3D`` and the reference scenes."""

    def __init__(self, params: SolverParams | None = None):
        self.params = params or SolverParams()
        self.bodies: list[_Body] = []
        self.cons: list[tuple] = []

    # body.ts Rigid constructor
    def rigid(self, size, density, friction, position, velocity=(0.0, 0.0, 0.0)) -> int:
        self.bodies.append(_Body(size, density, friction, position, velocity))
        return len(self.bodies) - 1

    # shapes.ts:28-36
    def sphere(self, r, density, friction, position, velocity=(0.0, 0.0, 0.0)) -> int:
        r = float(r)
        i = self.rigid((2 * r, 2 * r, 2 * r), density, friction, position, velocity)
        b = self.bodies[i]
        b.mass = (4 / 3) * math.pi * r * r * r * float(density) if density > 0 else 0.0
        inertia = 0.4 * b.mass * r * r
        b.moment = [inertia, inertia, inertia]
        b.radius = r
        b.shape = SHAPE_SPHERE
        return i

    # src/gpu/capsuleShape.js:4-41: along local Y, height tip to tip
    def capsule(self, r, height, density, friction, position, velocity=(0.0, 0.0, 0.0)) -> int:
        r, height, density = float(r), float(height), float(density)
        i = self.rigid((2 * r, height, 2 * r), density, friction, position, velocity)
        b = self.bodies[i]
        length = height - 2 * r
        cylinder = math.pi * r * r * length * density
        caps = (4 / 3) * math.pi * r ** 3 * density
        b.mass = cylinder + caps
        axial = (cylinder * r ** 2) / 2 + (caps * 2 * r ** 2) / 5
        radial = (cylinder * (length ** 2 / 12 + r ** 2 / 4)
                  + caps * ((2 * r ** 2) / 5 + length ** 2 / 4 + (3 * length * r) / 8))
        b.moment = [radial, axial, radial]
        b.radius = height / 2
        b.shape = SHAPE_CAPSULE
        return i

    def joint(self, a, b, ra, rb, stiff_lin=INF, stiff_ang=0.0, fracture=INF) -> int:
        self.cons.append((KIND_JOINT, -1 if a is None else int(a), int(b), ra, rb,
                          float(stiff_lin), float(stiff_ang), float(fracture)))
        return len(self.cons) - 1

    def spring(self, a, b, ra, rb, stiffness, rest=-1.0, break_strain=INF, break_force=INF) -> int:
        self.cons.append((KIND_SPRING, int(a), int(b), ra, rb, float(stiffness), float(rest), float(break_force),
                          float(break_strain)))
        return len(self.cons) - 1

    def angular(self, kind, a, b, axis_a, axis_b, p0, p1) -> int:
        self.cons.append((int(kind), -1 if a is None else int(a), int(b), axis_a, axis_b, float(p0), float(p1), 0.0))
        return len(self.cons) - 1

    def ignore(self, a, b) -> int:
        self.cons.append((KIND_IGNORE, int(a), int(b), (0, 0, 0), (0, 0, 0), 0.0, 0.0, 0.0))
        return len(self.cons) - 1

    def arrays(self) -> SceneArrays:
        n = len(self.bodies)
        m = len(self.cons)
        B = self.bodies

        def f64(rows, width):
            a = np.zeros((n, width), dtype=np.float64)
            for i, r in enumerate(rows):
                a[i] = r
            return a

        return SceneArrays(
            pos=f64([b.pos for b in B], 3),
            quat=f64([b.quat for b in B], 4),
            size=f64([b.size for b in B], 3),
            vel=f64([b.vel for b in B], 3),
            angvel=f64([b.angvel for b in B], 3),
            prev_vel=f64([b.prev_vel for b in B], 3),
            mass=np.array([b.mass for b in B], dtype=np.float64),
            moment=f64([b.moment for b in B], 3),
            friction=np.array([b.friction for b in B], dtype=np.float64),
            radius=np.array([b.radius for b in B], dtype=np.float64),
            shape=np.array([b.shape for b in B], dtype=np.int32),
            group=np.array([b.group for b in B], dtype=np.uint32),
            mask=np.array([b.mask for b in B], dtype=np.uint32),
            kind=np.array([c[0] for c in self.cons], dtype=np.int32),
            ca=np.array([c[1] for c in self.cons], dtype=np.int32),
            cb=np.array([c[2] for c in self.cons], dtype=np.int32),
            ra=np.array([c[3] for c in self.cons], dtype=np.float64).reshape(m, 3),
            rb=np.array([c[4] for c in self.cons], dtype=np.float64).reshape(m, 3),
            restitution=np.array([b.restitution for b in B], dtype=np.float64),
            allow_sleep=np.array([b.allow_sleep for b in B], dtype=bool),
            is_trigger=np.array([b.is_trigger for b in B], dtype=bool),
            p0=np.array([c[5] for c in self.cons], dtype=np.float64),
            p1=np.array([c[6] for c in self.cons], dtype=np.float64),
            p2=np.array([c[7] for c in self.cons], dtype=np.float64),
            p3=np.array([c[8] if len(c) > 8 else 0.0 for c in self.cons], dtype=np.float64),
            params=self.params,
        )


@dataclass(frozen=True)
class Hinge:
    """addHinge's handle (scenes.js:620-629): the two ball joints' constraint indices, and the
    limit's and motor's (None when absent)."""
    joints: tuple
    limit: int | None = None
    motor: int | None = None


def _angular_options(kind, axisA=(0, 1, 0), axisB=(0, 1, 0), speed=1.0, maxTorque=100.0, minAngle=-math.pi,
                     maxAngle=math.pi) -> dict:
    """angularConstraintOptions (src/gpu/angularConstraints.js:87-120): unit axes, a finite speed
    and nonnegative torque bound, angles ordered within [-pi, pi]."""
    def unit(v):
        a = [float(x) for x in v]
        ln = math.hypot(*a) if len(a) == 3 else 0.0
        if len(a) != 3 or not all(math.isfinite(x) for x in a) or ln < 1e-8:
            raise ValueError("Angular axis requires three finite, nonzero components")
        return [x / ln for x in a]

    speed, maxTorque = float(speed), float(maxTorque)
    if not math.isfinite(speed) or not math.isfinite(maxTorque) or maxTorque < 0:
        raise ValueError("Motor speed must be finite and maxTorque nonnegative")
    minAngle, maxAngle = float(minAngle), float(maxAngle)
    if (not math.isfinite(minAngle) or not math.isfinite(maxAngle) or minAngle < -math.pi or maxAngle > math.pi
            or minAngle > maxAngle):
        raise ValueError("Hinge angles must be ordered within -PI..PI radians")
    return {"type": kind, "axisA": unit(axisA), "axisB": unit(axisB), "speed": speed, "maxTorque": maxTorque,
            "minAngle": minAngle, "maxAngle": maxAngle}


def spring_material(breakStrain=INF, breakForce=INF) -> dict:
    """springMaterial (src/gpu/springMaterial.js:4-13): each limit positive or infinite."""
    out = {}
    for name, v in (("breakStrain", breakStrain), ("breakForce", breakForce)):
        v = float(v)
        if v != INF and (not math.isfinite(v) or v <= 0):
            raise ValueError(f"{name} must be positive or Infinity")
        out[name] = v
    return out


def _vector(v, n, name):
    if v is None or len(v) != n:
        raise ValueError(f"{name} must have {n} components")
    out = [float(x) for x in v]
    if not all(math.isfinite(x) for x in out):
        raise ValueError(f"{name} must be finite")
    return out


def _positive(v, name, allow_zero=False):
    v = float(v)
    if not math.isfinite(v) or v < 0 or (v == 0 and not allow_zero):
        raise ValueError(f"{name} must be {'non-negative' if allow_zero else 'positive'}")
    return v


def _mask(v):
    v = int(v)
    if v < 0 or v > 0xFFFFFFFF:
        raise ValueError("collision masks are 32-bit unsigned integers")
    return v


class AvbdScene3D:
    """The reference's portable 3D scene builder (``src/native/scenes.js:107-698``).

    ``AvbdScene3D(timeStep=, iterations=, gravity=, up=)``; ``addBox(size, **options)`` with
    full XYZ extents; ``addSphere(radius, **options)``; ``addJoint(a, b, anchorA, anchorB,
    linearStiffness=inf, angularStiffness=0, breakForce=inf, breakOnPull=False)``;
    ``addSpring(a, b, anchorA, anchorB, stiffness=1000, rest=-1)``. Body handles are the
    creation-order indices. Invalid arguments raise ``ValueError`` synchronously, as the
    reference throws.
    """

    def __init__(self, timeStep=None, iterations=None, gravity=None, up=(0.0, 1.0, 0.0), **solver):
        p = SolverParams()
        if timeStep is not None:
            p.dt = _positive(timeStep, "timeStep")
        if iterations is not None:
            if int(iterations) != iterations or iterations <= 0:
                raise ValueError("iterations must be a positive integer")
            p.iterations = int(iterations)
        if gravity is not None:
            if not math.isfinite(gravity):
                raise ValueError("gravity must be finite")
            p.gravity = float(gravity)
        u = _vector(up, 3, "up")
        if abs(math.sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]) - 1) > 1e-5:
            raise ValueError("up must be a unit vector")
        p.up = tuple(u)
        for k, v in solver.items():
            if not hasattr(p, k):
                raise ValueError(f"unknown solver option {k}")
            setattr(p, k, v)
        self._b = SceneBuilder(p)
        self.created = False

    @property
    def params(self) -> SolverParams:
        return self._b.params

    @property
    def bodyCount(self) -> int:
        return len(self._b.bodies)

    def _editable(self):
        if self.created:
            raise RuntimeError("Build this scene before createSolver; use the world's edit methods afterwards")

    def _validate(self, options):
        allowed = {"density", "friction", "position", "rotation", "velocity", "angularVelocity",
                   "mass", "restitution", "isTrigger", "group", "collidesWith", "allowSleep"}
        for k in options:
            if k not in allowed:
                raise ValueError(f"unknown body option {k}")
        if "allowSleep" in options and not isinstance(options["allowSleep"], bool):
            raise ValueError("allowSleep must be a boolean")
        if "restitution" in options:
            e = options["restitution"]
            if not isinstance(e, (int, float)) or not math.isfinite(e) or e < 0 or e > 1:
                raise ValueError("restitution must be between 0 and 1")
        if "isTrigger" in options and not isinstance(options["isTrigger"], bool):
            raise ValueError("isTrigger must be a boolean")

    def addBox(self, size, **options) -> int:
        self._editable()
        self._validate(options)
        s = _vector(size, 3, "size")
        for v in s:
            _positive(v, "size")
        i = self._b.rigid(s, _positive(options.get("density", 1), "density", True),
                          _positive(options.get("friction", 0.6), "friction", True),
                          _vector(options.get("position", (0, 0, 0)), 3, "position"))
        return self._configure(i, options)

    def addSphere(self, radius, **options) -> int:
        self._editable()
        self._validate(options)
        i = self._b.sphere(_positive(radius, "radius"),
                           _positive(options.get("density", 1), "density", True),
                           _positive(options.get("friction", 0.6), "friction", True),
                           _vector(options.get("position", (0, 0, 0)), 3, "position"))
        return self._configure(i, options)

    def addCapsule(self, radius, height, **options) -> int:
        """An analytic capsule along local Y; height is the full tip-to-tip extent
        (scenes.js:180-193)."""
        self._editable()
        self._validate(options)
        r, h = float(radius), float(height)
        if not (math.isfinite(r) and r > 0 and math.isfinite(h) and h >= 2 * r):
            raise ValueError("Capsule height must be at least twice its positive radius")
        i = self._b.capsule(r, h, _positive(options.get("density", 1), "density", True),
                            _positive(options.get("friction", 0.6), "friction", True),
                            _vector(options.get("position", (0, 0, 0)), 3, "position"))
        return self._configure(i, options)

    def _configure(self, i, options) -> int:
        # scenes.js:233-273
        b = self._b.bodies[i]
        b.group = _mask(options.get("group", MASK_ALL))
        b.mask = _mask(options.get("collidesWith", MASK_ALL))
        b.restitution = float(options.get("restitution", 0.0))
        b.allow_sleep = bool(options.get("allowSleep", True))
        b.is_trigger = bool(options.get("isTrigger", False))
        if options.get("allowSleep") is True:  # scenes.js:240 sleepOptIn
            self._b.params.sleeping = True
        if "mass" in options:
            mass = _positive(options["mass"], "mass", True)
            if b.mass == 0 and mass > 0:
                raise ValueError("A positive mass needs positive density")
            ratio = mass / b.mass if b.mass > 0 else 0.0
            b.mass = mass
            b.moment = [v * ratio for v in b.moment]
        if options.get("rotation") is not None:
            q = _vector(options["rotation"], 4, "rotation")
            ln = math.hypot(*q)
            if not ln:
                raise ValueError("rotation must be nonzero")
            b.quat = [v / ln for v in q]
        if options.get("velocity") is not None:
            b.vel = _vector(options["velocity"], 3, "velocity")
        if options.get("angularVelocity") is not None:
            b.angvel = _vector(options["angularVelocity"], 3, "angularVelocity")
        return i

    def _check(self, a, b):
        n = len(self._b.bodies)
        if b is None or not (0 <= int(b) < n) or (a is not None and not (0 <= int(a) < n)):
            raise ValueError("joint bodies must belong to this scene")
        if a is not None and int(a) == int(b):
            raise ValueError("a constraint needs two different bodies")

    def addJoint(self, a, b, anchorA=(0, 0, 0), anchorB=(0, 0, 0), linearStiffness=INF,
                 angularStiffness=0.0, breakForce=INF, breakOnPull=False) -> int:
        # scenes.js:508-537
        self._editable()
        self._check(a, b)
        for v in (linearStiffness, angularStiffness, breakForce):
            if v != INF:
                _positive(v, "joint stiffness/breakForce", True)
        frac = -breakForce if (breakOnPull and breakForce != INF) else breakForce
        return self._b.joint(a, b, _vector(anchorA, 3, "anchorA"), _vector(anchorB, 3, "anchorB"),
                             linearStiffness, angularStiffness, frac)

    def addMotor(self, a, b, axisA=(0, 1, 0), axisB=(0, 1, 0), speed=1.0, maxTorque=100.0) -> int:
        """A torque-limited motor turning b about the hinge axis relative to a at `speed` rad/s
        (scenes.js:575-582); returns its constraint index."""
        self._editable()
        self._check(a, b)
        o = _angular_options("motor", axisA, axisB, speed, maxTorque)
        return self._b.angular(KIND_MOTOR, a, b, o["axisA"], o["axisB"], o["speed"], o["maxTorque"])

    def addHinge(self, a, b, anchorA=(0, 0, 0), anchorB=(0, 0, 0), axisA=(0, 1, 0), axisB=(0, 1, 0), span=1.0,
                 minAngle=None, maxAngle=None, motor=None, **options) -> "Hinge":
        """Two ball joints span apart along the axis, with optional angle stops and a motor
        (scenes.js:587-630). Anchors and axes are body-local, except the first endpoint's when a
        is None (world frame)."""
        self._editable()
        self._check(a, b)
        if options:
            raise ValueError(f"unknown hinge option {next(iter(options))}")
        lim = _angular_options("limit", axisA, axisB, minAngle=-math.pi if minAngle is None else minAngle,
                               maxAngle=math.pi if maxAngle is None else maxAngle)
        span = _positive(span, "span")
        ua, ub = lim["axisA"], lim["axisB"]
        aa, bb = _vector(anchorA, 3, "anchorA"), _vector(anchorB, 3, "anchorB")
        joints = tuple(self.addJoint(a, b, [aa[i] + sign * span * 0.5 * ua[i] for i in range(3)],
                                     [bb[i] + sign * span * 0.5 * ub[i] for i in range(3)])
                       for sign in (-1, 1))
        limit = None
        if minAngle is not None or maxAngle is not None:
            limit = self._b.angular(KIND_LIMIT, a, b, ua, ub, lim["minAngle"], lim["maxAngle"])
        drive = None
        if motor is not None:
            m = dict(motor)
            unknown = set(m) - {"speed", "maxTorque", "axisA", "axisB"}
            if unknown:
                raise ValueError(f"unknown motor option {sorted(unknown)[0]}")
            drive = self.addMotor(a, b, m.get("axisA", ua), m.get("axisB", ub), m.get("speed", 1.0),
                                  m.get("maxTorque", 100.0))
        return Hinge(joints, limit, drive)

    def addSpring(self, a, b, anchorA=(0, 0, 0), anchorB=(0, 0, 0), stiffness=1000.0, rest=-1.0,
                  breakStrain=INF, breakForce=INF) -> int:
        # scenes.js:541-569: a tensile spring that tears past breakStrain (extension / rest) or
        # breakForce (stiffness x extension)
        self._editable()
        self._check(a, b)
        if a is None:
            raise ValueError("A spring requires two bodies")
        _positive(stiffness, "stiffness", True)
        if rest != -1:
            _positive(rest, "rest", True)
        m = spring_material(breakStrain, breakForce)
        return self._b.spring(a, b, _vector(anchorA, 3, "anchorA"), _vector(anchorB, 3, "anchorB"),
                              stiffness, rest, m["breakStrain"], m["breakForce"])

    def ignoreCollision(self, a, b) -> int:
        """A pair that never gets a contact manifold (``ref/forces.ts:299-306``)."""
        self._editable()
        self._check(a, b)
        return self._b.ignore(a, b)

    def arrays(self) -> SceneArrays:
        return self._b.arrays()
