"""The reference's native world API over the GB300 engine.

Mirrors ``createSolverPipeline({backend})`` (``src/native/pipeline.js:14-92``) with a
``"gb300"`` backend, the world object's stepping, reads and writes (``src/native/scenes.d.ts:
317-454``, ``src/native/runtime.js:46-272``) and, as an addition the reference does not have,
batches of worlds stepped together. Every method validates its arguments before calling the
engine and raises ``ValueError`` (the reference throws synchronously); engine failures raise
``AvbdError``.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib as L
from .scene import AvbdScene3D, SceneArrays, _mask


def _with_options(arrays: SceneArrays, options) -> SceneArrays:
    import copy
    p = copy.copy(arrays.params)
    if "broadphase" in options:
        if options["broadphase"] not in L.BROADPHASE:
            raise ValueError("broadphase must be 'grid', 'hploc' or 'auto'")
        p.broadphase = options["broadphase"]
    if "bvh" in options:
        r = (options["bvh"] or {}).get("rebuildInterval", p.bvh_rebuild)
        if int(r) != r or r < 1:
            raise ValueError("BVH rebuildInterval must be a positive integer")
        p.bvh_rebuild = int(r)
    if "colorRounds" in options:
        r = options["colorRounds"]
        if int(r) != r or r < 1:
            raise ValueError("colorRounds must be a positive integer")
        p.color_rounds = int(r)
    if options.get("sleeping"):
        p.sleeping = True
        p.sleep_speed, p.sleep_time = _sleep_thresholds(options["sleeping"], p)
    out = copy.copy(arrays)
    out.params = p
    if "spatialSort" in options:
        if not isinstance(options["spatialSort"], bool):
            raise ValueError("spatialSort must be a boolean")
        if options["spatialSort"]:
            out = spatial_sort(out)
    return out


def morton_order(pos: np.ndarray) -> np.ndarray:
    """Body indices along a Z-order curve of their positions, 10 bits per axis, ties by index
    (mortonOrder, src/vendor/three-avbd-lib/solver3D.ts:344-367)."""
    n = len(pos)
    if n == 0:
        return np.zeros(0, dtype=np.int64)
    lo, hi = pos.min(axis=0), pos.max(axis=0)
    q = np.minimum(1023, np.floor((pos - lo) / np.maximum(hi - lo, 1e-9) * 1024)).astype(np.int64)

    def spread(v):
        x = v & 0x3FF
        x = (x | (x << 16)) & 0x30000FF
        x = (x | (x << 8)) & 0x300F00F
        x = (x | (x << 4)) & 0x30C30C3
        x = (x | (x << 2)) & 0x9249249
        return x

    code = spread(q[:, 0]) | (spread(q[:, 1]) << 1) | (spread(q[:, 2]) << 2)
    return np.lexsort((np.arange(n), code))


def spatial_sort(arrays: SceneArrays) -> SceneArrays:
    """The scene with its bodies in Morton order (the reference GPU solver's default body slots,
    solver3D.ts:564); constraints follow their bodies. ``order[slot]`` is the creation index.

    Static and large bodies (radius above twice the median, at most 64 of them: the engine's
    large-body rule) keep the first slots in creation order and only the rest are sorted: pairs are
    enumerated by their higher-index body, so a static ground or a large body in a late slot would
    enumerate most of its world on one thread."""
    import copy
    pos = np.asarray(arrays.pos, dtype=np.float64)
    n = len(pos)
    first = np.asarray(arrays.mass) <= 0
    if n:
        r = np.sort(np.asarray(arrays.radius, dtype=np.float64))
        thr = 2.0 * r[n // 2]
        if np.sum(r > thr) > 64:
            thr = r[n - 65]
        first |= np.asarray(arrays.radius) > thr
    head = np.nonzero(first)[0]
    rest = np.nonzero(~first)[0]
    order = np.concatenate([head, rest[morton_order(pos[rest])]]).astype(np.int64)
    slot = np.empty_like(order)
    slot[order] = np.arange(len(order))
    out = copy.copy(arrays)
    for k in ("pos", "quat", "size", "vel", "angvel", "prev_vel", "mass", "moment", "friction", "radius",
              "shape", "group", "mask"):
        setattr(out, k, np.asarray(getattr(arrays, k))[order])
    for k in ("restitution", "allow_sleep", "is_trigger"):
        v = getattr(arrays, k)
        setattr(out, k, None if v is None else np.asarray(v)[order])
    if arrays.n_cons:
        ca = np.asarray(arrays.ca)
        out.ca = np.where(ca >= 0, slot[np.maximum(ca, 0)], -1).astype(ca.dtype)
        out.cb = slot[np.asarray(arrays.cb)].astype(np.asarray(arrays.cb).dtype)
    base = arrays.order if getattr(arrays, "order", None) is not None else np.arange(len(order))
    out.order = np.asarray(base)[order]
    return out


def _sleep_thresholds(opt, p):
    """(speed, time) of a sleeping option: true or {speedThreshold, timeThreshold}
    (src/native/cpu/sleeping.js:3-10)."""
    if opt is True:
        return 0.08, 0.6
    if not isinstance(opt, dict):
        raise ValueError("sleeping must be true or an options object")
    speed = opt.get("speedThreshold", 0.08)
    time = opt.get("timeThreshold", 0.6)
    for v in (speed, time):
        if not isinstance(v, (int, float)) or not np.isfinite(v) or v <= 0:
            raise ValueError("Sleep thresholds must be positive and finite")
    return float(speed), float(time)


def _watch_args(options, body_count):
    """(indices array or None, n, maxPairs, maxEvents) of watchContacts({indices, maxPairs,
    maxEvents}) (src/native/solver3D.js:256-284)."""
    options = options or {}
    max_pairs = options.get("maxPairs", 8192)
    max_events = options.get("maxEvents", 4096)
    for v in (max_pairs, max_events):
        if not isinstance(v, (int, np.integer)) or isinstance(v, bool) or v < 1:
            raise ValueError("Contact capacities must be positive integers")
    idx = options.get("indices")
    if idx is None:
        return None, 0, int(max_pairs), int(max_events)
    if not isinstance(idx, (list, tuple, np.ndarray)):
        raise ValueError("Watched indices must be an array")
    arr = np.ascontiguousarray(np.asarray(idx, dtype=np.int64))
    if arr.size and (arr.min() < 0 or arr.max() >= body_count):
        raise ValueError("A live body index is required")
    arr = np.ascontiguousarray(arr.astype(np.uint32))
    return arr, int(arr.size), int(max_pairs), int(max_events)


def _read_events(fn, *args) -> dict:
    """readContactEvents(): {events, dropped, full} with events as the reference reports them
    (type "begin"/"end", kind, a, b, step, point, normal, impulse, isTrigger)."""
    raw = _read_events_raw(fn, *args)
    ev = raw["records"]
    f = ev.view(np.float32)
    events = [{"type": "begin" if r[0] == 1 else "end", "kind": int(r[0]), "a": int(r[1]), "b": int(r[2]),
               "step": int(r[3]), "point": [float(x) for x in f[k, 4:7]], "impulse": float(f[k, 7]),
               "normal": [float(x) for x in f[k, 8:11]], "isTrigger": bool(f[k, 11] != 0)}
              for k, r in enumerate(ev)]
    return {"events": events, "dropped": raw["dropped"], "full": raw["full"]}


def _read_events_raw(fn, *args) -> dict:
    n, dropped, full = C.c_int64(), C.c_int64(), C.c_int32()
    L.check(fn(*args, None, 0, C.byref(n), C.byref(dropped), C.byref(full)))
    out = np.zeros((n.value, 12), dtype=np.uint32)
    L.check(fn(*args, L.uptr(out), n.value, C.byref(n), C.byref(dropped), C.byref(full)))
    return {"records": out[: n.value], "dropped": int(dropped.value), "full": bool(full.value)}


def _cast_filter(options, body_count) -> "L.CastFilter":
    """The body filter of a cast ({ignore, collidesWith, membership, includeTriggers},
    src/gpu/shapeQueries.js:97-135)."""
    options = options or {}
    cw = options.get("collidesWith", 0xFFFFFFFF)
    if not isinstance(cw, (int, np.integer)) or isinstance(cw, bool) or not 0 <= cw <= 0xFFFFFFFF:
        raise ValueError("Query mask must be an unsigned 32-bit integer")
    it = options.get("includeTriggers", True)
    if not isinstance(it, bool):
        raise ValueError("includeTriggers must be boolean")
    mem = options.get("membership")
    if mem is not None and (not isinstance(mem, (int, np.integer)) or isinstance(mem, bool) or not 0 <= mem <= 0xFFFFFFFF):
        raise ValueError("Query membership must be an unsigned 32-bit integer")
    ign = list(options.get("ignore", []))
    if len(ign) > 16 or any(not isinstance(i, (int, np.integer)) or not 0 <= i < body_count for i in ign):
        raise ValueError("Queries can ignore up to 16 live body indices")
    f = L.CastFilter()
    f.collides_with = int(cw)
    f.membership = 0 if mem is None else int(mem)
    f.has_membership = 0 if mem is None else 1
    f.include_triggers = int(it)
    f.n_ignore = len(ign)
    for k, i in enumerate(ign):
        f.ignore[k] = int(i)
    return f


def _cast(fn, args, casts, options, body_count):
    """sphereCastAll: [{origin, direction, radius?, maxDistance?}] -> [hit or None]; a hit is
    {index, distance, normal, center, point}."""
    options = options or {}
    q = np.zeros((len(casts), 8), dtype=np.float32)
    dirs = []
    for k, c in enumerate(casts):
        o = np.asarray(c["origin"], dtype=np.float64)
        d = np.asarray(c["direction"], dtype=np.float64)
        r = c.get("radius", 0.0) or 0.0
        md = c.get("maxDistance", options.get("maxDistance", 3e38))
        if o.shape != (3,) or d.shape != (3,) or not np.all(np.isfinite(o)) or not np.all(np.isfinite(d)) \
                or not np.linalg.norm(d):
            raise ValueError("A query requires 3 finite components and a nonzero direction")
        if not np.isfinite(r) or r < 0 or not np.isfinite(md) or md < 0:
            raise ValueError("Query radius and maximum distance must be finite and nonnegative")
        q[k] = [*o, md, *d, r]
        dirs.append((o, d / np.linalg.norm(d), float(r)))
    if not len(casts):
        return []
    f = _cast_filter(options, body_count)
    hits = np.zeros((len(casts), 8), dtype=np.float32)
    L.check(fn(*args, L.fptr(q), len(casts), C.byref(f), L.fptr(hits)))
    idx = hits.view(np.uint32)[:, 4]
    out = []
    for k, (o, d, r) in enumerate(dirs):
        t = float(hits[k, 3])
        if t < 0:
            out.append(None)
            continue
        n = hits[k, :3].astype(np.float64)
        center = o + t * d
        out.append({"index": int(idx[k]), "distance": t, "normal": n.tolist(), "center": center.tolist(),
                    "point": (center - r * n).tolist()})
    return out


def _arrays(scene) -> SceneArrays:
    if isinstance(scene, AvbdScene3D):
        scene.created = True
        return scene.arrays()
    if isinstance(scene, SceneArrays):
        return scene
    raise ValueError("expected an AvbdScene3D or SceneArrays")


class Fence:
    """onSubmittedWorkDone as a value: ``wait()`` blocks until the device passes it (thread-safe,
    so a worker thread may wait while the caller keeps queuing steps); ``done`` polls."""

    def __init__(self, h):
        self._h = h

    def wait(self):
        L.check(L.lib().avbd_fence_wait(self._h))

    @property
    def done(self) -> bool:
        d = C.c_int32()
        L.check(L.lib().avbd_fence_query(self._h, C.byref(d)))
        return bool(d.value)

    def destroy(self):
        if self._h is not None:
            L.check(L.lib().avbd_fence_destroy(self._h))
            self._h = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


class SolverPipeline:
    """A device context owning worlds and batches; ``destroy()`` releases all of them."""

    backend = "gb300"

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        L.check(L.lib().avbd_ctx_create(int(device), C.byref(h)))
        self._h = h
        self._children = []

    def _live(self):
        if self._h is None:
            raise RuntimeError("The pipeline has been destroyed")

    @property
    def stream(self) -> int:
        """The engine's cudaStream_t (as an integer handle)."""
        self._live()
        h = C.c_void_p()
        L.check(L.lib().avbd_ctx_stream(self._h, C.byref(h)))
        return int(h.value or 0)

    def synchronize(self):
        self._live()
        L.check(L.lib().avbd_ctx_synchronize(self._h))

    def fence(self) -> "Fence":
        """A fence after the work queued so far; ``wait()`` may run on another thread."""
        self._live()
        h = C.c_void_p()
        L.check(L.lib().avbd_ctx_fence(self._h, C.byref(h)))
        return Fence(h)

    def createSolver(self, scene, options=None) -> "World":
        """``pipeline.createSolver(scene, options)``; options ``broadphase`` ("auto", "grid",
        "hploc"), ``bvh: {rebuildInterval}`` and ``colorRounds`` as in AvbdGpuOptions
        (``src/native/scenes.d.ts:288-310``)."""
        self._live()
        arrays = _arrays(scene)
        if options:
            unknown = set(options) - {"spatialSort", "broadphase", "bvh", "colorRounds", "sleeping"}
            if unknown:
                raise ValueError(f"unsupported solver options {sorted(unknown)}")
            arrays = _with_options(arrays, options)
        w = World(self, arrays)
        self._children.append(w)
        return w

    def createBatch(self, scenes) -> "Batch":
        self._live()
        b = Batch(self, [_arrays(s) for s in scenes])
        self._children.append(b)
        return b

    def createServer(self, budgetBytes: int, initialBodies: int = 0, initialWorlds: int = 0) -> "Server":
        """A world server holding at most ``budgetBytes`` of device memory (see ``Server``)."""
        self._live()
        if not (isinstance(budgetBytes, (int, np.integer)) and budgetBytes > 0):
            raise ValueError("budgetBytes must be a positive integer")
        s = Server(self, int(budgetBytes), int(initialBodies), int(initialWorlds))
        self._children.append(s)
        return s

    def destroy(self):
        if self._h is None:
            return
        for c in self._children:
            c._h = None  # freed with the context
        self._children.clear()
        L.check(L.lib().avbd_ctx_destroy(self._h))
        self._h = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


def createSolverPipeline(backend: str = "gb300", device: int = 0) -> SolverPipeline:
    """``createSolverPipeline({backend: "gb300"})``; the reference's "webgpu" and "cpu"
    backends are not part of this engine."""
    if backend != "gb300":
        raise ValueError('backend must be "gb300"')
    return SolverPipeline(device)


# Body command kinds in the order of the reference's command shaders (src/native/runtime.js:36-44);
# kind 4 is the teleport.
_EDIT_KEYS = ["linearVelocity", "angularVelocity", "impulse", "force", "", "angularImpulse", "torque"]


def _components(value, count, name):
    try:
        a = [float(x) for x in (value.tolist() if isinstance(value, np.ndarray) else value)]
    except TypeError:
        raise ValueError(f"{name} requires {count} finite components") from None
    if len(a) != count or not all(math.isfinite(x) for x in a):
        raise ValueError(f"{name} requires {count} finite components")
    return a


def stage_properties(edits, body_count: int) -> list:
    """The property part of ``editBodies`` (``src/native/runtime.js:72-103``): per edit with any
    of restitution / group / collidesWith / allowSleep, validated, in edit order."""
    out = []
    for edit in edits:
        keys = {"isTrigger", "restitution", "group", "collidesWith", "allowSleep"} & set(edit)
        if not keys:
            continue
        index = edit.get("body")
        if not isinstance(index, (int, np.integer)) or not 0 <= int(index) < body_count:
            raise ValueError("A live body index is required")
        if "isTrigger" in edit and not isinstance(edit["isTrigger"], bool):
            raise ValueError("isTrigger must be a boolean")
        if "allowSleep" in edit and not isinstance(edit["allowSleep"], bool):
            raise ValueError("allowSleep must be a boolean")
        e = edit.get("restitution")
        if e is not None and (not isinstance(e, (int, float)) or not np.isfinite(e) or not 0 <= e <= 1):
            raise ValueError("restitution must be between 0 and 1")
        if "collidesWith" in edit and "group" not in edit:
            raise ValueError("A collision-mask edit requires group as well")
        for k in ("group", "collidesWith"):
            if k in edit:
                _mask(edit[k])
        out.append({"index": int(index), "restitution": e, "group": edit.get("group"),
                    "collidesWith": edit.get("collidesWith", 0xFFFFFFFF), "allowSleep": edit.get("allowSleep"),
                    "isTrigger": edit.get("isTrigger")})
    return out


def stage_edits(edits, body_count: int, dt: float, allow_properties: bool = False) -> np.ndarray:
    """``editBodies(edits)`` records (``src/native/runtime.js:62-167``): the whole batch is
    validated before anything is queued; per edit the teleport comes first, then velocity
    replacements, impulses and forces in kind order. Returns (n, 12) uint32 words. Property keys
    (restitution, group, collidesWith, allowSleep) are left to ``stage_properties`` when
    ``allow_properties``, else refused."""
    words = []
    unsupported = set() if allow_properties else {"isTrigger", "restitution", "allowSleep", "group", "collidesWith"}

    def record(index, kind, value, point):
        w = np.zeros(12, dtype=np.uint32)
        f = w.view(np.float32)
        w[0], w[1], w[2] = index, kind, int(point is not None)
        f[4:4 + len(value)] = value
        if point is not None:
            f[8:8 + len(point)] = point
        if kind in (3, 6):
            f[7] = dt
        return w

    for edit in edits:
        index = edit.get("body")
        if not isinstance(index, (int, np.integer)) or not 0 <= int(index) < body_count:
            raise ValueError("A live body index is required")
        index = int(index)
        bad = unsupported & set(edit)
        if bad:
            raise ValueError(f"body property edits {sorted(bad)} are not part of this engine")
        point = None if edit.get("worldPoint") is None else _components(edit["worldPoint"], 3, "worldPoint")
        if edit.get("position") is not None:
            p = _components(edit["position"], 3, "position")
            q = None
            if edit.get("rotation") is not None:
                q = _components(edit["rotation"], 4, "rotation")
                ln = math.hypot(*q)
                if not ln:
                    raise ValueError("rotation must be nonzero")
                q = [v / ln for v in q]
            words.append(record(index, 4, p, q))
        elif edit.get("rotation") is not None:
            raise ValueError("A rotation edit requires position; use teleport for a full pose")
        for kind, key in enumerate(_EDIT_KEYS):
            if kind == 4 or edit.get(key) is None:
                continue
            v = _components(edit[key], 3, key)
            words.append(record(index, kind, v, point if kind in (2, 3) else None))
    return np.stack(words) if words else np.zeros((0, 12), dtype=np.uint32)


def _motor_slot(kinds, constraint) -> int:
    """Joint slot (index among joints, springs and angular rows) of a motor's constraint index."""
    from .scene import KIND_IGNORE, KIND_MOTOR
    c = int(constraint)
    if not 0 <= c < len(kinds) or kinds[c] != KIND_MOTOR:
        raise ValueError("Motor needs an active motor slot")
    return int(np.count_nonzero(kinds[:c] != KIND_IGNORE))


def _joint_slots(kinds, constraints) -> np.ndarray:
    """Joint slots of constraint indices (ignore-collision pairs have none)."""
    from .scene import KIND_IGNORE
    c = np.asarray(constraints, dtype=np.int64).reshape(-1)
    if c.size and (c.min() < 0 or c.max() >= len(kinds) or np.any(kinds[c] == KIND_IGNORE)):
        raise ValueError("A live constraint slot is required")
    before = np.cumsum(kinds != KIND_IGNORE) - 1
    return np.ascontiguousarray(before[c].astype(np.int32))


def _motor_args(speed, maxTorque):
    mask, sp, mt = 0, 0.0, 0.0
    if speed is not None:
        sp = float(speed)
        if not math.isfinite(sp):
            raise ValueError("Motor speed must be finite")
        mask |= 1
    if maxTorque is not None:
        mt = float(maxTorque)
        if not (math.isfinite(mt) and mt >= 0):
            raise ValueError("maxTorque must be nonnegative")
        mask |= 2
    return mask, sp, mt


def _indices(indices, n):
    idx = np.ascontiguousarray(np.asarray(indices, dtype=np.int64).reshape(-1))
    if idx.size and (idx.min() < 0 or idx.max() >= n):
        raise ValueError("body index out of range")
    return idx.astype(np.uint32)


class Body:
    """A handle on the body in slot `index` of a world (``world.body(i)``; NativeBody of
    src/native/runtime.js:169-237): the world's per-body commands, each returning the handle."""

    def __init__(self, world: "World", index: int):
        self.world = world
        self.index = int(index)

    @property
    def gpuIndex(self) -> int:
        """The body's slot (the index every world call takes)."""
        return self.index

    def setLinearVelocity(self, v):
        self.world.setLinearVelocity(self.index, v)
        return self

    def setAngularVelocity(self, v):
        self.world.setAngularVelocity(self.index, v)
        return self

    def applyImpulse(self, v, p=None):
        self.world.applyImpulse(self.index, v, p)
        return self

    def applyForce(self, v, p=None):
        self.world.applyForce(self.index, v, p)
        return self

    def applyAngularImpulse(self, v):
        self.world.applyAngularImpulse(self.index, v)
        return self

    def applyTorque(self, v):
        self.world.applyTorque(self.index, v)
        return self

    def teleport(self, position, rotation=None):
        self.world.teleport(self.index, position, rotation)
        return self

    def setRestitution(self, value):
        self.world.setRestitution([self.gpuIndex], [value])
        return self

    def setTrigger(self, enabled):
        self.world.setSensor(self.index, enabled)
        return self

    def setCollisionGroups(self, group, collidesWith=0xFFFFFFFF):
        self.world.setFilters([self.gpuIndex], [group], [collidesWith])
        return self

    def setSleepEnabled(self, enabled):
        self.world.setSleepEnabled(self.index, enabled)
        return self

    def wakeUp(self):
        self.world.wakeUp(self.index)
        return self

    def readState(self) -> dict:
        """This body's state as world.readBodyState(index) gives it (runtime.js:234-236)."""
        return self.world.readBodyState(self.index)


class World:
    """One world (``pipeline.createSolver(scene)``)."""

    def __init__(self, pipe: SolverPipeline, arrays: SceneArrays):
        self._pipe = pipe
        self._packed = L.PackedScene(arrays)
        h = C.c_void_p()
        L.check(L.lib().avbd_world_create(pipe._h, C.byref(self._packed.desc), C.byref(self._packed.params), C.byref(h)))
        self._h = h
        self.bodyCount = arrays.n_bodies
        self.jointCount = self._packed.n_joints
        self._kinds = np.asarray(arrays.kind, dtype=np.int32).copy()
        self.dt = float(arrays.params.dt)
        # body slots: creation order, or Morton order with spatialSort (order[slot] = creation index)
        order = getattr(arrays, "order", None)
        self._slot = None
        if order is not None:
            self._slot = np.empty(len(order), dtype=np.int64)
            self._slot[np.asarray(order)] = np.arange(len(order))
        self.timeAccumulator = 0.0

    def _live(self):
        if self._h is None:
            raise RuntimeError("The solver has been destroyed")

    # stepping ---------------------------------------------------------------
    def step(self, steps: int = 1):
        self._live()
        if int(steps) != steps or steps < 0:
            raise ValueError("steps must be a non-negative integer")
        L.check(L.lib().avbd_world_step(self._h, int(steps)))
        return self

    def advance(self, elapsed: float, maxSubSteps: int = 6, maxFrameTime: float = 0.05) -> int:
        """Fixed-step accumulator (``src/native/runtime.js:238-272``, defaults maxSubSteps 6 and
        maxFrameTime 0.05 s); returns steps taken."""
        self._live()
        if not math.isfinite(elapsed) or elapsed < 0:
            raise ValueError("elapsed must be finite nonnegative seconds")
        if int(maxSubSteps) != maxSubSteps or maxSubSteps < 1 or not math.isfinite(maxFrameTime) or maxFrameTime <= 0:
            raise ValueError("Stepping limits must be positive")
        dt = self.dt
        self.timeAccumulator = min(maxSubSteps * dt, self.timeAccumulator + min(maxFrameTime, elapsed))
        count = 0
        while self.timeAccumulator + 1e-12 >= dt and count < maxSubSteps:
            count += 1
            self.timeAccumulator = max(0.0, self.timeAccumulator - dt)
        if count:
            self.step(count)
        return count

    # reads --------------------------------------------------------------------
    def readBodyState(self, index=None) -> dict:
        """With a body slot: the reference's state of that body (src/native/cpu/world.js:572-588:
        position, rotation, linearVelocity, angularVelocity, mass, effectiveMass, sleeping).
        Without one: positions, rotations, velocities, angular and previous velocities of every
        body (float32 arrays)."""
        self._live()
        if index is not None:
            i = int(_indices([index], self.bodyCount)[0])
            rec = self.readSelectedBodies([i]).reshape(40)
            sleeping = bool(self.readSleepState()[0][i])
            return {"position": [float(x) for x in rec[0:3]], "rotation": [float(x) for x in rec[4:8]],
                    "linearVelocity": [float(x) for x in rec[32:35]],
                    "angularVelocity": [float(x) for x in rec[36:39]],
                    "mass": float(self._packed.keep[6][i]), "effectiveMass": float(rec[19]), "sleeping": sleeping}
        n = self.bodyCount
        out = {k: np.zeros((n, 4 if k == "rotation" else 3), dtype=np.float32)
               for k in ("position", "rotation", "velocity", "angular", "prev_velocity")}
        L.check(L.lib().avbd_world_read_state(self._h, *(L.fptr(out[k]) for k in
                                                         ("position", "rotation", "velocity", "angular", "prev_velocity"))))
        return out

    def readSelectedBodies(self, indices, posesOnly: bool = False) -> np.ndarray:
        """8 floats per body (pos, friction, quat) or the 40-float body record."""
        self._live()
        idx = _indices(indices, self.bodyCount)
        stride = 8 if posesOnly else 40
        out = np.zeros(idx.size * stride, dtype=np.float32)
        L.check(L.lib().avbd_world_read_selected(self._h, L.uptr(idx), idx.size, int(bool(posesOnly)), L.fptr(out)))
        return out

    def readBodies(self) -> np.ndarray:
        return self.readSelectedBodies(np.arange(self.bodyCount))

    # ---- body commands (src/native/runtime.js:46-167, src/native/cpu/world.js:145-166)
    def editBodies(self, edits):
        """Queue a validated batch of body edits for the next step; property edits apply after the
        commands in runtime.js:157-165's order (isTrigger, restitution, group/collidesWith,
        allowSleep)."""
        self._live()
        edits = list(edits)
        props = stage_properties(edits, self.bodyCount)
        rec = stage_edits(edits, self.bodyCount, self.dt, allow_properties=True)
        if len(rec):
            L.check(L.lib().avbd_world_edit(self._h, L.uptr(rec), int(rec.shape[0])))
        for p in props:
            if p["isTrigger"] is not None:
                self.setSensor(p["index"], p["isTrigger"])
            if p["restitution"] is not None:
                self.setRestitution([p["index"]], [p["restitution"]])
            if p["group"] is not None:
                self.setFilters([p["index"]], [p["group"]], [p["collidesWith"]])
            if p["allowSleep"] is not None:
                self.setSleepEnabled(p["index"], p["allowSleep"])
        return self

    def body(self, index) -> Body:
        """A handle on the body in slot `index` (runtime.js:345-350; gpuIndex maps a creation index)."""
        if not 0 <= int(index) < self.bodyCount:
            raise ValueError("A live body index is required")
        return Body(self, int(index))

    def setMotor(self, constraint, speed=None, maxTorque=None):
        """setMotor (src/gpu/appGpuSolver3D.js:547-562): a new speed and/or torque bound of the
        motor created as constraint index `constraint` (addMotor, or a Hinge's motor); wakes the
        world."""
        self._live()
        slot = _motor_slot(self._kinds, constraint)
        mask, sp, mt = _motor_args(speed, maxTorque)
        L.check(L.lib().avbd_world_set_motor(self._h, slot, mask, sp, mt))

    def releaseJoints(self, constraints):
        """releaseJoints (src/native/cpu/world.js:397-410): the constraints at these constraint
        indices (joints, springs, motors, limits) stop acting; wakes the world."""
        self._live()
        slots = _joint_slots(self._kinds, constraints)
        L.check(L.lib().avbd_world_release_joints(self._h, L.iptr(slots), int(slots.size)))

    def disableConstraint(self, constraint):
        """disableConstraint (src/native/cpu/world.js:400-410): releaseJoints of one constraint."""
        self.releaseJoints([constraint])

    def setSpringMaterial(self, constraint, breakStrain=None, breakForce=None):
        """setSpringMaterial (src/gpu/appGpuSolver3D.js:810-835): new tear limits of a live spring
        (positive, or math.inf for none); wakes the world."""
        self._live()
        from .scene import KIND_SPRING, spring_material
        c = int(constraint)
        if not 0 <= c < len(self._kinds) or self._kinds[c] != KIND_SPRING:
            raise ValueError("Spring material requires an active spring slot")
        m = spring_material(math.inf if breakStrain is None else breakStrain,
                            math.inf if breakForce is None else breakForce)
        mask = (1 if breakStrain is not None else 0) | (2 if breakForce is not None else 0)
        slot = int(_joint_slots(self._kinds, [c])[0])
        L.check(L.lib().avbd_world_set_spring_material(self._h, slot, mask, m["breakStrain"], m["breakForce"]))

    def setWorldAnchor(self, constraint, point):
        """setWorldAnchor (src/gpu/appGpuSolver3D.js:928-941): move the world point of a joint whose
        first body is the world (a grab handle); wakes the world."""
        self._live()
        p = np.ascontiguousarray(np.asarray(point, dtype=np.float32).reshape(-1))
        if p.size != 3 or not np.all(np.isfinite(p)):
            raise ValueError("A world joint and finite xyz anchor are required")
        slot = int(_joint_slots(self._kinds, [constraint])[0])
        L.check(L.lib().avbd_world_set_world_anchor(self._h, slot, L.fptr(p)))

    def captureConstraintFrames(self, entries):
        """captureConstraintFrames (src/native/cpu/world.js:474-492): entries are constraint indices
        or {"slot": constraint, "spring": bool}; each live joint's rest rotation, or spring's rest
        length, is taken again from the current poses."""
        self._live()
        cons, spring = [], []
        for e in entries:
            if isinstance(e, dict):
                cons.append(int(e["slot"]))
                spring.append(1 if e.get("spring") else 0)
            else:
                cons.append(int(e))
                spring.append(0)
        slots = _joint_slots(self._kinds, cons)
        sp = np.ascontiguousarray(np.asarray(spring, dtype=np.int32))
        L.check(L.lib().avbd_world_capture_frames(self._h, L.iptr(slots), L.iptr(sp), int(slots.size)))

    def setSensor(self, index, enabled):
        """setSensor (src/native/cpu/world.js:342-350): the body becomes (or stops being) a
        trigger: its contacts are reported but apply no forces; wakes the world."""
        self._live()
        if not isinstance(enabled, bool):
            raise ValueError("isTrigger must be a boolean")
        idx = _indices([index], self.bodyCount)
        L.check(L.lib().avbd_world_set_sensor(self._h, L.uptr(idx), 1, int(enabled)))

    def setRestitution(self, indices, values):
        self._live()
        idx = np.ascontiguousarray(np.asarray(indices, dtype=np.int64).reshape(-1))
        val = np.ascontiguousarray(np.asarray(values, dtype=np.float32).reshape(-1))
        if idx.size != val.size:
            raise ValueError("Restitution arrays must have matching lengths")
        if idx.size and (idx.min() < 0 or idx.max() >= self.bodyCount):
            raise ValueError("A live body index is required")
        if not np.all((val >= 0) & (val <= 1)):
            raise ValueError("restitution must be between 0 and 1")
        ia = np.ascontiguousarray(idx.astype(np.uint32))
        L.check(L.lib().avbd_world_set_restitution(self._h, L.uptr(ia), int(ia.size), L.fptr(val)))
        return self

    def editRecords(self, records):
        """Queue already-staged command records (n x 12 uint32 words, see ``stage_edits``)."""
        self._live()
        rec = np.ascontiguousarray(records, dtype=np.uint32).reshape(-1, 12)
        if len(rec):
            L.check(L.lib().avbd_world_edit(self._h, L.uptr(rec), int(rec.shape[0])))
        return self

    def flushEdits(self):
        self._live()
        L.check(L.lib().avbd_world_flush_edits(self._h))
        return self

    def setLinearVelocity(self, index, value):
        return self.editBodies([{"body": index, "linearVelocity": value}])

    def setAngularVelocity(self, index, value):
        return self.editBodies([{"body": index, "angularVelocity": value}])

    def applyImpulse(self, index, value, worldPoint=None):
        return self.editBodies([{"body": index, "impulse": value, "worldPoint": worldPoint}])

    def applyForce(self, index, value, worldPoint=None):
        return self.editBodies([{"body": index, "force": value, "worldPoint": worldPoint}])

    def applyAngularImpulse(self, index, value):
        return self.editBodies([{"body": index, "angularImpulse": value}])

    def applyTorque(self, index, value):
        return self.editBodies([{"body": index, "torque": value}])

    def teleport(self, index, position, rotation=None):
        return self.editBodies([{"body": index, "position": position, "rotation": rotation}])

    def readCounters(self) -> dict:
        self._live()
        c = L.Counters()
        L.check(L.lib().avbd_world_counters(self._h, C.byref(c)))
        return {k: getattr(c, k) for k, _ in L.Counters._fields_}

    # writes -------------------------------------------------------------------
    def setPoses(self, indices, positions, rotations=None):
        self._live()
        idx = _indices(indices, self.bodyCount)
        p = np.ascontiguousarray(np.asarray(positions, dtype=np.float32).reshape(idx.size, 3))
        r = None if rotations is None else np.ascontiguousarray(np.asarray(rotations, dtype=np.float32).reshape(idx.size, 4))
        if not np.isfinite(p).all() or (r is not None and (not np.isfinite(r).all() or (np.abs(r).sum(1) == 0).any())):
            raise ValueError("poses must be finite and rotations nonzero")
        L.check(L.lib().avbd_world_set_poses(self._h, L.uptr(idx), idx.size, L.fptr(p), L.fptr(r)))

    def setVelocities(self, indices, linear=None, angular=None):
        self._live()
        idx = _indices(indices, self.bodyCount)
        v = None if linear is None else np.ascontiguousarray(np.asarray(linear, dtype=np.float32).reshape(idx.size, 3))
        a = None if angular is None else np.ascontiguousarray(np.asarray(angular, dtype=np.float32).reshape(idx.size, 3))
        for x in (v, a):
            if x is not None and not np.isfinite(x).all():
                raise ValueError("velocities must be finite")
        L.check(L.lib().avbd_world_set_velocities(self._h, L.uptr(idx), idx.size, L.fptr(v), L.fptr(a)))

    def setLinearVelocities(self, indices, linear):
        self.setVelocities(indices, linear=linear)

    def setAngularVelocities(self, indices, angular):
        self.setVelocities(indices, angular=angular)

    # parity dumps (readPairs / readContactList) ------------------------------------
    def readPairs(self) -> np.ndarray:
        self._live()
        n = C.c_int64()
        L.check(L.lib().avbd_world_pairs(self._h, None, 0, C.byref(n)))
        out = np.zeros((n.value, 2), dtype=np.uint32)
        L.check(L.lib().avbd_world_pairs(self._h, L.uptr(out), n.value, C.byref(n)))
        return out

    def readPairContacts(self) -> np.ndarray:
        self._live()
        n = C.c_int64()
        L.check(L.lib().avbd_world_pair_contacts(self._h, None, 0, C.byref(n)))
        out = np.zeros(n.value, dtype=np.int32)
        L.check(L.lib().avbd_world_pair_contacts(self._h, L.iptr(out), n.value, C.byref(n)))
        return out

    def readColors(self) -> np.ndarray:
        self._live()
        out = np.zeros(self.bodyCount, dtype=np.int32)
        L.check(L.lib().avbd_world_colors(self._h, L.iptr(out)))
        return out

    def exportState(self) -> dict:
        """Full solver state (bodies, joints, manifolds with their contacts, colours)."""
        self._live()
        nj, nm, nc = C.c_int32(), C.c_int64(), C.c_int64()
        L.check(L.lib().avbd_world_state_sizes(self._h, C.byref(nj), C.byref(nm), C.byref(nc)))
        j, m, c = nj.value, nm.value, nc.value
        st = {k: np.zeros((j, 3), dtype=np.float32) for k in ("jpen_lin", "jpen_ang", "jlam_lin", "jlam_ang")}
        st["jbroken"] = np.zeros(j, dtype=np.int32)
        st["mpairs"] = np.zeros((m, 2), dtype=np.uint32)
        st["mcount"] = np.zeros(m, dtype=np.int32)
        st["cfeature"] = np.zeros(c, dtype=np.uint32)
        for k in ("cra", "crb", "cpen", "clam"):
            st[k] = np.zeros((c, 3), dtype=np.float32)
        st["cstick"] = np.zeros(c, dtype=np.int32)
        L.check(L.lib().avbd_world_export_state(
            self._h, L.fptr(st["jpen_lin"]), L.fptr(st["jpen_ang"]), L.fptr(st["jlam_lin"]), L.fptr(st["jlam_ang"]),
            L.iptr(st["jbroken"]), L.uptr(st["mpairs"]), L.iptr(st["mcount"]), L.uptr(st["cfeature"]),
            L.fptr(st["cra"]), L.fptr(st["crb"]), L.fptr(st["cpen"]), L.fptr(st["clam"]), L.iptr(st["cstick"])))
        b = self.readBodyState()
        st.update(pos=b["position"], quat=b["rotation"], vel=b["velocity"], angvel=b["angular"],
                  prev_vel=b["prev_velocity"], colors=self.readColors())
        st["asleep"], st["sleep_time"] = self.readSleepState()
        return st

    # sleeping (src/native/cpu/world.js:859-890) ------------------------------
    def enableSleeping(self, options=None):
        """Island sleeping with {speedThreshold, timeThreshold} (defaults 0.08 m/s, 0.6 s)."""
        self._live()
        speed, time = _sleep_thresholds(True if options is None else options, None)
        L.check(L.lib().avbd_world_set_sleeping(self._h, 1, speed, time))
        return self

    def disableSleeping(self):
        self._live()
        L.check(L.lib().avbd_world_set_sleeping(self._h, 0, 0.0, 0.0))
        return self

    def setSleepEnabled(self, index, enabled):
        self._live()
        if not isinstance(enabled, bool):
            raise ValueError("Sleep flag must be boolean")
        L.check(L.lib().avbd_world_set_sleep_enabled(self._h, int(index), int(enabled)))
        return self

    def wakeAll(self):
        self._live()
        L.check(L.lib().avbd_world_wake_all(self._h))
        return self

    def wakeUp(self, index):
        if not 0 <= int(index) < self.bodyCount:
            raise ValueError("A live body index is required")
        return self.wakeAll()

    def readSleepStats(self) -> dict:
        self._live()
        n = C.c_int32()
        L.check(L.lib().avbd_world_sleep_state(self._h, None, None, C.byref(n)))
        return {"sleeping": int(n.value), "wakeRequested": False}

    def readSleepState(self):
        """(sleeping flags, seconds each body's island has been quiet) per body."""
        self._live()
        a = np.zeros(self.bodyCount, dtype=np.int32)
        t = np.zeros(self.bodyCount, dtype=np.float32)
        L.check(L.lib().avbd_world_sleep_state(self._h, L.iptr(a), L.fptr(t), None))
        return a.astype(bool), t

    # joints, filters, handles (src/native/scenes.d.ts:350-440) ----------------
    def readJoints(self) -> np.ndarray:
        """32 floats per joint or spring in creation order (the reference's joint record)."""
        self._live()
        out = np.zeros(self.jointCount * 32, dtype=np.float32)
        if self.jointCount:
            L.check(L.lib().avbd_world_read_joints(self._h, L.fptr(out)))
        return out

    def setFilters(self, indices, groups, collidesWith):
        self._live()
        idx = np.asarray(indices, dtype=np.int64).reshape(-1)
        g = np.asarray(groups, dtype=np.int64).reshape(-1)
        m = np.asarray(collidesWith, dtype=np.int64).reshape(-1)
        if not (idx.size == g.size == m.size):
            raise ValueError("Filter arrays must have matching lengths")
        if idx.size and (idx.min() < 0 or idx.max() >= self.bodyCount):
            raise ValueError("A live body index is required")
        for a in (g, m):
            if a.size and (a.min() < 0 or a.max() > 0xFFFFFFFF):
                raise ValueError("Collision masks must be unsigned 32-bit integers")
        ia, ga, ma = (np.ascontiguousarray(a.astype(np.uint32)) for a in (idx, g, m))
        L.check(L.lib().avbd_world_set_filters(self._h, L.uptr(ia), int(ia.size), L.uptr(ga), L.uptr(ma)))
        return self

    def gpuIndex(self, referenceIndex: int) -> int:
        """The slot of the body created as `referenceIndex` (itself unless spatialSort moved it);
        every other call takes and returns slots, as the reference's GPU world does."""
        if not 0 <= int(referenceIndex) < self.bodyCount:
            raise ValueError("A live body index is required")
        return int(referenceIndex) if self._slot is None else int(self._slot[int(referenceIndex)])

    def bodyIndex(self, body) -> int:
        return self.gpuIndex(body)

    # shape casts (src/native/solver3D.js:244-251) ----------------------------
    def raycast(self, origin, direction, options=None):
        return self.sphereCast(origin, 0.0, direction, options)

    def sphereCast(self, origin, radius, direction, options=None):
        return self.sphereCastAll([{"origin": origin, "radius": radius, "direction": direction}], options)[0]

    def raycastAll(self, rays, options=None):
        return self.sphereCastAll([{**r, "radius": 0.0} for r in rays], options)

    def sphereCastAll(self, casts, options=None):
        self._live()
        return _cast(L.lib().avbd_world_cast, (self._h,), casts, options, self.bodyCount)

    # contact events (src/native/solver3D.js:256-310) -------------------------
    def watchContacts(self, options=None):
        """Turn contact begin/end events on (every body watched) or choose the watched bodies
        ({indices, maxPairs, maxEvents})."""
        self._live()
        idx, n, mp, me = _watch_args(options, self.bodyCount)
        L.check(L.lib().avbd_world_watch_contacts(self._h, L.uptr(idx), n, mp, me))
        return self

    def readContactEvents(self) -> dict:
        self._live()
        self.watchContacts()
        return _read_events(L.lib().avbd_world_contact_events, self._h)

    def readContactEventsRaw(self) -> dict:
        """The events as an (n, 12) uint32 array (floats as bits) plus dropped/full."""
        self._live()
        self.watchContacts()
        return _read_events_raw(L.lib().avbd_world_contact_events, self._h)

    def resetContactHistory(self, indices):
        self._live()
        if not isinstance(indices, np.ndarray) or indices.dtype != np.uint32:
            raise ValueError("Contact resets require Uint32 3D body slots")
        arr = np.ascontiguousarray(indices)
        if arr.size and (np.any(np.diff(arr.astype(np.int64)) <= 0) or int(arr.max()) >= self.bodyCount):
            raise ValueError("Contact reset slots must be unique and ascending")
        L.check(L.lib().avbd_world_reset_contact_history(self._h, L.uptr(arr), int(arr.size)))
        return self

    def importSleepState(self, asleep, time):
        self._live()
        a = np.ascontiguousarray(asleep, dtype=np.int32)
        t = np.ascontiguousarray(time, dtype=np.float32)
        L.check(L.lib().avbd_world_import_sleep_state(self._h, L.iptr(a), L.fptr(t)))

    def profile(self, enable: bool = True):
        """Start (and reset) or stop per-kernel-class timing and traffic accounting."""
        self._live()
        L.check(L.lib().avbd_world_profile(self._h, int(bool(enable))))

    def profileRead(self) -> dict:
        self._live()
        p = L.Profile()
        L.check(L.lib().avbd_world_profile_read(self._h, C.byref(p)))
        return {k: getattr(p, k) for k, _ in L.Profile._fields_ if not k.startswith("pad")}

    def destroy(self):
        if self._h is None:
            return
        L.check(L.lib().avbd_world_destroy(self._h))
        self._h = None
        if self in self._pipe._children:
            self._pipe._children.remove(self)


class Batch:
    """Many independent worlds stepped together in one launch sequence per step."""

    def __init__(self, pipe: SolverPipeline, arrays_list):
        if not arrays_list:
            raise ValueError("a batch needs at least one world")
        self._pipe = pipe
        self._packed = [L.PackedScene(a) for a in arrays_list]
        descs = (L.SceneDesc * len(arrays_list))(*[p.desc for p in self._packed])
        params = (L.Params * len(arrays_list))(*[p.params for p in self._packed])
        h = C.c_void_p()
        L.check(L.lib().avbd_batch_create(pipe._h, descs, params, len(arrays_list), C.byref(h)))
        self._h = h
        self.worldCount = len(arrays_list)
        self.bodyCounts = [a.n_bodies for a in arrays_list]
        self._dts = [float(a.params.dt) for a in arrays_list]
        self._jointCounts = [p.n_joints for p in self._packed]
        self._kinds = [np.asarray(a.kind, dtype=np.int32).copy() for a in arrays_list]
        self.bodyCount = int(sum(self.bodyCounts))
        self._pinned = []  # page-locked blocks of pinnedPoses(), freed with the batch

    def step(self, steps: int = 1):
        if self._h is None:
            raise RuntimeError("The batch has been destroyed")
        L.check(L.lib().avbd_batch_step(self._h, int(steps)))
        return self

    def pinnedPoses(self) -> np.ndarray:
        """A page-locked (bodyCount, 8) float32 array for stepRead, freed with the batch."""
        ptr = C.c_void_p()
        L.check(L.lib().avbd_pinned_alloc(max(self.bodyCount, 1) * 32, C.byref(ptr)))
        self._pinned.append(ptr)
        buf = (C.c_float * (max(self.bodyCount, 1) * 8)).from_address(ptr.value)
        return np.ctypeslib.as_array(buf)[: self.bodyCount * 8].reshape(self.bodyCount, 8)

    def stepRead(self, steps: int, out: np.ndarray) -> int:
        """Queue ``steps`` steps and, after the last, a copy of every pose into ``out`` (page-locked:
        ``pinnedPoses()``); returns at once with a tag for ``readDone``."""
        if self._h is None:
            raise RuntimeError("The batch has been destroyed")
        if out.dtype != np.float32 or out.size != self.bodyCount * 8 or not out.flags["C_CONTIGUOUS"]:
            raise ValueError("out must be a contiguous float32 array of bodyCount x 8")
        tag = C.c_int64()
        L.check(L.lib().avbd_batch_step_read(self._h, int(steps), out.ctypes.data_as(C.c_void_p), C.byref(tag)))
        return int(tag.value)

    def readDone(self, tag: int, wait: bool = False) -> bool:
        """Whether the read of ``tag`` has landed (wait: block until it has, not for later steps)."""
        done = C.c_int32()
        L.check(L.lib().avbd_batch_read_done(self._h, int(tag), int(bool(wait)), C.byref(done)))
        return bool(done.value)

    def readBodyState(self, world: int) -> dict:
        if not 0 <= world < self.worldCount:
            raise ValueError("world index out of range")
        n = self.bodyCounts[world]
        out = {k: np.zeros((n, 4 if k == "rotation" else 3), dtype=np.float32)
               for k in ("position", "rotation", "velocity", "angular", "prev_velocity")}
        L.check(L.lib().avbd_batch_read_state(self._h, int(world), *(L.fptr(out[k]) for k in
                                                                     ("position", "rotation", "velocity", "angular", "prev_velocity"))))
        return out

    def setMotor(self, world: int, constraint, speed=None, maxTorque=None):
        """World.setMotor for world `world` of the batch."""
        if not 0 <= world < self.worldCount:
            raise ValueError("world index out of range")
        slot = _motor_slot(self._kinds[world], constraint)
        mask, sp, mt = _motor_args(speed, maxTorque)
        L.check(L.lib().avbd_batch_set_motor(self._h, int(world), slot, mask, sp, mt))

    def releaseJoints(self, world: int, constraints):
        """World.releaseJoints for world `world` of the batch."""
        if not 0 <= world < self.worldCount:
            raise ValueError("world index out of range")
        slots = _joint_slots(self._kinds[world], constraints)
        L.check(L.lib().avbd_batch_release_joints(self._h, int(world), L.iptr(slots), int(slots.size)))

    def _world(self, world: int) -> int:
        if not 0 <= int(world) < self.worldCount:
            raise ValueError("world index out of range")
        return int(world)

    def setFilters(self, world: int, indices, groups, collidesWith):
        """World.setFilters for world `world` of the batch (world-local body indices)."""
        w = self._world(world)
        idx = np.asarray(indices, dtype=np.int64).reshape(-1)
        g = np.asarray(groups, dtype=np.int64).reshape(-1)
        m = np.asarray(collidesWith, dtype=np.int64).reshape(-1)
        if not (idx.size == g.size == m.size):
            raise ValueError("Filter arrays must have matching lengths")
        if idx.size and (idx.min() < 0 or idx.max() >= self.bodyCounts[w]):
            raise ValueError("A live body index is required")
        for a in (g, m):
            if a.size and (a.min() < 0 or a.max() > 0xFFFFFFFF):
                raise ValueError("Collision masks must be unsigned 32-bit integers")
        ia, ga, ma = (np.ascontiguousarray(a.astype(np.uint32)) for a in (idx, g, m))
        L.check(L.lib().avbd_batch_set_filters(self._h, w, L.uptr(ia), int(ia.size), L.uptr(ga), L.uptr(ma)))

    def setRestitution(self, world: int, indices, values):
        """World.setRestitution for world `world` of the batch."""
        w = self._world(world)
        idx = _indices(indices, self.bodyCounts[w])
        val = np.ascontiguousarray(np.asarray(values, dtype=np.float32).reshape(-1))
        if idx.size != val.size:
            raise ValueError("Restitution arrays must have matching lengths")
        if val.size and not (np.all(val >= 0) and np.all(val <= 1)):
            raise ValueError("restitution must be between 0 and 1")
        L.check(L.lib().avbd_batch_set_restitution(self._h, w, L.uptr(idx), int(idx.size), L.fptr(val)))

    def setSensor(self, world: int, index, enabled):
        """World.setSensor for world `world` of the batch."""
        w = self._world(world)
        if not isinstance(enabled, bool):
            raise ValueError("isTrigger must be a boolean")
        idx = _indices([index], self.bodyCounts[w])
        L.check(L.lib().avbd_batch_set_sensor(self._h, w, L.uptr(idx), 1, int(enabled)))

    def setSpringMaterial(self, world: int, constraint, breakStrain=None, breakForce=None):
        """World.setSpringMaterial for world `world` of the batch."""
        from .scene import KIND_SPRING, spring_material
        w = self._world(world)
        kinds = self._kinds[w]
        c = int(constraint)
        if not 0 <= c < len(kinds) or kinds[c] != KIND_SPRING:
            raise ValueError("Spring material requires an active spring slot")
        m = spring_material(math.inf if breakStrain is None else breakStrain,
                            math.inf if breakForce is None else breakForce)
        mask = (1 if breakStrain is not None else 0) | (2 if breakForce is not None else 0)
        slot = int(_joint_slots(kinds, [c])[0])
        L.check(L.lib().avbd_batch_set_spring_material(self._h, w, slot, mask, m["breakStrain"], m["breakForce"]))

    def setWorldAnchor(self, world: int, constraint, point):
        """World.setWorldAnchor for world `world` of the batch."""
        w = self._world(world)
        p = np.ascontiguousarray(np.asarray(point, dtype=np.float32).reshape(-1))
        if p.size != 3 or not np.all(np.isfinite(p)):
            raise ValueError("A world joint and finite xyz anchor are required")
        slot = int(_joint_slots(self._kinds[w], [constraint])[0])
        L.check(L.lib().avbd_batch_set_world_anchor(self._h, w, slot, L.fptr(p)))

    def captureConstraintFrames(self, world: int, entries):
        """World.captureConstraintFrames for world `world` of the batch."""
        w = self._world(world)
        cons = [int(e["slot"]) if isinstance(e, dict) else int(e) for e in entries]
        spring = [1 if isinstance(e, dict) and e.get("spring") else 0 for e in entries]
        slots = _joint_slots(self._kinds[w], cons)
        sp = np.ascontiguousarray(np.asarray(spring, dtype=np.int32))
        L.check(L.lib().avbd_batch_capture_frames(self._h, w, L.iptr(slots), L.iptr(sp), int(slots.size)))

    def readJoints(self, world: int) -> np.ndarray:
        if not 0 <= world < self.worldCount:
            raise ValueError("world index out of range")
        n = self._jointCounts[world]
        out = np.zeros(n * 32, dtype=np.float32)
        if n:
            L.check(L.lib().avbd_batch_read_joints(self._h, int(world), L.fptr(out)))
        return out

    def sphereCastAll(self, world: int, casts, options=None):
        if not 0 <= world < self.worldCount:
            raise ValueError("world index out of range")
        return _cast(L.lib().avbd_batch_cast, (self._h, int(world)), casts, options, self.bodyCounts[world])

    def watchContacts(self, world: int, options=None):
        if not 0 <= world < self.worldCount:
            raise ValueError("world index out of range")
        idx, n, mp, me = _watch_args(options, self.bodyCounts[world])
        L.check(L.lib().avbd_batch_watch_contacts(self._h, int(world), L.uptr(idx), n, mp, me))
        return self

    def readContactEventsRaw(self, world: int) -> dict:
        self.watchContacts(world)
        return _read_events_raw(L.lib().avbd_batch_contact_events, self._h, int(world))

    def readContactEvents(self, world: int) -> dict:
        self.watchContacts(world)
        return _read_events(L.lib().avbd_batch_contact_events, self._h, int(world))

    def readSleepState(self, world: int):
        if not 0 <= world < self.worldCount:
            raise ValueError("world index out of range")
        n = self.bodyCounts[world]
        a = np.zeros(n, dtype=np.int32)
        t = np.zeros(n, dtype=np.float32)
        L.check(L.lib().avbd_batch_sleep_state(self._h, int(world), L.iptr(a), L.fptr(t), None))
        return a.astype(bool), t

    def readCounters(self) -> dict:
        c = L.Counters()
        L.check(L.lib().avbd_batch_counters(self._h, C.byref(c)))
        return {k: getattr(c, k) for k, _ in L.Counters._fields_}

    def readPoses(self, out: np.ndarray | None = None) -> np.ndarray:
        """Poses of all bodies of all worlds, (bodyCount, 8) float32: pos, friction, quat."""
        if out is None:
            out = np.zeros((self.bodyCount, 8), dtype=np.float32)
        if out.dtype != np.float32 or out.size != self.bodyCount * 8 or not out.flags["C_CONTIGUOUS"]:
            raise ValueError("out must be a contiguous float32 array of bodyCount x 8")
        L.check(L.lib().avbd_batch_read_poses(self._h, L.fptr(out)))
        return out

    def setVelocities(self, indices, linear=None, angular=None):
        """Batch-global body indices (world offset + body index)."""
        idx = _indices(indices, self.bodyCount)
        v = None if linear is None else np.ascontiguousarray(np.asarray(linear, dtype=np.float32).reshape(idx.size, 3))
        a = None if angular is None else np.ascontiguousarray(np.asarray(angular, dtype=np.float32).reshape(idx.size, 3))
        for x in (v, a):
            if x is not None and not np.isfinite(x).all():
                raise ValueError("velocities must be finite")
        L.check(L.lib().avbd_batch_set_velocities(self._h, L.uptr(idx), idx.size, L.fptr(v), L.fptr(a)))

    def editBodies(self, world: int, edits):
        """Body edits (world-local indices) of world ``world``, applied at the next step; property
        keys (isTrigger, restitution, group/collidesWith, allowSleep, in runtime.js:157-165's order)
        apply at once, as World.editBodies does."""
        if not 0 <= world < self.worldCount:
            raise ValueError("world index out of range")
        edits = list(edits)
        props = stage_properties(edits, self.bodyCounts[world])
        rec = stage_edits(edits, self.bodyCounts[world], self._dts[world], allow_properties=True)
        if len(rec):
            L.check(L.lib().avbd_batch_edit(self._h, int(world), L.uptr(rec), int(rec.shape[0])))
        for p in props:
            if p["isTrigger"] is not None:
                self.setSensor(world, p["index"], p["isTrigger"])
            if p["restitution"] is not None:
                self.setRestitution(world, [p["index"]], [p["restitution"]])
            if p["group"] is not None:
                self.setFilters(world, [p["index"]], [p["group"]], [p["collidesWith"]])
            if p["allowSleep"] is not None:
                L.check(L.lib().avbd_batch_set_sleep_enabled(self._h, int(world), p["index"], int(p["allowSleep"])))
        return self

    def profile(self, enable: bool = True):
        L.check(L.lib().avbd_batch_profile(self._h, int(bool(enable))))

    def profileRead(self) -> dict:
        p = L.Profile()
        L.check(L.lib().avbd_batch_profile_read(self._h, C.byref(p)))
        return {k: getattr(p, k) for k, _ in L.Profile._fields_ if not k.startswith("pad")}

    def destroy(self):
        if self._h is None:
            return
        L.check(L.lib().avbd_batch_destroy(self._h))
        self._h = None
        for ptr in self._pinned:
            L.lib().avbd_pinned_free(ptr)
        self._pinned = []
        if self in self._pipe._children:
            self._pipe._children.remove(self)


class Server:
    """Continuous batching of many worlds (``avbd_server_*``).

    ``admit(scene)`` returns a world id; ``advance(id, k)`` queues k steps and returns a ticket;
    each ``tick()`` steps every world with queued steps once, in one launch sequence, and
    ``completed()`` lists the tickets whose steps have all run. Worlds that do not fit in the
    device budget evict the least recently used idle worlds to host memory; evicted worlds are
    restored when work for them arrives. Results equal those of the same world stepped alone.
    """

    def __init__(self, pipe: SolverPipeline, budget: int, initial_bodies: int, initial_worlds: int):
        self._pipe = pipe
        h = C.c_void_p()
        desc = L.ServerDesc(budget, initial_bodies, initial_worlds)
        L.check(L.lib().avbd_server_create(pipe._h, C.byref(desc), C.byref(h)))
        self._h = h
        self._counts = {}
        self._dts = {}

    def _live(self):
        if self._h is None:
            raise RuntimeError("The server has been destroyed")

    def admit(self, scene) -> int:
        """Admit a world; raises ``AvbdError`` (code ``AVBD_E_CAPACITY``) if it cannot fit."""
        self._live()
        packed = scene if isinstance(scene, L.PackedScene) else L.PackedScene(_arrays(scene))
        wid = C.c_int64()
        L.check(L.lib().avbd_server_admit(self._h, C.byref(packed.desc), C.byref(packed.params), C.byref(wid)))
        self._counts[wid.value] = packed.n_bodies
        self._dts[wid.value] = float(packed.params.dt)
        return wid.value

    def editBodies(self, world: int, edits):
        """Body edits of a served world, applied before its next step."""
        self._live()
        if int(world) not in self._counts:
            raise ValueError(f"no such world {world}")
        rec = stage_edits(edits, self._counts[int(world)], self._dts[int(world)])
        if len(rec):
            L.check(L.lib().avbd_server_edit(self._h, int(world), L.uptr(rec), int(rec.shape[0])))
        return self

    def advance(self, world: int, steps: int = 1) -> int:
        self._live()
        if steps < 0:
            raise ValueError("steps must be non-negative")
        t = C.c_int64()
        L.check(L.lib().avbd_server_advance(self._h, int(world), int(steps), C.byref(t)))
        return t.value

    def tick(self, maxSteps: int = 1, replies: bool = False) -> int:
        """Up to ``maxSteps`` steps of every world with queued steps, queued on the device without
        waiting (the same bits as that many single ticks); returns the world-steps taken. With
        ``replies`` the poses of each world whose request a step completes are captured right
        after that step: those tickets come from ``ready()`` and their poses from ``takeReply``."""
        self._live()
        if int(maxSteps) != maxSteps or maxSteps < 1:
            raise ValueError("maxSteps must be a positive integer")
        n = C.c_int32()
        L.check(L.lib().avbd_server_tick_steps(self._h, int(maxSteps), int(bool(replies)), C.byref(n)))
        return n.value

    def ready(self, wait: bool = False, cap: int = 65536) -> list:
        """Tickets whose captured replies have arrived (wait: until every queued step has run)."""
        self._live()
        out = np.zeros(max(int(cap), 1), dtype=np.int64)
        n = C.c_int32()
        done = []
        while True:
            L.check(L.lib().avbd_server_ready(self._h, out.ctypes.data_as(L._i64p), out.size, int(bool(wait)), C.byref(n)))
            done.extend(int(x) for x in out[:n.value])
            if n.value < out.size:
                return done

    def takeReply(self, ticket: int) -> np.ndarray:
        """The captured poses of a ready ticket's world, (bodies, 8) float32; handed out once."""
        self._live()
        n = C.c_int32()
        L.check(L.lib().avbd_server_take_reply(self._h, int(ticket), None, 0, C.byref(n)))
        out = np.zeros((n.value, 8), dtype=np.float32)
        L.check(L.lib().avbd_server_take_reply(self._h, int(ticket), L.fptr(out), n.value, C.byref(n)))
        return out

    def completed(self, cap: int = 65536) -> list:
        self._live()
        out = np.zeros(max(int(cap), 1), dtype=np.int64)
        n = C.c_int32()
        done = []
        while True:
            L.check(L.lib().avbd_server_completed(self._h, out.ctypes.data_as(L._i64p), out.size, C.byref(n)))
            done.extend(int(x) for x in out[:n.value])
            if n.value < out.size:
                return done

    def readPoses(self, worlds) -> np.ndarray:
        """Poses of every body of the listed worlds, world after world: (bodies, 8) float32."""
        self._live()
        ids = np.ascontiguousarray(np.asarray(worlds, dtype=np.int64).reshape(-1))
        for w in ids:
            if int(w) not in self._counts:
                raise ValueError(f"no such world {int(w)}")
        total = int(sum(self._counts[int(w)] for w in ids))
        out = np.zeros((total, 8), dtype=np.float32)
        L.check(L.lib().avbd_server_read_poses(self._h, ids.ctypes.data_as(L._i64p), ids.size, L.fptr(out)))
        return out

    def readBodyState(self, world: int) -> dict:
        self._live()
        n = self._counts.get(int(world))
        if n is None:
            raise ValueError(f"no such world {world}")
        out = {k: np.zeros((n, 4 if k == "rotation" else 3), dtype=np.float32)
               for k in ("position", "rotation", "velocity", "angular", "prev_velocity")}
        L.check(L.lib().avbd_server_read_state(self._h, int(world), *(L.fptr(out[k]) for k in
                                                                       ("position", "rotation", "velocity", "angular", "prev_velocity"))))
        return out

    def sphereCastAll(self, world: int, casts, options=None):
        self._live()
        n = self._counts.get(int(world))
        if n is None:
            raise ValueError(f"no such world {world}")
        return _cast(L.lib().avbd_server_cast, (self._h, int(world)), casts, options, n)

    def watchContacts(self, world: int, options=None):
        self._live()
        n = self._counts.get(int(world))
        if n is None:
            raise ValueError(f"no such world {world}")
        idx, k, mp, me = _watch_args(options, n)
        L.check(L.lib().avbd_server_watch_contacts(self._h, int(world), L.uptr(idx), k, mp, me))
        return self

    def readContactEventsRaw(self, world: int) -> dict:
        self.watchContacts(world)
        return _read_events_raw(L.lib().avbd_server_contact_events, self._h, int(world))

    def readContactEvents(self, world: int) -> dict:
        self.watchContacts(world)
        return _read_events(L.lib().avbd_server_contact_events, self._h, int(world))

    def readSleepState(self, world: int):
        self._live()
        n = self._counts.get(int(world))
        if n is None:
            raise ValueError(f"no such world {world}")
        a = np.zeros(n, dtype=np.int32)
        t = np.zeros(n, dtype=np.float32)
        L.check(L.lib().avbd_server_sleep_state(self._h, int(world), L.iptr(a), L.fptr(t), None))
        return a.astype(bool), t

    def info(self, world: int) -> dict:
        self._live()
        nb, res = C.c_int32(), C.c_int32()
        q, d = C.c_int64(), C.c_int64()
        L.check(L.lib().avbd_server_world_info(self._h, int(world), C.byref(nb), C.byref(q), C.byref(d), C.byref(res)))
        return {"bodies": nb.value, "queued": q.value, "steps": d.value, "resident": bool(res.value)}

    def evict(self, world: int):
        self._live()
        L.check(L.lib().avbd_server_evict(self._h, int(world)))

    def release(self, world: int):
        self._live()
        L.check(L.lib().avbd_server_release(self._h, int(world)))
        self._counts.pop(int(world), None)

    def stats(self) -> dict:
        self._live()
        st = L.ServerStats()
        L.check(L.lib().avbd_server_read_stats(self._h, C.byref(st)))
        return {k: getattr(st, k) for k, _ in L.ServerStats._fields_}

    def destroy(self):
        if self._h is None:
            return
        L.check(L.lib().avbd_server_destroy(self._h))
        self._h = None
        if self in self._pipe._children:
            self._pipe._children.remove(self)
