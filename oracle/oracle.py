"""AVBD CPU ORACLE -- test infrastructure only.

ctypes wrapper over ``oracle/_build/liboracle.so`` (the C++ restatement of the reference's CPU
rigid-body path, ``avbd_oracle.hpp``). Used by ``tests/`` as the checker, by
``__graft_entry__.smoke()`` and by ``bench.py``'s CPU-baseline leg. The product never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)
_up = C.POINTER(C.c_uint32)


class _Scene(C.Structure):
    _fields_ = [("n_bodies", C.c_int), ("pos", _dp), ("quat", _dp), ("size", _dp), ("vel", _dp),
                ("angvel", _dp), ("prev_vel", _dp), ("mass", _dp), ("moment", _dp),
                ("friction", _dp), ("radius", _dp), ("shape", _ip), ("group", _up), ("mask", _up),
                ("n_cons", C.c_int), ("kind", _ip), ("ca", _ip), ("cb", _ip), ("ra", _dp),
                ("rb", _dp), ("p0", _dp), ("p1", _dp), ("p2", _dp), ("restitution", _dp),
                ("allow_sleep", _ip), ("p3", _dp), ("is_trigger", _ip)]


class _Params(C.Structure):
    _fields_ = [("dt", C.c_double), ("gravity", C.c_double), ("up", C.c_double * 3),
                ("iterations", C.c_int), ("alpha", C.c_double), ("beta_lin", C.c_double),
                ("beta_ang", C.c_double), ("gamma", C.c_double), ("app", C.c_int),
                ("mass_penalty", C.c_int), ("face_bias", C.c_int), ("colored", C.c_int),
                ("color_rounds", C.c_int), ("sleeping", C.c_int), ("sleep_speed", C.c_double),
                ("sleep_time", C.c_double)]


class _State(C.Structure):
    _fields_ = [("pos", _dp), ("quat", _dp), ("vel", _dp), ("angvel", _dp), ("prev_vel", _dp),
                ("jpen_lin", _dp), ("jpen_ang", _dp), ("jlam_lin", _dp), ("jlam_ang", _dp),
                ("jbroken", _ip), ("n_manifolds", C.c_int), ("mpairs", _ip), ("mcount", _ip),
                ("cfeature", _up), ("cra", _dp), ("crb", _dp), ("cpen", _dp), ("clam", _dp),
                ("cstick", _ip), ("colors", _ip)]


_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (g++ -ffp-contract=off, OpenMP)."""
    if force or not os.path.exists(LIB_PATH):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        L.oracle_world_create.restype = C.c_void_p
        L.oracle_world_create.argtypes = [C.c_int, C.POINTER(_Scene), C.POINTER(_Params)]
        for name in ("oracle_world_destroy", "oracle_world_step_collide", "oracle_world_step_solve"):
            getattr(L, name).argtypes = [C.c_void_p]
        L.oracle_world_step.argtypes = [C.c_void_p, C.c_int]
        L.oracle_world_set_colored.argtypes = [C.c_void_p, C.c_int]
        L.oracle_world_body_count.argtypes = [C.c_void_p]
        L.oracle_world_force_count.argtypes = [C.c_void_p]
        L.oracle_world_counts.argtypes = [C.c_void_p, _ip]
        L.oracle_world_read_bodies.argtypes = [C.c_void_p, _dp, _dp, _dp, _dp, _dp]
        L.oracle_world_read_colors.argtypes = [C.c_void_p, _ip]
        L.oracle_world_manifolds.argtypes = [C.c_void_p, _ip, _ip, C.c_int]
        L.oracle_world_candidate_pairs.argtypes = [C.c_void_p, _ip, C.c_int]
        L.oracle_world_collide.argtypes = [C.c_void_p, C.c_int, C.c_int, _dp, _up, _dp, _dp]
        L.oracle_world_import.argtypes = [C.c_void_p, C.POINTER(_State)]
        L.oracle_world_edit.argtypes = [C.c_void_p, C.POINTER(C.c_uint32), C.c_int]
        L.oracle_world_set_sleep.argtypes = [C.c_void_p, _ip, _dp]
        L.oracle_world_sleep_state.argtypes = [C.c_void_p, _ip, _dp]
        L.oracle_world_sleep_state.restype = C.c_int
        L.oracle_world_wake_all.argtypes = [C.c_void_p]
        L.oracle_world_sleep_after.argtypes = [C.c_void_p]
        L.oracle_worlds_step_parallel.argtypes = [C.POINTER(C.c_void_p), C.c_int, C.c_int, C.c_int]
        L.oracle_worlds_step_parallel.restype = C.c_int
        L.oracle_angle_atan2.argtypes = [C.c_int, _dp, _dp, _dp, C.c_int]
        L.oracle_world_set_motor.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_double]
        L.oracle_world_set_motor.restype = C.c_int
        L.oracle_world_release_joints.argtypes = [C.c_void_p, _ip, C.c_int]
        L.oracle_world_set_sensor.argtypes = [C.c_void_p, _ip, C.c_int, C.c_int]
        L.oracle_world_set_spring_material.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_double]
        L.oracle_world_set_spring_material.restype = C.c_int
        L.oracle_world_set_world_anchor.argtypes = [C.c_void_p, C.c_int, _dp]
        L.oracle_world_set_world_anchor.restype = C.c_int
        L.oracle_world_capture_frame.argtypes = [C.c_void_p, C.c_int, C.c_int]
        L.oracle_world_capture_frame.restype = C.c_int
        _lib = L
    return _lib


def _ptr(a, ct):
    return a.ctypes.data_as(C.POINTER(ct)) if a is not None else None


class OracleWorld:
    """One oracle world. ``fp64`` selects double (faithful) or float arithmetic; ``app``
    selects the app CPU path (up vector, grid broadphase, faceBias, massPenalty, spheres) or
    the pinned reference solver (Z up, O(n^2) broadphase); ``colored`` runs the primal in the
    GPU engine's colour order."""

    def __init__(self, scene, fp64=True, app=True, colored=False):
        L = lib()
        p = scene.params
        keep = []

        def d(a, shape=None):
            a = np.ascontiguousarray(a, dtype=np.float64)
            keep.append(a)
            return _ptr(a, C.c_double)

        def i32(a):
            a = np.ascontiguousarray(a, dtype=np.int32)
            keep.append(a)
            return _ptr(a, C.c_int32)

        def u32(a):
            a = np.ascontiguousarray(a, dtype=np.uint32)
            keep.append(a)
            return _ptr(a, C.c_uint32)

        s = _Scene(scene.n_bodies, d(scene.pos), d(scene.quat), d(scene.size), d(scene.vel),
                   d(scene.angvel), d(scene.prev_vel), d(scene.mass), d(scene.moment),
                   d(scene.friction), d(scene.radius), i32(scene.shape), u32(scene.group),
                   u32(scene.mask), scene.n_cons, i32(scene.kind), i32(scene.ca), i32(scene.cb),
                   d(scene.ra), d(scene.rb), d(scene.p0), d(scene.p1), d(scene.p2),
                   d(scene.restitution_or_zero()), i32(scene.allow_sleep_or_one()),
                   d(scene.p3_or_none() if hasattr(scene, "p3_or_none") else np.zeros(scene.n_cons)),
                   i32(scene.is_trigger_or_zero() if hasattr(scene, "is_trigger_or_zero") else np.zeros(scene.n_bodies)))
        prm = _Params(p.dt, p.gravity, (C.c_double * 3)(*p.up), p.iterations, p.alpha, p.beta_lin,
                      p.beta_ang, p.gamma, int(app), int(p.mass_penalty), int(p.face_bias),
                      int(colored), int(p.color_rounds), int(bool(p.sleeping)), float(p.sleep_speed),
                      float(p.sleep_time))
        self.h = L.oracle_world_create(int(fp64), C.byref(s), C.byref(prm))
        self.n = scene.n_bodies
        self.n_joints = int(np.sum((scene.kind == 0) | (scene.kind == 1)))
        self.fp64 = fp64

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.oracle_world_destroy(self.h)
            self.h = None

    def step(self, steps=1):
        lib().oracle_world_step(self.h, int(steps))

    def step_collide(self):
        lib().oracle_world_step_collide(self.h)

    def step_solve(self):
        lib().oracle_world_step_solve(self.h)

    def set_colored(self, on: bool):
        lib().oracle_world_set_colored(self.h, int(on))

    @property
    def force_count(self) -> int:
        return lib().oracle_world_force_count(self.h)

    def counts(self) -> dict:
        out = np.zeros(7, dtype=np.int32)
        lib().oracle_world_counts(self.h, _ptr(out, C.c_int32))
        return dict(manifolds=int(out[0]), joints=int(out[1]), springs=int(out[2]),
                    ignores=int(out[3]), contacts=int(out[4]), colors=int(out[5]),
                    conflicts=int(out[6]))

    def bodies(self):
        n = self.n
        pos, quat = np.zeros((n, 3)), np.zeros((n, 4))
        vel, ang, prev = np.zeros((n, 3)), np.zeros((n, 3)), np.zeros((n, 3))
        lib().oracle_world_read_bodies(self.h, _ptr(pos, C.c_double), _ptr(quat, C.c_double),
                                       _ptr(vel, C.c_double), _ptr(ang, C.c_double),
                                       _ptr(prev, C.c_double))
        return dict(pos=pos, quat=quat, vel=vel, angvel=ang, prev_vel=prev)

    def colors(self):
        out = np.zeros(self.n, dtype=np.int32)
        lib().oracle_world_read_colors(self.h, _ptr(out, C.c_int32))
        return out

    def manifolds(self):
        cap = 1 << 16
        while True:
            pairs = np.zeros((cap, 2), dtype=np.int32)
            counts = np.zeros(cap, dtype=np.int32)
            n = lib().oracle_world_manifolds(self.h, _ptr(pairs, C.c_int32), _ptr(counts, C.c_int32), cap)
            if n <= cap:
                return pairs[:n], counts[:n]
            cap = n

    def candidate_pairs(self):
        cap = 1 << 16
        while True:
            out = np.zeros((cap, 2), dtype=np.int32)
            n = lib().oracle_world_candidate_pairs(self.h, _ptr(out, C.c_int32), cap)
            if n <= cap:
                return out[:n]
            cap = n

    def collide(self, a, b):
        basis = np.zeros(9)
        feats = np.zeros(8, dtype=np.uint32)
        ra, rb = np.zeros((8, 3)), np.zeros((8, 3))
        n = lib().oracle_world_collide(self.h, int(a), int(b), _ptr(basis, C.c_double),
                                       _ptr(feats, C.c_uint32), _ptr(ra, C.c_double), _ptr(rb, C.c_double))
        return dict(count=n, basis=basis.reshape(3, 3), features=feats[:n], ra=ra[:n], rb=rb[:n])

    def import_state(self, st: dict):
        """Load a full solver state (see ``_State``); arrays as produced by the engine's
        state export."""
        keep = []

        def d(a):
            a = np.ascontiguousarray(a, dtype=np.float64)
            keep.append(a)
            return _ptr(a, C.c_double)

        def i32(a):
            if a is None:
                return None
            a = np.ascontiguousarray(a, dtype=np.int32)
            keep.append(a)
            return _ptr(a, C.c_int32)

        def u32(a):
            a = np.ascontiguousarray(a, dtype=np.uint32)
            keep.append(a)
            return _ptr(a, C.c_uint32)

        s = _State(d(st["pos"]), d(st["quat"]), d(st["vel"]), d(st["angvel"]), d(st["prev_vel"]),
                   d(st["jpen_lin"]), d(st["jpen_ang"]), d(st["jlam_lin"]), d(st["jlam_ang"]),
                   i32(st["jbroken"]), int(len(st["mcount"])), i32(st["mpairs"]),
                   i32(st["mcount"]), u32(st["cfeature"]), d(st["cra"]), d(st["crb"]),
                   d(st["cpen"]), d(st["clam"]), i32(st["cstick"]), i32(st.get("colors")))
        lib().oracle_world_import(self.h, C.byref(s))

    def set_sleep(self, asleep, time):
        """Load per-body sleep state (flags, accumulated quiet seconds)."""
        a = np.ascontiguousarray(asleep, dtype=np.int32)
        t = np.ascontiguousarray(time, dtype=np.float64)
        lib().oracle_world_set_sleep(self.h, _ptr(a, C.c_int32), _ptr(t, C.c_double))

    def sleep_state(self):
        """(sleeping flags, quiet seconds) per body."""
        a = np.zeros(self.n, dtype=np.int32)
        t = np.zeros(self.n, dtype=np.float64)
        lib().oracle_world_sleep_state(self.h, _ptr(a, C.c_int32), _ptr(t, C.c_double))
        return a.astype(bool), t

    def wake_all(self):
        lib().oracle_world_wake_all(self.h)

    def sleep_after(self):
        """The sleeping pass alone (``step`` runs it after the solve when sleeping is on)."""
        lib().oracle_world_sleep_after(self.h)

    def set_motor(self, jid, speed=None, max_torque=None):
        """setMotor of the motor with joint slot `jid` (speed and/or torque bound)."""
        mask = (1 if speed is not None else 0) | (2 if max_torque is not None else 0)
        ok = lib().oracle_world_set_motor(self.h, int(jid), mask, float(speed or 0.0), float(max_torque or 0.0))
        if not ok:
            raise ValueError("Motor needs an active motor slot")

    def release_joints(self, jids):
        """releaseJoints of these joint slots."""
        j = np.ascontiguousarray(np.asarray(jids, dtype=np.int32).reshape(-1))
        lib().oracle_world_release_joints(self.h, _ptr(j, C.c_int), j.size)

    def set_sensor(self, indices, enabled):
        i = np.ascontiguousarray(np.asarray(indices, dtype=np.int32).reshape(-1))
        lib().oracle_world_set_sensor(self.h, _ptr(i, C.c_int), i.size, int(bool(enabled)))

    def set_spring_material(self, jid, break_strain=None, break_force=None):
        mask = (1 if break_strain is not None else 0) | (2 if break_force is not None else 0)
        inf = float("inf")
        ok = lib().oracle_world_set_spring_material(self.h, int(jid), mask, float(inf if break_strain is None else break_strain),
                                                    float(inf if break_force is None else break_force))
        if not ok:
            raise ValueError("Spring material requires an active spring slot")

    def set_world_anchor(self, jid, point):
        p = np.ascontiguousarray(np.asarray(point, dtype=np.float64).reshape(3))
        if not lib().oracle_world_set_world_anchor(self.h, int(jid), _ptr(p, C.c_double)):
            raise ValueError("A world joint and finite xyz anchor are required")

    def capture_frames(self, entries):
        """entries: (joint slot, spring) pairs."""
        for jid, spring in entries:
            if not lib().oracle_world_capture_frame(self.h, int(jid), int(bool(spring))):
                raise ValueError("A live spring or joint slot is required")

    def edit(self, records):
        """Apply body command records (n x 12 uint32 words, ``src/gpu/bodyCommands2D.js``
        layout) with the CPU world's flushEdits semantics (``src/native/cpu/world.js:229-300``)."""
        r = np.ascontiguousarray(records, dtype=np.uint32).reshape(-1, 12)
        lib().oracle_world_edit(self.h, r.ctypes.data_as(C.POINTER(C.c_uint32)), int(r.shape[0]))


def angle_atan2(y, x, fp64=True):
    """The angular rows' atan2 (half-angle reductions and a Taylor series), elementwise."""
    y = np.ascontiguousarray(np.asarray(y, dtype=np.float64).reshape(-1))
    x = np.ascontiguousarray(np.asarray(x, dtype=np.float64).reshape(-1))
    out = np.zeros_like(y)
    lib().oracle_angle_atan2(1 if fp64 else 0, _ptr(y, C.c_double), _ptr(x, C.c_double), _ptr(out, C.c_double), y.size)
    return out


def step_parallel(worlds, steps, threads=0) -> int:
    """Step independent oracle worlds concurrently (OpenMP); returns the threads used."""
    arr = (C.c_void_p * len(worlds))(*[w.h for w in worlds])
    return lib().oracle_worlds_step_parallel(arr, len(worlds), int(steps), int(threads))
