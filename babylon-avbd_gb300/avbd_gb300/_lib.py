"""ctypes binding of the engine's C ABI (``include/avbd_gb300.h``).

The library is ``libavbd_gb300.so`` next to this file, built by ``babylon-avbd_gb300/build.py``.
There is no fallback: if the library is missing or fails to load, importing the engine raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libavbd_gb300.so")

_fp = C.POINTER(C.c_float)
_ip = C.POINTER(C.c_int32)
_up = C.POINTER(C.c_uint32)
_i64p = C.POINTER(C.c_int64)


class Params(C.Structure):
    _fields_ = [("dt", C.c_float), ("gravity", C.c_float), ("up", C.c_float * 3),
                ("iterations", C.c_int32), ("alpha", C.c_float), ("beta_lin", C.c_float),
                ("beta_ang", C.c_float), ("gamma", C.c_float), ("mass_penalty", C.c_int32),
                ("face_bias", C.c_int32), ("color_rounds", C.c_int32), ("broadphase", C.c_int32),
                ("bvh_rebuild", C.c_int32), ("sleeping", C.c_int32), ("sleep_speed", C.c_float),
                ("sleep_time", C.c_float)]


class SceneDesc(C.Structure):
    _fields_ = [("n_bodies", C.c_int32), ("position", _fp), ("rotation", _fp), ("size", _fp),
                ("velocity", _fp), ("angular_velocity", _fp), ("prev_velocity", _fp),
                ("mass", _fp), ("moment", _fp), ("friction", _fp), ("radius", _fp),
                ("shape", _ip), ("group", _up), ("collides_with", _up), ("n_cons", C.c_int32),
                ("cons_kind", _ip), ("cons_a", _ip), ("cons_b", _ip), ("cons_ra", _fp),
                ("cons_rb", _fp), ("cons_p0", _fp), ("cons_p1", _fp), ("cons_p2", _fp), ("restitution", _fp),
                ("allow_sleep", _ip), ("cons_p3", _fp), ("is_trigger", _ip)]


class CastFilter(C.Structure):
    _fields_ = [("collides_with", C.c_uint32), ("membership", C.c_uint32), ("has_membership", C.c_int32),
                ("include_triggers", C.c_int32), ("n_ignore", C.c_int32), ("ignore", C.c_uint32 * 16)]


class Counters(C.Structure):
    _fields_ = [("pairs", C.c_int64), ("manifolds", C.c_int64), ("contacts", C.c_int64),
                ("joints", C.c_int64), ("colors", C.c_int32), ("conflicts", C.c_int32),
                ("overflow", C.c_int32), ("steps", C.c_int32)]


class Profile(C.Structure):
    _fields_ = [("steps", C.c_int32), ("pad", C.c_int32), ("ms_collide", C.c_double),
                ("ms_topology", C.c_double), ("ms_primal", C.c_double), ("ms_dual", C.c_double),
                ("ms_other", C.c_double), ("primal_launches", C.c_int64), ("launches", C.c_int64),
                ("bytes_primal", C.c_double), ("bytes_dual", C.c_double), ("bytes_collide", C.c_double),
                ("graph_captures", C.c_int64), ("graph_replays", C.c_int64), ("graphs_on", C.c_int32),
                ("ticks_held", C.c_int32), ("tuned", C.c_int32), ("solve_queue", C.c_int32),
                ("solve_waves", C.c_int32), ("solve_blocks", C.c_int32), ("radix_bits", C.c_int32),
                ("solve_tile", C.c_int32)]


class ServerDesc(C.Structure):
    _fields_ = [("budget_bytes", C.c_int64), ("initial_bodies", C.c_int32), ("initial_worlds", C.c_int32)]


class ServerStats(C.Structure):
    _fields_ = [(k, C.c_int64) for k in (
        "budget_bytes", "device_bytes", "peak_device_bytes", "live_worlds", "resident_worlds",
        "evicted_worlds", "pending_worlds", "resident_bodies", "admitted", "rejected", "evictions",
        "restores", "ticks", "body_steps", "completed")]


# (name, restype, argtypes); every function returns int status unless noted
SIGNATURES = [
    ("avbd_last_error", C.c_char_p, []),
    ("avbd_version", C.c_char_p, []),
    ("avbd_ctx_create", C.c_int, [C.c_int, C.POINTER(C.c_void_p)]),
    ("avbd_ctx_destroy", C.c_int, [C.c_void_p]),
    ("avbd_ctx_stream", C.c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
    ("avbd_ctx_synchronize", C.c_int, [C.c_void_p]),
    ("avbd_ctx_fence", C.c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
    ("avbd_fence_wait", C.c_int, [C.c_void_p]),
    ("avbd_fence_query", C.c_int, [C.c_void_p, _ip]),
    ("avbd_fence_destroy", C.c_int, [C.c_void_p]),
    ("avbd_world_create", C.c_int, [C.c_void_p, C.POINTER(SceneDesc), C.POINTER(Params), C.POINTER(C.c_void_p)]),
    ("avbd_world_destroy", C.c_int, [C.c_void_p]),
    ("avbd_world_step", C.c_int, [C.c_void_p, C.c_int32]),
    ("avbd_world_read_state", C.c_int, [C.c_void_p, _fp, _fp, _fp, _fp, _fp]),
    ("avbd_world_read_selected", C.c_int, [C.c_void_p, _up, C.c_int32, C.c_int32, _fp]),
    ("avbd_world_read_selected_noalloc", C.c_int, [C.c_void_p, _up, C.c_int32, C.c_int32, _fp]),
    ("avbd_world_set_poses", C.c_int, [C.c_void_p, _up, C.c_int32, _fp, _fp]),
    ("avbd_world_set_velocities", C.c_int, [C.c_void_p, _up, C.c_int32, _fp, _fp]),
    ("avbd_world_counters", C.c_int, [C.c_void_p, C.POINTER(Counters)]),
    ("avbd_world_pairs", C.c_int, [C.c_void_p, _up, C.c_int64, _i64p]),
    ("avbd_world_pair_contacts", C.c_int, [C.c_void_p, _ip, C.c_int64, _i64p]),
    ("avbd_world_colors", C.c_int, [C.c_void_p, _ip]),
    ("avbd_world_state_sizes", C.c_int, [C.c_void_p, _ip, _i64p, _i64p]),
    ("avbd_world_export_state", C.c_int, [C.c_void_p, _fp, _fp, _fp, _fp, _ip, _up, _ip, _up, _fp, _fp, _fp, _fp, _ip]),
    ("avbd_batch_create", C.c_int, [C.c_void_p, C.POINTER(SceneDesc), C.POINTER(Params), C.c_int32, C.POINTER(C.c_void_p)]),
    ("avbd_batch_destroy", C.c_int, [C.c_void_p]),
    ("avbd_batch_step", C.c_int, [C.c_void_p, C.c_int32]),
    ("avbd_batch_world_count", C.c_int, [C.c_void_p, _ip, _i64p]),
    ("avbd_batch_read_state", C.c_int, [C.c_void_p, C.c_int32, _fp, _fp, _fp, _fp, _fp]),
    ("avbd_batch_counters", C.c_int, [C.c_void_p, C.POINTER(Counters)]),
    ("avbd_batch_read_poses", C.c_int, [C.c_void_p, _fp]),
    ("avbd_batch_step_read", C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, _i64p]),
    ("avbd_batch_read_done", C.c_int, [C.c_void_p, C.c_int64, C.c_int32, _ip]),
    ("avbd_pinned_alloc", C.c_int, [C.c_int64, C.POINTER(C.c_void_p)]),
    ("avbd_pinned_free", C.c_int, [C.c_void_p]),
    ("avbd_check_division", C.c_int, [C.c_int32, C.c_int64, C.c_uint32, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    ("avbd_batch_set_velocities", C.c_int, [C.c_void_p, _up, C.c_int32, _fp, _fp]),
    ("avbd_world_profile", C.c_int, [C.c_void_p, C.c_int32]),
    ("avbd_world_profile_read", C.c_int, [C.c_void_p, C.POINTER(Profile)]),
    ("avbd_batch_profile", C.c_int, [C.c_void_p, C.c_int32]),
    ("avbd_batch_profile_read", C.c_int, [C.c_void_p, C.POINTER(Profile)]),
    ("avbd_server_create", C.c_int, [C.c_void_p, C.POINTER(ServerDesc), C.POINTER(C.c_void_p)]),
    ("avbd_server_destroy", C.c_int, [C.c_void_p]),
    ("avbd_server_admit", C.c_int, [C.c_void_p, C.POINTER(SceneDesc), C.POINTER(Params), _i64p]),
    ("avbd_server_advance", C.c_int, [C.c_void_p, C.c_int64, C.c_int32, _i64p]),
    ("avbd_server_tick", C.c_int, [C.c_void_p, _ip]),
    ("avbd_server_tick_steps", C.c_int, [C.c_void_p, C.c_int32, C.c_int32, _ip]),
    ("avbd_server_ready", C.c_int, [C.c_void_p, _i64p, C.c_int32, C.c_int32, _ip]),
    ("avbd_server_take_reply", C.c_int, [C.c_void_p, C.c_int64, _fp, C.c_int64, _ip]),
    ("avbd_server_completed", C.c_int, [C.c_void_p, _i64p, C.c_int32, _ip]),
    ("avbd_server_read_poses", C.c_int, [C.c_void_p, _i64p, C.c_int32, _fp]),
    ("avbd_server_read_state", C.c_int, [C.c_void_p, C.c_int64, _fp, _fp, _fp, _fp, _fp]),
    ("avbd_server_world_info", C.c_int, [C.c_void_p, C.c_int64, _ip, _i64p, _i64p, _ip]),
    ("avbd_server_evict", C.c_int, [C.c_void_p, C.c_int64]),
    ("avbd_server_release", C.c_int, [C.c_void_p, C.c_int64]),
    ("avbd_server_read_stats", C.c_int, [C.c_void_p, C.POINTER(ServerStats)]),
    ("avbd_world_edit", C.c_int, [C.c_void_p, _up, C.c_int32]),
    ("avbd_world_flush_edits", C.c_int, [C.c_void_p]),
    ("avbd_batch_edit", C.c_int, [C.c_void_p, C.c_int32, _up, C.c_int32]),
    ("avbd_server_edit", C.c_int, [C.c_void_p, C.c_int64, _up, C.c_int32]),
    ("avbd_world_set_sleeping", C.c_int, [C.c_void_p, C.c_int32, C.c_float, C.c_float]),
    ("avbd_world_set_sleep_enabled", C.c_int, [C.c_void_p, C.c_int32, C.c_int32]),
    ("avbd_world_wake_all", C.c_int, [C.c_void_p]),
    ("avbd_world_sleep_state", C.c_int, [C.c_void_p, _ip, _fp, _ip]),
    ("avbd_world_import_sleep_state", C.c_int, [C.c_void_p, _ip, _fp]),
    ("avbd_batch_sleep_state", C.c_int, [C.c_void_p, C.c_int32, _ip, _fp, _ip]),
    ("avbd_world_watch_contacts", C.c_int, [C.c_void_p, _up, C.c_int32, C.c_int32, C.c_int32]),
    ("avbd_world_cast", C.c_int, [C.c_void_p, _fp, C.c_int32, C.c_void_p, _fp]),
    ("avbd_world_read_joints", C.c_int, [C.c_void_p, _fp]),
    ("avbd_world_set_filters", C.c_int, [C.c_void_p, _up, C.c_int32, _up, _up]),
    ("avbd_world_set_restitution", C.c_int, [C.c_void_p, _up, C.c_int32, _fp]),
    ("avbd_batch_read_joints", C.c_int, [C.c_void_p, C.c_int32, _fp]),
    ("avbd_world_set_motor", C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_float, C.c_float]),
    ("avbd_batch_set_motor", C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_float, C.c_float]),
    ("avbd_world_release_joints", C.c_int, [C.c_void_p, _ip, C.c_int32]),
    ("avbd_world_set_sensor", C.c_int, [C.c_void_p, _up, C.c_int32, C.c_int32]),
    ("avbd_batch_set_filters", C.c_int, [C.c_void_p, C.c_int32, _up, C.c_int32, _up, _up]),
    ("avbd_batch_set_restitution", C.c_int, [C.c_void_p, C.c_int32, _up, C.c_int32, _fp]),
    ("avbd_batch_set_sensor", C.c_int, [C.c_void_p, C.c_int32, _up, C.c_int32, C.c_int32]),
    ("avbd_batch_set_sleep_enabled", C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32]),
    ("avbd_batch_set_spring_material", C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_float, C.c_float]),
    ("avbd_batch_set_world_anchor", C.c_int, [C.c_void_p, C.c_int32, C.c_int32, _fp]),
    ("avbd_batch_capture_frames", C.c_int, [C.c_void_p, C.c_int32, _ip, _ip, C.c_int32]),
    ("avbd_world_set_spring_material", C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_float, C.c_float]),
    ("avbd_world_set_world_anchor", C.c_int, [C.c_void_p, C.c_int32, _fp]),
    ("avbd_world_capture_frames", C.c_int, [C.c_void_p, _ip, _ip, C.c_int32]),
    ("avbd_batch_release_joints", C.c_int, [C.c_void_p, C.c_int32, _ip, C.c_int32]),
    ("avbd_batch_cast", C.c_int, [C.c_void_p, C.c_int32, _fp, C.c_int32, C.c_void_p, _fp]),
    ("avbd_server_cast", C.c_int, [C.c_void_p, C.c_int64, _fp, C.c_int32, C.c_void_p, _fp]),
    ("avbd_world_reset_contact_history", C.c_int, [C.c_void_p, _up, C.c_int32]),
    ("avbd_world_contact_events", C.c_int, [C.c_void_p, _up, C.c_int64, _i64p, _i64p, _ip]),
    ("avbd_batch_watch_contacts", C.c_int, [C.c_void_p, C.c_int32, _up, C.c_int32, C.c_int32, C.c_int32]),
    ("avbd_batch_contact_events", C.c_int, [C.c_void_p, C.c_int32, _up, C.c_int64, _i64p, _i64p, _ip]),
    ("avbd_server_watch_contacts", C.c_int, [C.c_void_p, C.c_int64, _up, C.c_int32, C.c_int32, C.c_int32]),
    ("avbd_server_contact_events", C.c_int, [C.c_void_p, C.c_int64, _up, C.c_int64, _i64p, _i64p, _ip]),
    ("avbd_server_sleep_state", C.c_int, [C.c_void_p, C.c_int64, _ip, _fp, _ip]),
]

# include/avbd_gb300.h
AVBD_E_CAPACITY = -5
BROADPHASE = {"grid": 0, "hploc": 1, "auto": 2}
NOALLOC_MAX_SELECTED = 8192

_lib = None


class AvbdError(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, code, message):
        super().__init__(f"{message} (status {code})")
        self.code = code


def lib() -> C.CDLL:
    """Load the engine library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"engine library not built: {LIB_PATH} (run babylon-avbd_gb300/build.py)")
        L = C.CDLL(LIB_PATH)
        for name, res, args in SIGNATURES:
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(status: int):
    if status != 0:
        raise AvbdError(status, lib().avbd_last_error().decode())


def fptr(a):
    return None if a is None else a.ctypes.data_as(_fp)


def iptr(a):
    return None if a is None else a.ctypes.data_as(_ip)


def uptr(a):
    return None if a is None else a.ctypes.data_as(_up)


class PackedScene:
    """A scene converted to the float32/int32 arrays the C ABI reads (kept alive with it)."""

    def __init__(self, arrays):
        f32 = lambda a: np.ascontiguousarray(a, dtype=np.float32)  # noqa: E731
        i32 = lambda a: np.ascontiguousarray(a, dtype=np.int32)  # noqa: E731
        u32 = lambda a: np.ascontiguousarray(a, dtype=np.uint32)  # noqa: E731
        s = arrays
        self.keep = [f32(s.pos), f32(s.quat), f32(s.size), f32(s.vel), f32(s.angvel), f32(s.prev_vel),
                     f32(s.mass), f32(s.moment), f32(s.friction), f32(s.radius), i32(s.shape),
                     u32(s.group), u32(s.mask), i32(s.kind), i32(s.ca), i32(s.cb), f32(s.ra),
                     f32(s.rb), f32(s.p0), f32(s.p1), f32(s.p2), f32(s.restitution_or_zero()),
                     i32(s.allow_sleep_or_one()), f32(s.p3_or_none()), i32(s.is_trigger_or_zero())]
        k = self.keep
        self.desc = SceneDesc(s.n_bodies, fptr(k[0]), fptr(k[1]), fptr(k[2]), fptr(k[3]), fptr(k[4]),
                              fptr(k[5]), fptr(k[6]), fptr(k[7]), fptr(k[8]), fptr(k[9]), iptr(k[10]),
                              uptr(k[11]), uptr(k[12]), s.n_cons, iptr(k[13]), iptr(k[14]),
                              iptr(k[15]), fptr(k[16]), fptr(k[17]), fptr(k[18]), fptr(k[19]),
                              fptr(k[20]), fptr(k[21]), iptr(k[22]), fptr(k[23]), iptr(k[24]))
        p = s.params
        self.params = Params(p.dt, p.gravity, (C.c_float * 3)(*p.up), p.iterations, p.alpha,
                             p.beta_lin, p.beta_ang, p.gamma, int(p.mass_penalty), int(p.face_bias),
                             int(p.color_rounds), BROADPHASE[p.broadphase], int(p.bvh_rebuild),
                             int(bool(p.sleeping)), float(p.sleep_speed), float(p.sleep_time))
        self.n_bodies = s.n_bodies
        self.n_joints = int(np.sum(s.kind != 2)) if s.n_cons else 0
