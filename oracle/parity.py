"""AVBD CPU ORACLE -- test infrastructure only.

One-step parity between the CUDA engine and the oracle from the same starting state:
the engine's full state after `warm` steps (bodies, joint and contact warm-start state,
colours) is loaded into the oracle, both take one step, and the results are compared:

* candidate pair set (bounding spheres overlap etc.) -- must be identical;
* contacts per pair (oracle narrowphase in float32 on the same poses) -- must be identical;
* Jones-Plassmann colours -- identical, and valid (no constraint joins two bodies of a colour);
* poses and velocities -- |gpu - cpu| <= tol * (|cpu| + 1) with tol = 1e-5 against the
  float32 oracle run in the engine's colour order; the errors against the float64 oracle in
  the same order and against the float64 oracle in the reference CPU's own sequential order
  (newest body first, src/native/cpu/cpuSolver3D.ts:207) are reported beside it.
"""
from __future__ import annotations

import numpy as np

import oracle as O

TOL = 1e-5


def _err(gpu, cpu):
    g = np.asarray(gpu, dtype=np.float64)
    c = np.asarray(cpu, dtype=np.float64)
    if g.size == 0:
        return 0.0
    return float(np.max(np.abs(g - c) / (np.abs(c) + 1.0)))


def compare_step(world, scene, warm: int, edits=None, sequential=True):
    """Run the comparison on an engine world built from `scene`; returns a report dict.
    `edits` (body command records, n x 12 words) are queued on the engine world and applied to
    the oracles before the compared step. `sequential` adds the float64 oracle in the
    reference's sequential order (max_err_fp64_sequential)."""
    if warm:
        world.step(warm)
    st = world.exportState()
    rep = {}
    oracles = {}
    runs = [("fp32", False, True), ("fp64", True, True)]
    if sequential:
        runs.append(("fp64_sequential", True, False))
    for name, fp64, colored in runs:
        o = O.OracleWorld(scene, fp64=fp64, app=True, colored=colored)
        o.import_state(st)
        if "asleep" in st:
            o.set_sleep(st["asleep"], st["sleep_time"])
        if edits is not None and len(edits):
            o.edit(edits)
        oracles[name] = o
    if edits is not None and len(edits):
        world.editRecords(edits)
    o32 = oracles["fp32"]
    cand = o32.candidate_pairs()
    world.step(1)
    gpu_pairs = world.readPairs().astype(np.int64)
    gpu_counts = world.readPairContacts()
    rep["pairs_gpu"] = int(len(gpu_pairs))
    rep["pairs_cpu"] = int(len(cand))
    rep["pairs_equal"] = bool(len(gpu_pairs) == len(cand) and np.array_equal(gpu_pairs, cand.astype(np.int64)))
    cpu_counts = np.array([o32.collide(int(a), int(b))["count"] for a, b in gpu_pairs], dtype=np.int32)
    rep["contact_counts_equal"] = bool(np.array_equal(cpu_counts, gpu_counts))
    rep["contact_count_mismatches"] = int(np.sum(cpu_counts != gpu_counts))
    rep["contacts"] = int(gpu_counts.sum())
    for o in oracles.values():
        o.step(1)
    g = world.readBodyState()
    for name, o in oracles.items():
        b = o.bodies()
        rep[f"pos_err_{name}"] = _err(g["position"], b["pos"])
        rep[f"quat_err_{name}"] = _err(g["rotation"], b["quat"])
        rep[f"vel_err_{name}"] = _err(g["velocity"], b["vel"])
        rep[f"angvel_err_{name}"] = _err(g["angular"], b["angvel"])
    gcol = world.readColors()
    ccol = o32.colors()
    dyn = scene.mass > 0
    rep["colors_equal"] = bool(np.array_equal(gcol[dyn], ccol[dyn]))
    rep["colors"] = int(gcol[dyn].max() + 1) if dyn.any() else 0
    rep["coloring_valid"] = coloring_valid(world, scene, gcol)
    rep["max_err_fp32"] = max(rep[f"{k}_err_fp32"] for k in ("pos", "quat", "vel", "angvel"))
    rep["max_err_fp64"] = max(rep[f"{k}_err_fp64"] for k in ("pos", "quat", "vel", "angvel"))
    if sequential:
        rep["max_err_fp64_sequential"] = max(rep[f"{k}_err_fp64_sequential"] for k in ("pos", "quat", "vel", "angvel"))
    return rep


def coloring_valid(world, scene, colors) -> bool:
    """No live constraint (joint, spring or manifold with contacts) joins two dynamic bodies
    of one colour."""
    dyn = scene.mass > 0
    pairs = world.readPairs().astype(np.int64)
    counts = world.readPairContacts()
    edges = [pairs[counts > 0]]
    st = world.exportState()
    if scene.n_cons:
        keep = scene.kind != 2
        ca, cb = scene.ca[keep], scene.cb[keep]
        alive = st["jbroken"] == 0
        j = np.stack([ca, cb], axis=1)[alive & (ca >= 0)]
        edges.append(j.astype(np.int64))
    e = np.concatenate(edges) if edges else np.zeros((0, 2), np.int64)
    if len(e) == 0:
        return True
    both = dyn[e[:, 0]] & dyn[e[:, 1]]
    e = e[both]
    return bool(np.all(colors[e[:, 0]] != colors[e[:, 1]]))


def _rotate(q, v):
    u, w = q[:, :3], q[:, 3:4]
    t = 2.0 * np.cross(u, v)
    return v + w * t + np.cross(u, t)


def stability_metrics(scene, pos, quat, vel, angvel, sphere=None, footprint=None, max_radius=None):
    """Size-independent state of a long run, computed the same way from any body state:
    `top` and `mean_y` (highest and mean dynamic body centre along y), `ground_pen` (deepest
    point of a dynamic body below the ground top y = 0, over bodies within `footprint` of the
    origin in x and z (a body that rolled off the ground's edge is not penetrating it) and of
    bounding radius below `max_radius`),
    `sphere_pen` (deepest box corner or sphere surface inside the static sphere (centre, R)) and
    `ke` (total kinetic energy, linear plus rotational in the body frame)."""
    pos, quat = np.asarray(pos, np.float64), np.asarray(quat, np.float64)
    vel, angvel = np.asarray(vel, np.float64), np.asarray(angvel, np.float64)
    dyn = scene.mass > 0
    half = np.asarray(scene.size, np.float64) / 2
    corners = np.stack([pos + _rotate(quat, half * np.array([sx, sy, sz]))
                        for sx in (-1, 1) for sy in (-1, 1) for sz in (-1, 1)], axis=1)
    box = scene.shape == 0
    low = np.where(box, corners[:, :, 1].min(axis=1), pos[:, 1] - scene.radius)
    sel = dyn.copy()
    if footprint is not None:
        sel &= (np.abs(pos[:, 0]) < footprint) & (np.abs(pos[:, 2]) < footprint)
    if max_radius is not None:
        sel &= np.asarray(scene.radius) < max_radius
    out = {"top": float(pos[dyn, 1].max()), "mean_y": float(pos[dyn, 1].mean()),
           "ground_pen": max(0.0, -float(low[sel].min())) if sel.any() else 0.0}
    m = scene.mass[dyn]
    ke = 0.5 * float((m * (vel[dyn] ** 2).sum(axis=1)).sum())
    local = _rotate(quat[dyn] * np.array([-1.0, -1.0, -1.0, 1.0]), angvel[dyn])
    out["ke"] = ke + 0.5 * float((np.asarray(scene.moment, np.float64)[dyn] * local ** 2).sum())
    if sphere is not None:
        c, R = np.asarray(sphere[0], np.float64), float(sphere[1])
        dist = np.where(box[dyn], np.linalg.norm(corners[dyn] - c, axis=2).min(axis=1),
                        np.linalg.norm(pos[dyn] - c, axis=1) - scene.radius[dyn])
        out["sphere_pen"] = max(0.0, float((R - dist).max()))
    return out
