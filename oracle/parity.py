"""AVBD CPU ORACLE -- test infrastructure only.

One-step parity between the CUDA engine and the oracle from the same starting state:
the engine's full state after `warm` steps (bodies, joint and contact warm-start state,
colours) is loaded into the oracle, both take one step, and the results are compared:

* candidate pair set (bounding spheres overlap etc.) -- must be identical;
* contacts per pair (oracle narrowphase in float32 on the same poses) -- must be identical;
* Jones-Plassmann colours -- identical, and valid (no constraint joins two bodies of a colour);
* poses and velocities -- |gpu - cpu| <= tol * (|cpu| + 1) with tol = 1e-5 against the
  float32 oracle run in the engine's colour order; the error against the float64 oracle in
  the same order is reported beside it.
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


def compare_step(world, scene, warm: int, edits=None):
    """Run the comparison on an engine world built from `scene`; returns a report dict.
    `edits` (body command records, n x 12 words) are queued on the engine world and applied to
    the oracles before the compared step."""
    if warm:
        world.step(warm)
    st = world.exportState()
    rep = {}
    oracles = {}
    for name, fp64 in (("fp32", False), ("fp64", True)):
        o = O.OracleWorld(scene, fp64=fp64, app=True, colored=True)
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
