"""AVBD CPU ORACLE -- test infrastructure only.

Contact begin/end events of one step, restated from the reference's ContactWatch
(src/vendor/three-avbd-lib/contacts.ts: `touching` and `ended`, and its run/setWatched/resetBodies
bookkeeping) over two consecutive exported solver states of one world:

* a pair touches in a step when its manifold has contacts and one of its bodies' watch words has
  bit 0 set; the set of touching pairs of each step is kept;
* begin: touching now, and not (in last step's set and both watch words unchanged since then);
  it carries the mean of the contact points (rA turned by A's rotation plus A's position, summed
  then divided), |sum of the contacts' normal lambda| x dt, and the manifold normal;
* end: in last step's set, both watch words unchanged, and not touching now;
* a watch word is bit 0 (watched) plus twice the number of history resets.

Float arithmetic here is float64 on the engine's float32 inputs; kinds, bodies and steps compare
exactly, points, impulses and normals within a tolerance.
"""
from __future__ import annotations

import numpy as np

BEGIN, END = 1, 2


def _turn(q, v):
    u = q[:3]
    t = 2.0 * np.cross(u, v)
    return v + q[3] * t + np.cross(u, t)


def touching(state, watch) -> set:
    """Pairs (a, b), a > b, with contacts and a watched body, from an exported state."""
    out = set()
    for (a, b), c in zip(np.asarray(state["mpairs"], dtype=np.int64), state["mcount"]):
        if c > 0 and ((int(watch[a]) | int(watch[b])) & 1):
            out.add((int(a), int(b)))
    return out


def step_events(prev_set, watch_prev, state, watch, step, dt, normal_of, triggers=None):
    """Events of one step: (list of (kind, a, b, step, point, impulse, normal), this step's set).
    `state` is the world's state exported after the step, `normal_of(a, b)` the manifold normal
    of the pair in that step. A pair with a trigger body (`triggers[i]`) reports no impulse
    (src/native/cpu/world.js:757-762)."""
    events = []
    now = set()
    first = np.concatenate([[0], np.cumsum(state["mcount"])])
    for m, ((a, b), c) in enumerate(zip(np.asarray(state["mpairs"], dtype=np.int64), state["mcount"])):
        a, b = int(a), int(b)
        if c == 0 or not ((int(watch[a]) | int(watch[b])) & 1):
            continue
        now.add((a, b))
        same = watch[a] == watch_prev[a] and watch[b] == watch_prev[b]
        if (a, b) in prev_set and same:
            continue
        pA = np.asarray(state["pos"][a], dtype=np.float64)
        qA = np.asarray(state["quat"][a], dtype=np.float64)
        point = np.zeros(3)
        force = 0.0
        for k in range(first[m], first[m + 1]):
            point += _turn(qA, np.asarray(state["cra"][k], dtype=np.float64)) + pA
            force += float(state["clam"][k][0])
        trig = triggers is not None and bool(triggers[a] or triggers[b])
        events.append((BEGIN, a, b, step, point / c, 0.0 if trig else abs(force) * dt,
                       np.asarray(normal_of(a, b), dtype=np.float64)))
    for a, b in sorted(prev_set):
        if not (watch[a] == watch_prev[a] and watch[b] == watch_prev[b]):
            continue
        if (a, b) not in now:
            events.append((END, a, b, step, np.zeros(3), 0.0, np.zeros(3)))
    events.sort(key=lambda e: (e[3], e[0], e[1], e[2]))
    return events, now
