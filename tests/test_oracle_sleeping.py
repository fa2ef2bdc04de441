"""The oracle's island sleeping against a float64 restatement of the reference's
src/native/cpu/sleeping.js (CpuSleeping.after / wake), step by step, plus the behaviour the
reference documents: quiet supported islands fall asleep after timeThreshold seconds with zero
velocity, unsupported or sleep-disallowed islands stay awake, an awake body touching a sleeping
one wakes the world, and queued body commands wake it (src/native/cpu/world.js:132-133).
"""
import math

import numpy as np
import pytest

from avbd_gb300 import AvbdScene3D


def _after(o, mass, allow, joints, dt, speed_thr, time_thr, asleep, time):
    """CpuSleeping.after of sleeping.js on the oracle's post-solve state (float64)."""
    n = len(mass)
    root = list(range(n))

    def find(i):
        while root[i] != i:
            root[i] = root[root[i]]
            i = root[i]
        return i

    support, edges = set(), []

    def link(a, b):
        if a < 0:
            support.add(b)
            return
        if mass[a] <= 0:
            support.add(b)
        elif mass[b] <= 0:
            support.add(a)
        else:
            root[find(a)] = find(b)
        edges.append((a, b))

    pairs, counts = o.manifolds()
    for (a, b), c in zip(pairs, counts):
        if c > 0:
            link(int(a), int(b))
    for a, b in joints:
        link(a, b)
    st = o.bodies()
    supported = {find(s) for s in support}
    stable = {}
    for i in range(n):
        if mass[i] > 0:
            r = find(i)
            speed = math.sqrt(sum(float(x) ** 2 for x in (*st["vel"][i], *st["angvel"][i])))
            stable.setdefault(r, r in supported)
            stable[r] = stable[r] and bool(allow[i]) and speed <= speed_thr
    asleep, time = asleep.copy(), time.copy()
    for i in range(n):
        if mass[i] > 0:
            time[i] = time[i] + dt if stable[find(i)] else 0.0
            if time[i] >= time_thr:
                asleep[i] = True
    if any(a >= 0 and mass[a] > 0 and mass[b] > 0 and asleep[a] != asleep[b] for a, b in edges):
        asleep[:] = False
        time[:] = 0.0
    return asleep, time


def _pile(late=True, allow=True):
    """Three short stacks of boxes and a few spheres on a wide ground (y up)."""
    sc = AvbdScene3D(timeStep=1 / 60, iterations=10, gravity=-10)
    sc.addBox([40, 1, 40], position=[0, -0.5, 0], density=0)
    rng = np.random.default_rng(3)
    for x in (-4.0, 0.0, 4.0):
        for k in range(4):
            sc.addBox([1, 1, 1], position=[x + rng.uniform(-0.05, 0.05), 0.5 + 1.02 * k, rng.uniform(-0.05, 0.05)],
                      allowSleep=allow)
    for k in range(4):
        sc.addSphere(0.4, position=[-8.0 + 2.2 * k, 0.45, 6.0], allowSleep=allow)
    if late:  # lands on the middle stack after about 3.5 s
        sc.addBox([1, 1, 1], position=[0.2, 60.0, 0.1], allowSleep=allow)
    arr = sc.arrays()
    arr.params.sleeping, arr.params.sleep_speed, arr.params.sleep_time = True, 0.08, 0.6
    return arr


def test_oracle_sleeping_matches_the_reference_restatement(oracle_mod):
    sc = _pile()
    o = oracle_mod.OracleWorld(sc, fp64=True, app=True, colored=True)
    asleep, time = o.sleep_state()
    seen_sleep = seen_wake = False
    prev = 0
    for step in range(420):
        o.step_collide()
        o.step_solve()
        want_a, want_t = _after(o, sc.mass, sc.allow_sleep, [], sc.params.dt, 0.08, 0.6, asleep, time)
        o.sleep_after()
        asleep, time = o.sleep_state()
        assert np.array_equal(asleep, want_a), step
        assert np.abs(time - want_t).max() < 1e-12, step
        cnt = int(asleep.sum())
        seen_sleep |= cnt > 0
        seen_wake |= prev > 0 and cnt == 0
        prev = cnt
        if asleep.any():
            assert np.all(o.bodies()["vel"][asleep] == 0)
    assert seen_sleep and seen_wake


def test_sleeping_bodies_hold_still_and_edits_wake_the_world(oracle_mod):
    sc = _pile(late=False)
    o = oracle_mod.OracleWorld(sc, fp64=False, app=True, colored=True)
    for _ in range(300):
        o.step(1)
        if o.sleep_state()[0][sc.mass > 0].all():
            break
    asleep, _ = o.sleep_state()
    assert asleep[sc.mass > 0].all()
    before = o.bodies()
    o.step(20)
    after = o.bodies()
    assert np.array_equal(before["pos"], after["pos"]) and np.array_equal(before["quat"], after["quat"])
    # a queued command wakes every body
    from avbd_gb300.pipeline import stage_edits
    o.edit(stage_edits([{"body": 3, "linearVelocity": [0, 2, 0]}], sc.n_bodies, sc.params.dt))
    assert not o.sleep_state()[0].any()
    o.step(1)
    assert not np.array_equal(after["pos"], o.bodies()["pos"])


@pytest.mark.parametrize("case", ["no_support", "disallowed"])
def test_islands_that_must_stay_awake(oracle_mod, case):
    sc = _pile(late=False)
    if case == "no_support":  # zero gravity, nothing touches the ground: no island is supported
        sc.params.gravity = 0.0
        sc.pos[1:, 1] += 5.0
        sc.vel[:] = 0.0
        sc.prev_vel[:] = 0.0
    else:  # one body of each island may not sleep
        sc.allow_sleep[[4, 8, 12, 13, 14, 15, 16]] = False
    o = oracle_mod.OracleWorld(sc, fp64=False, app=True, colored=True)
    o.step(200)
    assert not o.sleep_state()[0].any()
