"""World server (continuous batching, budgeted admission, LRU eviction) through the C ABI.

The serving contract is that a world's results do not depend on how it is served: K queued
steps, run one per tick among any other worlds, across evictions to host memory and restores,
give the same bits as the same scene stepped K times on its own. Every comparison here is
exact (np.array_equal on float32 state).
"""
import numpy as np
import pytest

import ref_scenes
from avbd_gb300 import _lib as L
from avbd_gb300 import createSolverPipeline, workloads
from avbd_gb300.scene import SolverParams

pytestmark = pytest.mark.gpu

KEYS = ("position", "rotation", "velocity", "angular", "prev_velocity")


@pytest.fixture(scope="module")
def pipe():
    p = createSolverPipeline("gb300", device=0)
    yield p
    p.destroy()


def _scenes():
    """Box/sphere piles of different sizes plus joint scenes (rope, bridge, breakable)."""
    out = [workloads.mixed_pile(n, seed=900 + n, extent=4.0 + n / 100) for n in (60, 150, 240, 90)]
    for idx in (5, 12, 13):
        sc = ref_scenes.build(idx)
        sc.params = SolverParams(dt=1 / 60, gravity=-10.0, up=(0.0, 0.0, 1.0), iterations=10)
        out.append(sc)
    return out


def _alone(pipe, scene, steps):
    w = pipe.createSolver(scene)
    w.step(steps)
    st = w.readBodyState()
    w.destroy()
    return st


def _assert_same(a, b, what):
    for k in KEYS:
        assert np.array_equal(a[k], b[k]), (what, k, float(np.max(np.abs(a[k] - b[k]))))


def _drain(server, max_ticks=10_000):
    for _ in range(max_ticks):
        if server.tick() == 0 and server.stats()["pending_worlds"] == 0:
            return
    raise AssertionError("server did not drain")


def test_served_worlds_equal_worlds_stepped_alone(pipe):
    scenes = _scenes()
    server = pipe.createServer(budgetBytes=8 << 30)
    ids = [server.admit(sc) for sc in scenes]
    rng = np.random.default_rng(5)
    total = {i: 0 for i in ids}
    tickets = []
    # interleave requests with ticks: worlds join and leave the tick's batch
    for round_ in range(6):
        for i in ids:
            if rng.random() < 0.6:
                k = int(rng.choice([1, 4, 16]))
                tickets.append(server.advance(i, k))
                total[i] += k
        for _ in range(int(rng.integers(1, 6))):
            server.tick()
    _drain(server)
    done = server.completed()
    assert sorted(done) == sorted(tickets)
    for i, sc in zip(ids, scenes):
        info = server.info(i)
        assert info["steps"] == total[i] and info["queued"] == 0
        _assert_same(server.readBodyState(i), _alone(pipe, sc, total[i]), ("world", i))
    st = server.stats()
    assert st["body_steps"] == sum(total[i] * server.info(i)["bodies"] for i in ids)
    server.destroy()


def test_eviction_and_restore_are_exact(pipe):
    """A budget that holds only some of the worlds: admitting and advancing the rest evicts the
    least recently used idle ones, which are restored when their next request arrives."""
    scenes = [workloads.mixed_pile(200, seed=700 + k, extent=5.0) for k in range(8)]
    probe = pipe.createServer(budgetBytes=1 << 40, initialBodies=1024, initialWorlds=16)
    budget = probe.stats()["device_bytes"] + (64 << 10)  # the initial arena: about 5 of these worlds
    probe.destroy()
    server = pipe.createServer(budgetBytes=budget, initialBodies=1024, initialWorlds=16)
    ids, total = [], {}
    for sc in scenes:
        i = server.admit(sc)
        ids.append(i)
        total[i] = 0
        server.advance(i, 3)
        total[i] += 3
        _drain(server)
    st = server.stats()
    assert st["evictions"] > 0 and st["evicted_worlds"] > 0, st
    assert st["peak_device_bytes"] <= budget, st
    # advance every world again (evicted ones come back), explicitly evict one mid-run
    for i in ids:
        server.advance(i, 5)
        total[i] += 5
    server.tick()
    server.tick()
    idle = [i for i in ids if server.info(i)["resident"]]
    _drain(server)
    victim = ids[-1]
    server.evict(victim)
    assert not server.info(victim)["resident"]
    before = server.readBodyState(victim)  # read from the host copy
    server.advance(victim, 2)
    total[victim] += 2
    _drain(server)
    assert server.info(victim)["resident"]
    st = server.stats()
    assert st["restores"] > 0 and st["peak_device_bytes"] <= budget, st
    for i, sc in zip(ids, scenes):
        _assert_same(server.readBodyState(i), _alone(pipe, sc, total[i]), ("world", i))
    assert not np.array_equal(before["position"], server.readBodyState(victim)["position"])
    assert idle  # some worlds stayed resident through the second round
    server.destroy()


def test_read_poses_mixes_resident_and_evicted_worlds(pipe):
    scenes = [workloads.mixed_pile(n, seed=300 + n, extent=4.0) for n in (40, 70, 55)]
    server = pipe.createServer(budgetBytes=4 << 30)
    ids = [server.admit(sc) for sc in scenes]
    for i in ids:
        server.advance(i, 7)
    _drain(server)
    server.evict(ids[1])
    poses = server.readPoses([ids[2], ids[1], ids[0]])
    rows = 0
    for i in (ids[2], ids[1], ids[0]):
        st = server.readBodyState(i)
        n = st["position"].shape[0]
        assert np.array_equal(poses[rows:rows + n, 0:3], st["position"])
        assert np.array_equal(poses[rows:rows + n, 4:8], st["rotation"])
        rows += n
    assert rows == poses.shape[0]
    server.destroy()


def test_admission_fails_cleanly_when_nothing_can_be_evicted(pipe):
    small = workloads.mixed_pile(100, seed=11, extent=4.0)
    server = pipe.createServer(budgetBytes=1 << 40, initialBodies=1024, initialWorlds=16)
    budget = server.stats()["device_bytes"] + (32 << 10)
    server.destroy()
    server = pipe.createServer(budgetBytes=budget, initialBodies=1024, initialWorlds=16)
    a = server.admit(small)
    server.advance(a, 50)  # busy: not evictable
    big = workloads.mixed_pile(1500, seed=12, extent=8.0)
    with pytest.raises(L.AvbdError) as e:
        server.admit(big)
    assert e.value.code == L.AVBD_E_CAPACITY
    st = server.stats()
    assert st["rejected"] == 1 and st["live_worlds"] == 1
    _drain(server)
    _assert_same(server.readBodyState(a), _alone(pipe, small, 50), "survivor")
    # tickets for zero steps complete at once; unknown worlds are refused
    t = server.advance(a, 0)
    assert t in server.completed()
    with pytest.raises(L.AvbdError):
        server.advance(12345, 1)
    server.release(a)
    assert server.stats()["live_worlds"] == 0
    server.destroy()
