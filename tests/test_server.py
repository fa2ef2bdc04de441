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


def _poses(state):
    """8 floats per body (pos, friction slot, quat) as a reply carries them, from a state read."""
    return state["position"], state["rotation"]


def test_multi_step_ticks_with_replies_equal_worlds_alone(pipe):
    """Requests of K = 1, 4 and 16 steps run in one multi-step tick each (the steps queued back to
    back on the device) give the same bits as the worlds stepped alone, and each reply carries its
    world's poses right after the step that completed the request."""
    scenes = _scenes()[:5]
    server = pipe.createServer(budgetBytes=8 << 30)
    ids = [server.admit(sc) for sc in scenes]
    ks = [1, 4, 16, 7, 16]
    tickets = {server.advance(w, k): (i, k) for i, (w, k) in enumerate(zip(ids, ks))}
    taken = server.tick(maxSteps=16, replies=True)
    assert taken == sum(ks)
    assert server.completed() == []  # captured replies are reported by ready(), not completed()
    got = set()
    for _ in range(2000):
        got.update(server.ready())
        if len(got) == len(tickets):
            break
    else:
        got.update(server.ready(wait=True))
    assert got == set(tickets)
    for t, (i, k) in tickets.items():
        rep = server.takeReply(t)
        ref = _alone(pipe, scenes[i], k)
        assert rep.shape == (scenes[i].n_bodies, 8)
        assert np.array_equal(rep[:, :3], ref["position"]) and np.array_equal(rep[:, 4:], ref["rotation"]), (i, k)
        _assert_same(server.readBodyState(ids[i]), ref, f"world {i}")
    with pytest.raises(L.AvbdError):
        server.takeReply(next(iter(tickets)))  # handed out once
    server.destroy()


def test_world_admitted_while_ticks_are_in_flight(pipe):
    """Admission does not wait for the queued ticks: a world admitted while another world's steps
    are still running on the device evolves bit for bit as it does alone, and so does the other."""
    a_scene, b_scene = _scenes()[1], _scenes()[2]
    server = pipe.createServer(budgetBytes=8 << 30, initialBodies=4096, initialWorlds=16)
    a = server.admit(a_scene)
    server.advance(a, 24)
    server.tick(maxSteps=12)          # 12 steps queued, not waited for
    b = server.admit(b_scene)         # admitted while they run
    server.advance(b, 10)
    server.tick(maxSteps=16)          # a's last 12 steps with b's 10
    _assert_same(server.readBodyState(a), _alone(pipe, a_scene, 24), "a")
    _assert_same(server.readBodyState(b), _alone(pipe, b_scene, 10), "b")
    server.destroy()


def test_fence_wait_on_a_worker_thread_then_replies_without_waiting(pipe):
    """The Node addon's request loop: a multi-step tick with replies is queued, a worker thread
    waits on a fence after it (the one thread-safe entry point) while the caller queues the next
    tick, and then every reply of the first tick is ready without waiting for the device."""
    import threading
    scenes = _scenes()[:3]
    server = pipe.createServer(budgetBytes=8 << 30)
    ids = [server.admit(sc) for sc in scenes]
    first = {server.advance(w, 8): i for i, w in enumerate(ids)}
    server.tick(maxSteps=8, replies=True)
    fence = pipe.fence()
    waited = threading.Event()
    worker = threading.Thread(target=lambda: (fence.wait(), waited.set()))
    worker.start()
    second = {server.advance(w, 4): i for i, w in enumerate(ids)}
    server.tick(maxSteps=4, replies=True)  # queued while the worker waits
    worker.join(timeout=60)
    assert waited.is_set() and fence.done
    fence.destroy()
    got = set(server.ready())
    assert set(first) <= got
    for t, i in first.items():
        rep = server.takeReply(t)
        ref = _alone(pipe, scenes[i], 8)
        assert np.array_equal(rep[:, :3], ref["position"]) and np.array_equal(rep[:, 4:], ref["rotation"]), i
    got |= set(server.ready(wait=True))
    assert set(second) <= got
    for t, i in second.items():
        rep = server.takeReply(t)
        ref = _alone(pipe, scenes[i], 12)
        assert np.array_equal(rep[:, :3], ref["position"]), i
    server.destroy()
