"""Asynchronous ticks (needs a GPU).

A step is queued without waiting for the device (the reference's step never waits,
src/native/solver3D.js:350-359) and its launch sequence replays as a CUDA graph. Capacities that
overflow hold the tick on the device (every later state change of it and of the ticks queued
after it is skipped, as the reference's protectSolverStep turns an overflowing step's solve into
no-ops, src/gpu/gpuSolverKernels.js:72-102) and the held ticks re-run after growth: the bits equal
those of ticks run one at a time. The solve loop's schedules (the tile queue with several chunk
sizes and grid sizes, colour barriers) give the same bits. The tile queue's bounded wait, made to
run out on purpose, reports an error instead of hanging.
"""
import time

import numpy as np
import pytest

from avbd_gb300 import _lib as L
from avbd_gb300 import createSolverPipeline, workloads
from avbd_gb300.scene import SceneBuilder, SolverParams

pytestmark = pytest.mark.gpu

KEYS = ("position", "rotation", "velocity", "angular", "prev_velocity")


@pytest.fixture(scope="module")
def pipe():
    p = createSolverPipeline("gb300", device=0)
    yield p
    p.destroy()


def _dense_cluster(seed=7, n=300):
    rng = np.random.default_rng(seed)
    b = SceneBuilder(SolverParams(dt=1 / 60, gravity=-9.81, up=(0, 1, 0), iterations=4))
    b.rigid([40, 1, 40], 0, 0.5, [0, -0.5, 0])
    for _ in range(n):
        b.sphere(0.5, 1000, 0.5, list(rng.uniform([-2, 0.5, -2], [2, 4.5, 2])))
    return b.arrays()


def test_step_returns_before_the_device_finishes(pipe, monkeypatch):
    monkeypatch.setenv("AVBD_TUNE", "0")  # the autotuner's timed ticks launch directly
    worlds, _, _ = workloads.world_mix(256, target=130_000)
    b = pipe.createBatch(worlds)
    b.step(3)
    pipe.synchronize()
    t0 = time.perf_counter()
    b.step(12)
    queued = time.perf_counter() - t0
    pipe.synchronize()
    total = time.perf_counter() - t0
    print(f"queued in {queued * 1e3:.2f} ms, done after {total * 1e3:.2f} ms")
    assert queued < 0.5 * total
    prof = b.profileRead()
    assert prof["graphs_on"] == 1 and prof["graph_replays"] >= 9, prof  # recorded at its second sighting
    b.destroy()


def test_held_ticks_rerun_exactly(pipe):
    """Eight ticks queued together, the first of them overflowing the initial pair regions (and
    every tick behind it held), against the same eight ticks run one at a time with a read after
    each (the overflow then holds one tick only)."""
    scene = _dense_cluster()
    a = pipe.createSolver(scene)
    a.step(8)
    got = a.readBodyState()
    assert a.profileRead()["ticks_held"] >= 2
    b = pipe.createSolver(scene)
    for _ in range(8):
        b.step(1)
        b.readBodyState()
    ref = b.readBodyState()
    for k in KEYS:
        assert np.array_equal(got[k], ref[k]), k
    a.destroy()
    b.destroy()


SCHEDULES = [("queue", 1, 0, 128), ("queue", 2, 0, 128), ("queue", 4, 0, 128), ("queue", 2, 24, 128), ("queue", 8, 3, 128),
             ("queue", 1, 0, 256), ("queue", 2, 24, 256), ("barrier", 1, 0, 128), ("barrier", 2, 0, 128), ("barrier", 1, 5, 128),
             ("barrier", 1, 0, 256), ("barrier", 2, 0, 256)]


def test_solve_schedules_give_the_same_bits(pipe, monkeypatch):
    scenes = [workloads.mixed_pile(n, seed=300 + n, extent=5.0) for n in (16, 90, 400, 7)]
    scenes.append(workloads.cloth_wall(grid=8, wall=(3, 2, 2)))
    scenes.append(workloads.box_pile_c0(nx=4, ny=3, nz=4))
    states = []
    for mode, waves, blocks, tile in SCHEDULES:
        monkeypatch.setenv("AVBD_SOLVE", mode)
        monkeypatch.setenv("AVBD_SOLVE_WAVES", str(waves))
        monkeypatch.setenv("AVBD_SOLVE_BLOCKS", str(blocks))
        monkeypatch.setenv("AVBD_SOLVE_TILE", str(tile))
        batch = pipe.createBatch(scenes)
        batch.step(20)
        states.append([batch.readBodyState(k) for k in range(len(scenes))])
        batch.destroy()
    for s, cfg in zip(states[1:], SCHEDULES[1:]):
        for k in range(len(scenes)):
            for key in KEYS:
                assert np.array_equal(s[k][key], states[0][k][key]), (cfg, k, key)


def test_queue_wait_limit_reports_an_error(pipe, monkeypatch):
    """The tile queue's waits bounded at ~1 ms and made to wait for a count nothing reaches: the
    solve stops, the device stays usable, and the next call reports the error."""
    monkeypatch.setenv("AVBD_SOLVE", "queue")
    monkeypatch.setenv("AVBD_SOLVE_WAIT_CYCLES", "2000000")
    monkeypatch.setenv("AVBD_SOLVE_WAIT_PROBE", "1")
    w = pipe.createSolver(workloads.box_pile_c0(nx=3, ny=3, nz=3))
    w.step(1)
    with pytest.raises(L.AvbdError) as err:
        w.readBodyState()
    assert "wait limit" in str(err.value)
    w.destroy()
    monkeypatch.delenv("AVBD_SOLVE_WAIT_PROBE")
    monkeypatch.delenv("AVBD_SOLVE_WAIT_CYCLES")
    v = pipe.createSolver(workloads.box_pile_c0(nx=3, ny=3, nz=3))  # a fresh world runs normally
    v.step(3)
    assert np.isfinite(v.readBodyState()["position"]).all()
    v.destroy()


def test_pipelined_reads_equal_synchronous_reads(pipe):
    """Batch reads queued behind their steps (stepRead into two page-locked buffers, readDone on
    the previous one) give the poses a synchronous read gives after the same steps, also when the
    first steps overflow the initial pair regions and are held and re-run (with their reads)."""
    scenes = [_dense_cluster(seed=s) for s in (7, 8, 9)]
    a = pipe.createBatch(scenes)
    bufs = [a.pinnedPoses(), a.pinnedPoses()]
    got, tags = [], []
    for k in range(8):
        tags.append(a.stepRead(1, bufs[k % 2]))
        if k >= 1:
            assert a.readDone(tags[k - 1], wait=True)
            got.append(bufs[(k - 1) % 2].copy())
    assert a.readDone(tags[-1], wait=True)
    got.append(bufs[7 % 2].copy())
    assert a.profileRead()["ticks_held"] >= 1
    b = pipe.createBatch(scenes)
    for k in range(8):
        b.step(1)
        assert np.array_equal(got[k], b.readPoses()), k
    with pytest.raises(L.AvbdError):
        a.stepRead(1, np.zeros((a.bodyCount, 8), dtype=np.float32))  # not page-locked
    a.destroy()
    b.destroy()


def test_pipelined_reads_with_velocity_commands_and_held_steps(pipe):
    """Velocity commands queued between pipelined steps, with the first steps held (initial pair
    regions too small) and re-run: the poses read equal those of the same commands and steps made
    one at a time with synchronous reads."""
    scenes = [_dense_cluster(seed=s, n=260) for s in (21, 22)]
    rng = np.random.default_rng(3)
    cmds = []
    for k in range(6):
        dynamic = [o + i for o, sc in zip((0, scenes[0].n_bodies), scenes) for i in range(1, sc.n_bodies)]
        idx = rng.choice(dynamic, size=5, replace=False).astype(np.int64)
        vel = rng.uniform(-2, 2, size=(5, 3)).astype(np.float32)
        cmds.append((idx, vel))
    a = pipe.createBatch(scenes)
    bufs = [a.pinnedPoses(), a.pinnedPoses()]
    got, tags = [], []
    for k, (idx, vel) in enumerate(cmds):
        a.setVelocities(idx, linear=vel)
        tags.append(a.stepRead(1, bufs[k % 2]))
        if k >= 1:
            assert a.readDone(tags[k - 1], wait=True)
            got.append(bufs[(k - 1) % 2].copy())
    assert a.readDone(tags[-1], wait=True)
    got.append(bufs[(len(cmds) - 1) % 2].copy())
    b = pipe.createBatch(scenes)
    for k, (idx, vel) in enumerate(cmds):
        b.setVelocities(idx, linear=vel)
        b.step(1)
        assert np.array_equal(got[k], b.readPoses()), k
    a.destroy()
    b.destroy()
