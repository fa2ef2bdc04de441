"""The allocation-free selected-bodies read (avbd_world_read_selected_noalloc), called through
the C ABI.

Hosts that must not allocate device memory while they run (a per-frame pose read in a render or
input loop, where cudaMalloc/cudaFree can wait for the whole device; a server whose device budget
is committed to world state) use this variant: it stages through one fixed per-GPU device buffer
instead of allocating. Its output must equal the allocating avbd_world_read_selected's bit for
bit (the tolerance of the parity tests) on two calls in a row, and requests above the buffer's
capacity must be refused. This file is collected last so a failure here leaves every other test
already run.
"""
import numpy as np
import pytest

from avbd_gb300 import _lib as L
from avbd_gb300 import createSolverPipeline, workloads

pytestmark = pytest.mark.gpu


def _read_noalloc(world, idx, poses_only):
    stride = 8 if poses_only else 40
    out = np.full(idx.size * stride, np.nan, dtype=np.float32)
    status = L.lib().avbd_world_read_selected_noalloc(world._h, L.uptr(idx), idx.size, int(poses_only), L.fptr(out))
    L.check(status)
    return out


def test_noalloc_read_matches_allocating_read():
    pipe = createSolverPipeline("gb300", device=0)
    scene = workloads.box_pile_c0(nx=4, ny=4, nz=4)
    world = pipe.createSolver(scene)
    world.step(20)
    rng = np.random.default_rng(11)
    for poses_only in (False, True):
        # two calls in a row, different selections; each against the allocating entry point
        for call in range(2):
            idx = rng.integers(0, world.bodyCount, size=37 + call * 20).astype(np.uint32)
            expected = world.readSelectedBodies(idx, posesOnly=poses_only)
            got = _read_noalloc(world, idx, poses_only)
            assert np.array_equal(got, expected), (poses_only, call)
    world.step(1)
    idx = np.arange(world.bodyCount, dtype=np.uint32)
    assert np.array_equal(_read_noalloc(world, idx, False), world.readSelectedBodies(idx))
    # the capacity limit is enforced before any work is queued
    big = np.zeros(L.NOALLOC_MAX_SELECTED + 1, dtype=np.uint32)
    out = np.zeros(big.size * 8, dtype=np.float32)
    status = L.lib().avbd_world_read_selected_noalloc(world._h, L.uptr(big), big.size, 1, L.fptr(out))
    assert status == L.AVBD_E_CAPACITY
    assert b"at most" in L.lib().avbd_last_error()
    pipe.destroy()
