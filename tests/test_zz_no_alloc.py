"""f2d_world_overlap_aabb_noalloc against f2d_world_overlap_aabb (GPU only).

The allocation-free variant keeps its scratch in a file-scope device array
(at most F2D_OVERLAP_NOALLOC_MAX_SHAPES shapes) instead of allocating per
call. Two calls in a row must each return exactly what the allocating entry
point returns -- count, order and ids, with a roomy and with a short output
buffer -- and a world past the array's size, or one whose pending uploads
would allocate (grown rows, a changed sensor list), must be rejected without
output.
Collected last so that it also runs after every other test in one process.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from forge2d_gb300 import scenes

pytestmark = pytest.mark.gpu

MAX_SHAPES = 262144          # F2D_OVERLAP_NOALLOC_MAX_SHAPES
TOO_MANY, NEEDS_GROWTH = -1, -2


def _call(lib, fn, wid, box, cat, mask, capacity):
    """One overlap call; the output buffer is pre-filled with -7 so that
    rows past the returned count can be checked as untouched."""
    out = np.full((max(capacity, 1), 2), -7, np.int32)
    n = fn(wid, box[0], box[1], box[2], box[3], cat, mask, out.ctypes.data_as(C.POINTER(C.c_int32)), capacity)
    return n, out


def test_noalloc_overlap_matches_allocating_entry_point(gpu_lib):
    import torch
    from forge2d_gb300.world import GpuWorld

    g = GpuWorld(scenes.world_def(enableSleep=0, enableContinuous=1))
    scenes.pile(g, count=3000, seed=17, width=40.0, height=120.0)
    for _ in range(30):
        assert g.step(1.0 / 60.0, 4) == 0
    lib = g.lib
    rng = np.random.default_rng(3)
    boxes = [(-25.0, -3.0, 25.0, 130.0)]          # everything
    for _ in range(12):
        lo = rng.uniform(-22, 15, 2)
        hi = lo + rng.uniform(0.5, 12, 2)
        boxes.append((lo[0], lo[1], hi[0], hi[1]))
    boxes.append((500.0, 500.0, 501.0, 501.0))    # nothing
    cases = [(box, cat, mask, capacity) for box in boxes for cat, mask in ((1, -1), (1, 2))
             for capacity in (1 << 14, 7)]
    refs = [_call(lib, lib.f2d_world_overlap_aabb, g.id, *case) for case in cases]
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    checked = 0
    for case, ref in zip(cases, refs):
        capacity = case[3]
        for _ in range(2):       # two calls in a row share the static scratch
            got = _call(lib, lib.f2d_world_overlap_aabb_noalloc, g.id, *case)
            assert got[0] == ref[0]
            m = min(ref[0], capacity)
            assert np.array_equal(got[1][:m], ref[1][:m])
            assert (got[1][m:] == -7).all()
        checked += ref[0] > 0
    assert checked > 10
    # no device memory was taken by the allocation-free calls
    assert torch.cuda.mem_get_info()[0] == free_before
    g.close()


def test_noalloc_overlap_rejects_oversize_and_pending_growth(gpu_lib):
    from forge2d_gb300.world import GpuWorld

    g = GpuWorld(scenes.world_def(enableSleep=0))
    ground = g.create_body(scenes.body_def(type=0))
    g.create_box(ground, scenes.shape_def(), 5.0, 1.0)
    body = g.create_body(scenes.body_def(type=2, positionY=3.0))
    g.create_circle(body, scenes.shape_def(), 0.0, 0.0, 0.5)
    g.step(1.0 / 60.0, 4)
    n, _ = g.overlap_aabb_noalloc(-10.0, -10.0, 10.0, 10.0)
    assert n == 2
    # shapes created past the device capacity since the last step
    for k in range(4096):
        g.create_circle(ground, scenes.shape_def(), float(k % 64), float(k // 64), 0.1)
    n, rows = g.overlap_aabb_noalloc(-10.0, -10.0, 10.0, 10.0)
    assert n == NEEDS_GROWTH and len(rows) == 0
    g.step(1.0 / 60.0, 4)
    n, _ = g.overlap_aabb_noalloc(-1000.0, -1000.0, 1000.0, 1000.0)
    assert n == 4098
    g.close()

    # a sensor shape created after a step makes the next upload reallocate
    # the sensor buffers: the call is refused instead of allocating, and
    # answers again once a step has done the upload
    import torch
    sw = GpuWorld(scenes.world_def(enableSleep=0))
    base = sw.create_body(scenes.body_def(type=0))
    sw.create_box(base, scenes.shape_def(), 5.0, 1.0)
    sw.step(1.0 / 60.0, 4)
    n, _ = sw.overlap_aabb_noalloc(-10.0, -10.0, 10.0, 10.0)
    assert n == 1
    holder = sw.create_body(scenes.body_def(type=2, positionY=4.0))
    sw.create_circle(holder, scenes.shape_def(isSensor=1, enableSensorEvents=1), 0.0, 0.0, 0.5)
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    n, rows = sw.overlap_aabb_noalloc(-10.0, -10.0, 10.0, 10.0)
    assert n == NEEDS_GROWTH and len(rows) == 0
    assert torch.cuda.mem_get_info()[0] == free_before
    sw.step(1.0 / 60.0, 4)
    n, _ = sw.overlap_aabb_noalloc(-10.0, -10.0, 10.0, 10.0)
    assert n >= 1
    sw.close()

    # a world holding more shapes than the static scratch takes is refused
    big = GpuWorld(scenes.world_def(enableSleep=0))
    big.reserve(bodies=2, shapes=MAX_SHAPES + 1)
    anchor = big.create_body(scenes.body_def(type=0))
    lib = big.lib
    sd = big._sd(scenes.shape_def())
    i1, wg = C.c_int32(0), C.c_int32(0)
    for k in range(MAX_SHAPES + 1):
        lib.f2d_create_circle_shape(anchor[0], anchor[1], sd, float(k % 512), float(k // 512), 0.25,
                                    C.byref(i1), C.byref(wg))
    n, rows = big.overlap_aabb_noalloc(-1.0, -1.0, 1.0, 1.0, capacity=16)
    assert n == TOO_MANY and len(rows) == 0
    big.close()
