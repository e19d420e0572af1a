"""Behaviour of the public API on the GPU world, after forge2d's own tests
(F2D/test/ffi/smoke_test.dart, world_test.dart, events_test.dart): box drop,
closest ray cast, AABB overlap, body accessors and impulses. Answers come
from the reference (tests/golden/api_ref.json) or from the oracle."""
from __future__ import annotations

import json
import math
import os

import numpy as np
import pytest

from forge2d_gb300 import scenes

pytestmark = pytest.mark.gpu

GOLD = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "api_ref.json")))


def test_box_drop_comes_to_rest(gpu_lib):
    from forge2d_gb300.world import World
    w = World(gravity=(0.0, -10.0))
    ground = w.create_body(type=0, positionY=-1.0)
    ground.create_box(50.0, 1.0)
    box = w.create_body(type=2, positionY=10.0)
    box.create_box(0.5, 0.5)
    for _ in range(200):
        assert w.step(1.0 / 60.0, 4) == 0
    x, y = box.position
    gx, gy = GOLD["drop"]["position"]
    assert abs(x - gx) < 1e-4 and abs(y - gy) < 1e-3
    assert box.mass == pytest.approx(1.0)
    # the reference's box is asleep by then (sleeping on by default)
    assert w._w.awake_body_count() == GOLD["drop"]["awake_bodies"] == 0
    assert not box.is_awake
    box.set_awake(True)
    assert box.is_awake
    w.destroy()


def test_ray_and_overlap_answers(gpu_lib):
    from forge2d_gb300.world import GpuWorld
    g = GpuWorld(scenes.world_def(gravityY=0.0))
    bb = g.create_body(scenes.body_def(type=0, positionX=2.0))
    s = g.create_box(bb, scenes.shape_def(), 0.5, 0.5)
    assert s[0] - 1 == GOLD["ray"]["shape"]
    hit = g.cast_ray_closest(0.0, 0.0, 10.0, 0.0)
    assert hit is not None
    assert [hit[0]] + hit[1].tolist() == pytest.approx(GOLD["ray"]["hit"], abs=1e-6)
    assert g.cast_ray_closest(0.0, 5.0, 10.0, 0.0) is None
    # filtered out by the query mask
    assert g.cast_ray_closest(0.0, 0.0, 10.0, 0.0, cat=1, mask=2) is None
    c1 = g.create_body(scenes.body_def(type=0, positionX=-5.0, positionY=5.0))
    s1 = g.create_circle(c1, scenes.shape_def(), 0.0, 0.0, 0.5)
    c2 = g.create_body(scenes.body_def(type=0, positionX=20.0, positionY=20.0))
    g.create_circle(c2, scenes.shape_def(), 0.0, 0.0, 0.5)
    assert s1[0] - 1 == GOLD["overlap"]["inside"]
    assert sorted(int(x) for x in g.overlap_aabb(-6.0, 4.0, -4.0, 6.0)) == GOLD["overlap"]["result"]
    assert len(g.overlap_aabb(100.0, 100.0, 101.0, 101.0)) == 0
    g.close()


def test_queries_match_oracle_on_moving_pile(gpu_lib, port_lib):
    wkw = dict(enableSleep=0, enableContinuous=1)
    kw = dict(count=400, seed=4, width=20.0, height=20.0)
    from forge2d_gb300.world import GpuWorld
    g = GpuWorld(scenes.world_def(**wkw))
    p = port_lib.PortWorld(scenes.world_def(**wkw))
    scenes.build(g, "pile", **kw)
    scenes.build(p, "pile", **kw)
    rng = np.random.default_rng(9)
    hits = 0
    for f in range(1, 61):
        g.step(1.0 / 60.0, 4)
        p.step(1.0 / 60.0, 4)
        if f % 10:
            continue
        for _ in range(25):
            o = rng.uniform(-12, 12, 2)
            t = rng.uniform(-15, 15, 2)
            a = g.cast_ray_closest(o[0], o[1], t[0], t[1])
            b = p.cast_ray_closest(o[0], o[1], t[0], t[1])
            assert (a is None) == (b is None)
            if a is not None:
                hits += 1
                assert a[0] == b[0]
                assert np.array_equal(a[1].view(np.uint32), b[1].view(np.uint32))
            lo = rng.uniform(-12, 8, 2)
            hi = lo + rng.uniform(0.1, 6, 2)
            assert sorted(g.overlap_aabb(lo[0], lo[1], hi[0], hi[1]).tolist()) == \
                sorted(p.overlap_aabb(lo[0], lo[1], hi[0], hi[1]).tolist())
    assert hits > 30
    g.close()
    p.close()


def test_chain_queries_match_oracle(gpu_lib, port_lib):
    """Chain segments: the segment ids of each chain, and ray casts that
    pass one-sided segments from behind, against the oracle."""
    wkw = dict(enableSleep=0, enableContinuous=1)
    from forge2d_gb300.world import GpuWorld
    g = GpuWorld(scenes.world_def(**wkw))
    p = port_lib.PortWorld(scenes.world_def(**wkw))
    scenes.build(g, "chain_terrain", count=150)
    scenes.build(p, "chain_terrain", count=150)
    ch = g.create_chain(g.create_body(scenes.body_def(type=scenes.STATIC)), [(0, 0), (1, 0), (2, 0), (3, 1)])
    segs = g.chain_segments(ch)
    assert len(segs) == 1 and g.lib.f2d_shape_get_type(*segs[0]) == 4
    rng = np.random.default_rng(3)
    hits = 0
    for f in range(1, 41):
        g.step(1.0 / 60.0, 4)
        p.step(1.0 / 60.0, 4)
        if f % 10:
            continue
        for _ in range(40):
            o = rng.uniform(-24, 24, 2) + np.array([0.0, 20.0])
            t = rng.uniform(-30, 30, 2)
            a = g.cast_ray_closest(o[0], o[1], t[0], t[1])
            b = p.cast_ray_closest(o[0], o[1], t[0], t[1])
            assert (a is None) == (b is None)
            if a is not None:
                hits += 1
                assert a[0] == b[0]
                assert np.array_equal(a[1].view(np.uint32), b[1].view(np.uint32))
    assert hits > 50
    g.close()
    p.close()


def test_body_accessors_and_impulses(gpu_lib):
    from forge2d_gb300.world import World
    w = World(gravity=(0.0, 0.0))
    b = w.create_body(type=2, positionX=1.0, positionY=2.0)
    b.create_circle(0.5)
    m = b.mass
    assert m == pytest.approx(math.pi * 0.25, rel=1e-6)
    assert b.position == pytest.approx((1.0, 2.0))
    b.linear_velocity = (3.0, -1.0)
    assert b.linear_velocity == pytest.approx((3.0, -1.0))
    w.step(0.5, 4)
    assert b.position == pytest.approx((2.5, 1.5), abs=1e-5)
    b.apply_linear_impulse_to_center((m * 1.0, 0.0))
    assert b.linear_velocity == pytest.approx((4.0, -1.0), abs=1e-5)
    b.angular_velocity = 2.0
    assert b.angular_velocity == pytest.approx(2.0)
    b.set_transform((0.0, 0.0), (0.0, 1.0))
    assert b.position == pytest.approx((0.0, 0.0))
    assert b.rotation == pytest.approx((0.0, 1.0), abs=1e-6)
    w.gravity = (0.0, -5.0)
    assert w.gravity == (0.0, -5.0)
    assert b.is_valid and b.type == 2
    w.destroy()


def test_per_body_reads_after_a_step_are_cheap(gpu_lib):
    """forge2d reads each body's position through bodyGetPosition
    (raw_box2d.dart); after a step the first read refreshes the host mirror
    of every body row at once (under 50 ms for 100k bodies) and later reads
    copy nothing; the reads return the device state (checked against the
    bulk reader)."""
    import ctypes as C
    import time
    from forge2d_gb300.world import GpuWorld
    g = GpuWorld(scenes.world_def(enableSleep=0, enableContinuous=1))
    scenes.build(g, "pile", count=100_000, seed=1234)
    for _ in range(3):
        assert g.step(1.0 / 60.0, 4) == 0
    assert g.sync() == 0
    ids = [g._body(b) for b in sorted(g._wg["body"])]
    fn = g.lib.f2d_body_get_position
    x, y = C.c_double(0.0), C.c_double(0.0)
    px, py = C.byref(x), C.byref(y)
    got = np.zeros((len(ids), 2))
    t0 = time.perf_counter()
    fn(ids[0][0], ids[0][1], px, py)     # refreshes the whole mirror
    first_ms = 1000.0 * (time.perf_counter() - t0)
    t1 = time.perf_counter()
    for k, (i1, wg) in enumerate(ids):
        fn(i1, wg, px, py)
        got[k, 0] = x.value
        got[k, 1] = y.value
    per_call_us = 1e6 * (time.perf_counter() - t1) / len(ids)
    rows = g.bodies()
    assert np.array_equal(got.astype(np.float32), rows[:len(ids), :2])
    assert len(ids) > 100_000
    # one bulk refresh; afterwards a read costs the ctypes call (a device
    # synchronisation and seven copies per read cost tens of microseconds)
    assert first_ms < 50.0, first_ms
    assert per_call_us < 8.0, per_call_us
    # a body moved on the host stays authoritative until the next step
    i1, wg = ids[5]
    g.lib.f2d_body_set_transform(i1, wg, 1.5, 900.0, 1.0, 0.0)
    fn(i1, wg, px, py)
    assert (x.value, y.value) == (1.5, 900.0)
    assert g.step(1.0 / 60.0, 4) == 0
    fn(i1, wg, px, py)
    assert abs(y.value - 900.0) < 1.0
    g.close()
