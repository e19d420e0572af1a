"""Parity of the CUDA world step with the oracle and the reference (GPU only).

* native mode (the default): the GPU keeps the reference's broadphase trees
  and creates contacts in the reference's order with LIFO id reuse, as the
  CPU restatement does, so every body state, manifold, colour count and
  event must agree with the restatement bit for bit, frame by frame, and
  with the reference's own committed fixtures;
* parity mode: replaying the reference's contact ids (the fixtures' plans)
  gives the same bit-exact result;
* the 256-frame penetration / kinetic-energy series equal the reference's.
"""
from __future__ import annotations

import os

import numpy as np
import pytest

from forge2d_gb300 import scenes

from parity import (MULTI_BLASTS, blast, compare_contacts, edit_motors, install_callbacks, multishape_scene, ray_answers,
                    rounded_rays, rounded_scene)
from test_oracle_golden import (CASES, GOLD, SENSOR_CASES, STATS_CASES, check_sensor_rows, check_sets, frame_stats,
                                replay, sensor_rows)

pytestmark = pytest.mark.gpu


def gpu_world(gpu_lib, wkw, solver="auto"):
    """solver "grid" forces the grid-wide cooperative solver kernel (the one
    large worlds use) instead of the thread-block-cluster one."""
    import os
    from forge2d_gb300.world import GpuWorld
    if solver == "grid":
        os.environ["F2D_NO_CLUSTER_SOLVER"] = "1"
    try:
        return GpuWorld(scenes.world_def(**wkw))
    finally:
        os.environ.pop("F2D_NO_CLUSTER_SOLVER", None)


def assert_bodies_equal(g, p, frame):
    gb, pb = g.bodies()[:, :9], p.bodies()[:, :9]
    assert gb.shape == pb.shape
    bad = np.argwhere(gb.view(np.uint32) != pb.view(np.uint32))
    assert len(bad) == 0, "frame %d: first differing (body, field) %s gpu %r port %r" % (
        frame, bad[0].tolist(), gb[tuple(bad[0])], pb[tuple(bad[0])])


NATIVE = [
    ("pyramid40", dict(enableSleep=0), "pyramid", dict(), 256, 16),
    ("pile400_ccd", dict(enableSleep=0, enableContinuous=1), "pile",
     dict(count=400, seed=1, width=30.0, height=50.0), 300, 25),
    ("pile600_no_ccd", dict(enableSleep=0, enableContinuous=0), "pile",
     dict(count=600, seed=2, width=24.0, height=60.0), 200, 25),
    ("pile_dense_overflow", dict(enableSleep=0, enableContinuous=1), "pile",
     dict(count=1500, seed=3, width=12.0, height=120.0, wall_height=130.0), 150, 30),
    ("pile_filtered", dict(enableSleep=0, enableContinuous=1), "pile",
     dict(count=700, seed=4, width=30.0, height=60.0, filters=True), 200, 25),
    ("chains", dict(enableSleep=0), "pyramids_chains", dict(pyramids=3, rows=8, chains=10, links=25), 300, 25),
    ("joint_gallery", dict(enableSleep=0), "joint_gallery", dict(copies=6), 400, 25),
    # weld cantilevers (stiff and soft), distance rods, springs with limits, motors
    ("joint_zoo", dict(enableSleep=0), "joint_zoo", dict(copies=8), 400, 25),
    # prismatic lifts and springs, wheeled carts, motor, mouse and filter joints
    ("joint_rigs", dict(enableSleep=0), "joint_rigs", dict(copies=8), 400, 25),
    # chain shapes (one-sided segments, GJK-cached manifolds), with and
    # without continuous collision
    ("chain_terrain", dict(enableSleep=0, enableContinuous=0), "chain_terrain", dict(count=600), 300, 25),
    ("chain_terrain_ccd", dict(enableSleep=0, enableContinuous=1), "chain_terrain", dict(count=600), 300, 25),
    ("batched24", dict(enableSleep=0, enableContinuous=1), "batched", dict(worlds=24, seed=3), 200, 25),
    # overflow constraints solved by levels: a 150-deep chain (past the
    # parallel levels, into the serial tail), overflow joints, and many
    # short independent chains
    ("overflow_heap", dict(enableSleep=0, enableContinuous=1), "overflow_heap", dict(), 200, 25),
    ("overflow_platforms", dict(enableSleep=0), "overflow_heap",
     dict(platforms=12, per=30, long_count=8, spokes=0), 120, 20),
    # more overflow constraints than the shared-memory lists hold
    ("overflow_long", dict(enableSleep=0), "overflow_heap", dict(platforms=0, long_count=3200, spokes=0), 40, 10),
]


@pytest.mark.parametrize("solver", ["auto", "grid"])
@pytest.mark.parametrize("name,wkw,scene,kw,frames,every", NATIVE, ids=[n[0] for n in NATIVE])
def test_gpu_matches_port_bit_exact(gpu_lib, port_lib, name, wkw, scene, kw, frames, every, solver):
    g = gpu_world(gpu_lib, wkw, solver)
    p = port_lib.PortWorld(scenes.world_def(**wkw))
    scenes.build(g, scene, **kw)
    scenes.build(p, scene, **kw)
    saw_overflow = False
    for f in range(1, frames + 1):
        assert g.step(1.0 / 60.0, 4) == 0
        p.step(1.0 / 60.0, 4)
        assert_bodies_equal(g, p, f)
        if f % every == 0 or f == frames:
            assert compare_contacts(g, p) == [], "frame %d" % f
            gc, pc = g.color_counts(), p.color_counts()
            assert np.array_equal(gc, pc), "frame %d colours gpu %s port %s" % (f, gc, pc)
            saw_overflow |= bool(gc[11] > 0)
    assert g.sync() == 0
    if name in ("pile_dense_overflow", "overflow_heap", "overflow_platforms", "overflow_long"):
        assert saw_overflow, "scene meant to exercise the overflow colour did not reach it"
    g.close()
    p.close()


@pytest.mark.parametrize("sleep", [0, 1])
def test_gpu_explode_matches_port(gpu_lib, port_lib, sleep):
    """b2World_Explode between steps (waking sleeping sets, falloff, mask):
    bit-identical to the oracle."""
    wkw = dict(enableSleep=sleep, enableContinuous=1)
    g = gpu_world(gpu_lib, wkw)
    p = port_lib.PortWorld(scenes.world_def(**wkw))
    for w in (g, p):
        scenes.build(w, "pile", count=300, seed=3, width=20.0, height=30.0)
    for f in range(1, 401):
        blast(g, f)
        blast(p, f)
        assert g.step(1.0 / 60.0, 4) == 0
        p.step(1.0 / 60.0, 4)
        assert_bodies_equal(g, p, f)
    assert g.sync() == 0
    g.close()
    p.close()


@pytest.mark.parametrize("sleep", [0, 1])
def test_gpu_explode_multishape_matches_port(gpu_lib, port_lib, sleep):
    """Explosions over bodies of several shapes through sleeping sets: shapes
    in the dynamic tree's query order (wake order, impulse sums)."""
    wkw = dict(enableSleep=sleep, enableContinuous=1)
    g = gpu_world(gpu_lib, wkw)
    p = port_lib.PortWorld(scenes.world_def(**wkw))
    for w in (g, p):
        multishape_scene(w)
    for f in range(1, 321):
        if f in MULTI_BLASTS:
            x, y, r, fo, ipl, mask = MULTI_BLASTS[f]
            for w in (g, p):
                w.explode(x, y, r, fo, ipl, mask=mask)
        assert g.step(1.0 / 60.0, 4) == 0
        p.step(1.0 / 60.0, 4)
        assert_bodies_equal(g, p, f)
    g.close()
    p.close()


@pytest.mark.parametrize("sleep", [0, 1])
def test_gpu_motor_edits_match_port(gpu_lib, port_lib, sleep):
    """Joint motors switched and retuned between steps (uploaded with the
    next step; switching clears the motor impulse on the device)."""
    wkw = dict(enableSleep=sleep, enableContinuous=1)
    g = gpu_world(gpu_lib, wkw)
    p = port_lib.PortWorld(scenes.world_def(**wkw))
    mg, mp = [], []
    scenes.build(g, "joint_rigs", copies=3, motors=mg)
    scenes.build(p, "joint_rigs", copies=3, motors=mp)
    for f in range(1, 341):
        edit_motors(g, mg, f)
        edit_motors(p, mp, f)
        assert g.step(1.0 / 60.0, 4) == 0
        p.step(1.0 / 60.0, 4)
        assert_bodies_equal(g, p, f)
    assert g.sync() == 0
    g.close()
    p.close()


@pytest.mark.parametrize("scene,kw", [("joint_gallery", dict(copies=2)), ("joint_zoo", dict(copies=2)),
                                      ("joint_rigs", dict(copies=2))], ids=["revolute", "weld_distance", "rigs"])
def test_gpu_joint_constraint_matches_port(gpu_lib, port_lib, scene, kw):
    """Constraint force and torque of every joint (b2Joint_GetConstraint*)."""
    wkw = dict(enableSleep=0, enableContinuous=1)
    g = gpu_world(gpu_lib, wkw)
    p = port_lib.PortWorld(scenes.world_def(**wkw))
    scenes.build(g, scene, **kw)
    scenes.build(p, scene, **kw)
    world0 = g._body(0)[1] & 0xffff
    nonzero = 0
    for f in range(1, 201):
        g.step(1.0 / 60.0, 4)
        p.step(1.0 / 60.0, 4)
        if f % 20 == 0:
            for j in range(40):
                a = g.joint_constraint((j + 1, world0 | (1 << 16)))
                b = p.joint_constraint(j)
                assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), (f, j, a, b)
                nonzero += bool(np.any(a != 0))
    assert nonzero > 50
    g.close()
    p.close()


def test_gpu_cast_ray_callback_matches_port(gpu_lib, port_lib):
    """Callback ray casts (closest-hit and all-hits callbacks) on the chain
    scene against the oracle."""
    wkw = dict(enableSleep=0, enableContinuous=0)
    g = gpu_world(gpu_lib, wkw)
    p = port_lib.PortWorld(scenes.world_def(**wkw))
    for w in (g, p):
        scenes.build(w, "chain_terrain", count=150)
    for _ in range(60):
        g.step(1.0 / 60.0, 4)
        p.step(1.0 / 60.0, 4)
    rng = np.random.default_rng(1)
    rays = [(rng.uniform(-20, 20, 2) + [0.0, 15.0], rng.uniform(-30, 30, 2)) for _ in range(150)]
    assert ray_answers(g, rays) == ray_answers(p, rays)
    g.close()
    p.close()


def test_gpu_rounded_polygon_rays_match_port(gpu_lib, port_lib):
    """Rays against rounded boxes and polygons (the shape-cast path) on the
    GPU against the oracle."""
    wkw = dict(enableSleep=0, enableContinuous=1)
    g = gpu_world(gpu_lib, wkw)
    p = port_lib.PortWorld(scenes.world_def(**wkw))
    for w in (g, p):
        rounded_scene(w)
    for _ in range(40):
        g.step(1.0 / 60.0, 4)
        p.step(1.0 / 60.0, 4)
    rays = rounded_rays()
    assert ray_answers(g, rays) == ray_answers(p, rays)
    g.close()
    p.close()


@pytest.mark.parametrize("sleep", [0, 1])
def test_gpu_callbacks_match_port(gpu_lib, port_lib, sleep):
    """Custom filter (new pairs on the host between pair finding and contact
    creation; continuous candidates between a listing pass and the impact
    pass) and pre-solve (host decision between the manifold listing and the
    contact update): bit-identical to the oracle with the same callbacks."""
    wkw = dict(enableSleep=sleep, enableContinuous=1)
    g = gpu_world(gpu_lib, wkw)
    p = port_lib.PortWorld(scenes.world_def(**wkw))
    for w in (g, p):
        scenes.build(w, "pile", count=600, seed=6, width=24.0, height=50.0, presolve=True)
        install_callbacks(w)
    for f in range(1, 241):
        assert g.step(1.0 / 60.0, 4) == 0
        p.step(1.0 / 60.0, 4)
        assert_bodies_equal(g, p, f)
        if f % 40 == 0:
            assert compare_contacts(g, p) == [], "frame %d" % f
    # removing the callbacks brings the CUDA graph back; results stay equal
    for w in (g, p):
        w.set_custom_filter(None)
        w.set_pre_solve(None)
    for f in range(241, 301):
        assert g.step(1.0 / 60.0, 4) == 0
        p.step(1.0 / 60.0, 4)
        assert_bodies_equal(g, p, f)
    assert g.sync() == 0
    g.close()
    p.close()


@pytest.mark.parametrize("sleep", [0, 1])
def test_gpu_sensor_events_match_port(gpu_lib, port_lib, sleep):
    """Sensor begin / end events of every frame, in order, against the
    oracle (native contact order)."""
    wkw = dict(enableSleep=sleep, enableContinuous=1)
    g = gpu_world(gpu_lib, wkw)
    p = port_lib.PortWorld(scenes.world_def(**wkw))
    scenes.build(g, "sensor_field", count=500)
    scenes.build(p, "sensor_field", count=500)
    totals = [0, 0]
    for f in range(1, 301):
        assert g.step(1.0 / 60.0, 4) == 0
        p.step(1.0 / 60.0, 4)
        assert_bodies_equal(g, p, f)
        for k, (a, b) in enumerate(zip(g.sensor_events(), p.sensor_events())):
            assert np.array_equal(a, b), (f, k, a[:4], b[:4])
            totals[k] += len(a)
    assert totals[0] > 100 and totals[1] > 50, totals
    assert g.sync() == 0
    g.close()
    p.close()


def test_gpu_events_match_port(gpu_lib, port_lib):
    wkw = dict(enableSleep=0, enableContinuous=1)
    kw = dict(count=300, seed=21, width=16.0, height=24.0, enable_hit_events=True, enable_contact_events=True)
    g = gpu_world(gpu_lib, wkw)
    p = port_lib.PortWorld(scenes.world_def(**wkw))
    scenes.build(g, "pile", **kw)
    scenes.build(p, "pile", **kw)
    totals = np.zeros(4, np.int64)
    for f in range(1, 121):
        g.step(1.0 / 60.0, 4)
        p.step(1.0 / 60.0, 4)
        assert np.array_equal(g.event_counts(), p.event_counts()), f
        for a, b in ((g.begin_events(), p.begin_events()), (g.end_events(), p.end_events())):
            assert sorted(map(tuple, a.tolist())) == sorted(map(tuple, b.tolist())), f
        # begin events in contact-id order with their manifolds, bit for bit
        assert np.array_equal(g.begin_events(), p.begin_events()), f
        assert np.array_equal(g.begin_manifolds().view(np.uint32), p.begin_manifolds().view(np.uint32)), f
        gi, gf = g.hit_events()
        pi, pf = p.hit_events()
        assert sorted(tuple(i) + tuple(x) for i, x in zip(gi.tolist(), gf.view(np.uint32).tolist())) == \
            sorted(tuple(i) + tuple(x) for i, x in zip(pi.tolist(), pf.view(np.uint32).tolist())), f
        gi, gf = g.move_events()
        pi, pf = p.move_events()
        grow = sorted((int(i[0]) - 1,) + tuple(x) for i, x in zip(gi.tolist(), gf.view(np.uint32).tolist()))
        prow = sorted((int(i[0]),) + tuple(x) for i, x in zip(pi.tolist(), pf.view(np.uint32).tolist()))
        assert grow == prow, f
        totals += p.event_counts()
    assert (totals > 0).all(), totals
    g.close()
    p.close()


@pytest.mark.parametrize("plan", [False, True], ids=["native", "parity_mode"])
@pytest.mark.parametrize("name", sorted(CASES))
def test_gpu_replays_reference_fixture_bit_exact(gpu_lib, name, plan):
    """Against the reference itself (committed fixtures): bodies, solver
    sets, colour counts and the first checkpoint's contacts (ids, shapes,
    colours, manifolds) bit for bit, natively and in parity mode."""
    wkw, scene, kw = CASES[name]
    g = gpu_world(gpu_lib, wkw)
    scenes.build(g, scene, **kw)
    gold = np.load(os.path.join(GOLD, name + "_ref.npz"))
    checks = set(int(c) for c in gold["checkpoints"])
    first = int(gold["checkpoints"][0])
    seen = []
    rows = ([], [])

    def on_frame(f):
        if name in SENSOR_CASES:
            sensor_rows(g, f, rows)
        if f not in checks:
            return
        full = g.bodies()
        b = full[:, :9]
        ref = gold["bodies_%d" % f]
        bad = np.argwhere(b.view(np.uint32) != ref.view(np.uint32))
        assert len(bad) == 0, "frame %d: first differing (body, field) %s" % (f, bad[0].tolist())
        check_sets(full, gold, f)
        assert np.array_equal(g.color_counts(), gold["colors_%d" % f]), f
        if f == first:
            ints, fl = g.contacts()
            ri, rf = gold["contact_ints_%d" % f], gold["contact_floats_%d" % f]
            assert np.array_equal(ints[:, [0, 1, 2, 3, 4, 7, 8]], ri[:, [0, 1, 2, 3, 4, 7, 8]])
            assert np.array_equal(fl.view(np.uint32), rf.view(np.uint32))
        seen.append(f)

    replay(g, name, on_frame=on_frame, plan=plan)
    assert sorted(seen) == sorted(checks)
    if name in SENSOR_CASES:
        check_sensor_rows(rows, gold)
    g.close()


@pytest.mark.parametrize("name", STATS_CASES)
def test_gpu_stats_series_parity_mode(gpu_lib, name):
    """256-frame max-penetration and KE series in parity mode: identical to
    the reference's (tolerance 0; the benchmark spec's bound is 1%)."""
    ref = np.load(os.path.join(GOLD, name + "_stats_ref.npy"))
    wkw, scene, kw = CASES[name]
    g = gpu_world(gpu_lib, wkw)
    scenes.build(g, scene, **kw)
    mass = g.mass()
    rows = []
    replay(g, name, frames=len(ref), on_frame=lambda f: rows.append(frame_stats(g, mass)))
    got = np.array(rows)
    assert np.array_equal(got, ref)
    g.close()


@pytest.mark.parametrize("name", STATS_CASES)
def test_gpu_stats_series_native_mode(gpu_lib, name):
    """Native mode (no reference ids handed over): the 256-frame
    max-penetration and KE series equal the reference's and the port's bit
    for bit (tolerance 0; the benchmark spec's bound is 1%)."""
    ref = np.load(os.path.join(GOLD, name + "_stats_ref.npy"))
    wkw, scene, kw = CASES[name]
    import oracle.oracle as orc
    g = gpu_world(gpu_lib, wkw)
    p = orc.PortWorld(scenes.world_def(**wkw))
    scenes.build(g, scene, **kw)
    scenes.build(p, scene, **kw)
    mass = g.mass()
    gs, ps = [], []
    for _ in range(len(ref)):
        g.step(1.0 / 60.0, 4)
        p.step(1.0 / 60.0, 4)
        gs.append(frame_stats(g, mass))
        ps.append(frame_stats(p, mass))
    gs, ps = np.array(gs), np.array(ps)
    assert np.array_equal(gs, ps)
    assert np.array_equal(gs, ref)
    g.close()
    p.close()


@pytest.mark.parametrize("scene,kw", [("pile", dict(count=3000, seed=9, width=40.0, height=120.0)),
                                      ("batched", dict(worlds=48, seed=5))], ids=["pile3000", "batched48"])
def test_autotune_changes_timing_only(gpu_lib, scene, kw):
    """The autotuner's candidates (solver launch shape, leaf-order period)
    leave every result unchanged: a tuned world equals an untuned twin
    stepped the same number of times, bit for bit."""
    wkw = dict(enableSleep=0, enableContinuous=1)
    a = gpu_world(gpu_lib, wkw)
    b = gpu_world(gpu_lib, wkw)
    scenes.build(a, scene, **kw)
    scenes.build(b, scene, **kw)
    st, chosen, taken = a.autotune(1.0 / 60.0, 4, 2)
    assert st == 0 and taken > 0
    assert chosen[0] in (1, 2, 3) and chosen[1] in (4, 8, 16, 32)
    assert a.tuning() == chosen
    for _ in range(taken):
        assert b.step(1.0 / 60.0, 4) == 0
    for _ in range(20):
        a.step(1.0 / 60.0, 4)
        b.step(1.0 / 60.0, 4)
    assert a.sync() == 0 and b.sync() == 0
    ab, bb = a.bodies()[:, :9], b.bodies()[:, :9]
    assert np.array_equal(ab.view(np.uint32), bb.view(np.uint32))
    a.close()
    b.close()
