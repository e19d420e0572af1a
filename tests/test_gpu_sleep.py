"""Islands and sleep on the GPU (worlds created with sleeping on), bit for
bit against the oracle: bodies fall asleep on the same frame with the same
solver-set ids and sleep times, contacts and colours agree, sleeping sets
wake through contacts and through the body API, and the move events carry
the same fellAsleep flags in the same order."""
from __future__ import annotations

import numpy as np
import pytest

from forge2d_gb300 import scenes

from parity import compare_contacts

pytestmark = pytest.mark.gpu


def gpu_world(wkw, solver="auto"):
    import os
    from forge2d_gb300.world import GpuWorld
    if solver == "grid":
        os.environ["F2D_NO_CLUSTER_SOLVER"] = "1"
    try:
        return GpuWorld(scenes.world_def(**wkw))
    finally:
        os.environ.pop("F2D_NO_CLUSTER_SOLVER", None)


def step_both(g, p, f):
    assert g.step(1.0 / 60.0, 4) == 0
    p.step(1.0 / 60.0, 4)
    gb, pb = g.bodies(), p.bodies()
    bad = np.argwhere(gb.view(np.uint32) != pb.view(np.uint32))
    assert len(bad) == 0, "frame %d: body/field %s gpu %r port %r" % (
        f, bad[0].tolist(), gb[tuple(bad[0])], pb[tuple(bad[0])])
    assert g.awake_body_count() == p.awake_body_count(), f


def compare_state(g, p, f):
    assert compare_contacts(g, p) == [], "frame %d" % f
    gc, pc = g.color_counts(), p.color_counts()
    assert np.array_equal(gc, pc), "frame %d colours gpu %s port %s" % (f, gc, pc)
    gi, gf = g.move_events()
    pi, pf = p.move_events()
    # same bodies in the same (awake-set) order, same fellAsleep flags and transforms
    assert (gi[:, 0] - 1).tolist() == pi[:, 0].tolist(), "frame %d move-event bodies" % f
    assert gi[:, 2].tolist() == pi[:, 1].tolist(), "frame %d fellAsleep flags" % f
    assert np.array_equal(gf.view(np.uint32), pf.view(np.uint32)), "frame %d move-event transforms" % f


SCENES = [
    ("pyramid_sleep", dict(enableSleep=1), "pyramid", dict(rows=12), 300),
    ("pile_sleep", dict(enableSleep=1, enableContinuous=1), "pile",
     dict(count=300, seed=3, width=20.0, height=30.0), 450),
    ("chains_sleep", dict(enableSleep=1), "pyramids_chains", dict(pyramids=2, rows=6, chains=4, links=10), 400),
    # weld and distance joints link islands and sleep with them
    ("joint_zoo_sleep", dict(enableSleep=1), "joint_zoo", dict(copies=3), 400),
    ("joint_rigs_sleep", dict(enableSleep=1), "joint_rigs", dict(copies=3), 400),
    ("chain_terrain_sleep", dict(enableSleep=1, enableContinuous=1), "chain_terrain", dict(count=200), 500),
]


@pytest.mark.parametrize("sleep", [0, 1])
def test_gpu_mouse_target_moves(gpu_lib, port_lib, sleep):
    """MouseJoint.setTarget between steps (uploaded with the next step; no
    wake): the held boxes follow the new targets as in the oracle."""
    wkw = dict(enableSleep=sleep)
    g = gpu_world(wkw)
    p = port_lib.PortWorld(scenes.world_def(**wkw))
    mg = scenes.build(g, "joint_rigs", copies=3)
    mp = scenes.build(p, "joint_rigs", copies=3)
    f = 0
    for t, (dx, dy) in enumerate([(0.0, 0.0), (-1.5, 4.0), (2.0, 1.5), (0.5, 6.0)]):
        if t:
            for k in range(3):
                x = -90.0 + 5.0 + 30.0 * k + 20.0 + dx
                g.mouse_set_target(mg[k], x, dy)
                p.mouse_set_target(mp[k], x, dy)
        for _ in range(80):
            f += 1
            step_both(g, p, f)
        compare_state(g, p, f)
    assert g.sync() == 0
    g.close()
    p.close()


@pytest.mark.parametrize("solver", ["auto", "grid"])
@pytest.mark.parametrize("name,wkw,scene,kw,frames", SCENES, ids=[s[0] for s in SCENES])
def test_gpu_sleep_matches_port(gpu_lib, port_lib, name, wkw, scene, kw, frames, solver):
    g = gpu_world(wkw, solver)
    p = port_lib.PortWorld(scenes.world_def(**wkw))
    scenes.build(g, scene, **kw)
    scenes.build(p, scene, **kw)
    fewest = None
    for f in range(1, frames + 1):
        step_both(g, p, f)
        n = g.awake_body_count()
        fewest = n if fewest is None else min(fewest, n)
        if f % 25 == 0 or f == frames:
            compare_state(g, p, f)
    if name == "pyramid_sleep":
        assert g.awake_body_count() == 0
    else:
        assert fewest < g.counters()["shapes"] - 1, "no island fell asleep"
    assert g.sync() == 0
    g.close()
    p.close()


def test_gpu_wake_by_contact_and_api(gpu_lib, port_lib):
    wkw = dict(enableSleep=1)
    g = gpu_world(wkw)
    p = port_lib.PortWorld(scenes.world_def(**wkw))
    for w in (g, p):
        scenes.build(w, "pyramid", rows=10)
        scenes.build(w, "pyramids_chains", pyramids=1, rows=4, chains=3, links=6, gap=30.0)
    f = 0
    for _ in range(150):
        f += 1
        step_both(g, p, f)
    assert g.awake_body_count() < 30
    for w in (g, p):
        b = w.create_body(scenes.body_def(type=scenes.DYNAMIC, positionX=0.3, positionY=14.0))
        w.create_circle(b, scenes.shape_def(), 0.0, 0.0, 0.5)
        b2 = w.create_body(scenes.body_def(type=scenes.DYNAMIC, positionX=-3.2, positionY=16.0))
        w.create_box(b2, scenes.shape_def(), 0.4, 0.4)
    woke = False
    for _ in range(120):
        f += 1
        step_both(g, p, f)
        woke |= g.awake_body_count() > 50
        if f % 20 == 0:
            compare_state(g, p, f)
    assert woke, "the falling bodies were meant to wake the pyramid"
    for w in (g, p):
        w.set_awake(5, False)
        w.set_awake(30, True)
    for _ in range(40):
        f += 1
        step_both(g, p, f)
    compare_state(g, p, f)
    for w in (g, p):
        w.enable_sleeping(False)
    assert g.awake_body_count() == p.awake_body_count()
    for _ in range(40):
        f += 1
        step_both(g, p, f)
    compare_state(g, p, f)
    g.close()
    p.close()
