"""The destroy path on the GPU against the oracle (GPU only).

The same destroy script as the oracle's pin against the reference
(b2DestroyBody, b2DestroyShape, b2DestroyJoint, b2DestroyChain between
steps; freed ids reused by new bodies and proxies; a joint created between
touching bodies ending their contacts), run on the CUDA world and on the CPU
restatement: every body row bit for bit on every frame, end events (the
destroyed contacts' ones first) on every frame, contacts and colours every
ten frames, with and without sleeping.
"""
from __future__ import annotations

import numpy as np
import pytest

from forge2d_gb300 import scenes

from parity import compare_contacts, destroy_script, touching_pair
from test_oracle_pin import build_destroy_scene

pytestmark = pytest.mark.gpu


def _bodies_equal(g, p, f, cols):
    gb, pb = g.bodies()[:, :cols], p.bodies()[:, :cols]
    assert gb.shape == pb.shape, f
    bad = np.argwhere(gb.view(np.uint32) != pb.view(np.uint32))
    assert len(bad) == 0, "frame %d: body/field %s gpu %r port %r" % (f, bad[0].tolist(), gb[tuple(bad[0])],
                                                                       pb[tuple(bad[0])])


@pytest.mark.parametrize("sleep", [0, 1])
def test_gpu_destroy_path_matches_port(gpu_lib, port_lib, sleep):
    from forge2d_gb300.world import GpuWorld
    wkw = dict(enableSleep=sleep, enableContinuous=1)
    gpu = GpuWorld(scenes.world_def(**wkw))
    port = port_lib.PortWorld(scenes.world_def(**wkw))
    gids = build_destroy_scene(gpu)
    pids = build_destroy_scene(port)
    assert gids["box"] == pids["box"] and gids["last"] == pids["last"]
    ends = 0
    for f in range(1, 141):
        if f == 90:
            gids["touch"] = touching_pair(gpu)
            pids["touch"] = touching_pair(port)
            assert gids["touch"] == pids["touch"] and pids["touch"] is not None
        destroy_script(gpu, f, gids)
        destroy_script(port, f, pids)
        assert gpu.step(1.0 / 60.0, 4) == 0, f
        port.step(1.0 / 60.0, 4)
        _bodies_equal(gpu, port, f, 12 if sleep else 9)
        assert np.array_equal(gpu.end_events(), port.end_events()), f
        assert np.array_equal(gpu.begin_events(), port.begin_events()), f
        ends += len(port.end_events())
        if f % 10 == 0:
            assert compare_contacts(gpu, port) == [], f
            assert np.array_equal(gpu.color_counts(), port.color_counts()), f
            assert gpu.counters()["awake_bodies"] == port.awake_body_count(), f
    assert ends > 0
    gpu.close()
    port.close()


def test_gpu_destroyed_ids_are_invalid_and_reused(gpu_lib):
    """Destroyed handles stop being valid; the freed ids come back last in,
    first out with a new generation."""
    from forge2d_gb300.world import GpuWorld
    g = GpuWorld(scenes.world_def(enableSleep=0))
    lib = g.lib
    bodies = [g.create_body(scenes.body_def(type=2, positionX=float(k))) for k in range(4)]
    shapes = [g.create_circle(b, scenes.shape_def(), 0.0, 0.0, 0.4) for b in bodies]
    j = g.create_revolute(scenes.revolute_def(bodyA=bodies[0], bodyB=bodies[1]))
    g.step()
    g.destroy_body(bodies[2])
    g.destroy_body(bodies[1])  # takes the joint with it
    assert not lib.f2d_body_is_valid(*bodies[1]) and not lib.f2d_body_is_valid(*bodies[2])
    assert not lib.f2d_shape_is_valid(*shapes[1]) and not lib.f2d_joint_is_valid(*j)
    assert lib.f2d_body_is_valid(*bodies[0]) and lib.f2d_shape_is_valid(*shapes[0])
    nb = g.create_body(scenes.body_def(type=2))
    assert nb[0] == bodies[1][0] and nb[1] != bodies[1][1]  # last freed, new generation
    ns = g.create_circle(nb, scenes.shape_def(), 0.0, 0.0, 0.4)
    assert ns[0] == shapes[1][0]
    nj = g.create_revolute(scenes.revolute_def(bodyA=bodies[0], bodyB=nb))
    assert nj[0] == j[0] and nj[1] != j[1]
    assert g.step() == 0
    c = g.counters()
    assert c["shapes"] == 3 and c["joints"] == 1
    g.close()
