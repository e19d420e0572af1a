"""Body type changes, disable and enable on the GPU against the oracle (GPU
only).

The type script of parity.py (b2Body_SetType between all three types with
and without joints, b2Body_Disable / b2Body_Enable of bodies with joints, a
type change while disabled) on the scene of the destroy path, run on the CUDA
world and on the CPU restatement: every body row bit for bit every frame,
begin and end events every frame, contacts and colours every five frames,
with and without sleeping.
"""
from __future__ import annotations

import numpy as np
import pytest

from forge2d_gb300 import native, scenes

from parity import compare_contacts, type_script
from test_oracle_pin import build_destroy_scene

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("sleep", [0, 1])
def test_gpu_type_changes_match_port(gpu_lib, port_lib, sleep):
    from forge2d_gb300.world import GpuWorld
    wkw = dict(enableSleep=sleep, enableContinuous=1)
    gpu = GpuWorld(scenes.world_def(**wkw))
    port = port_lib.PortWorld(scenes.world_def(**wkw))
    gids, pids = build_destroy_scene(gpu), build_destroy_scene(port)
    assert gids["box"] == pids["box"] and gids["last"] == pids["last"]
    cols = 12 if sleep else 9
    for f in range(1, 141):
        type_script(gpu, f)
        type_script(port, f)
        assert gpu.step(1.0 / 60.0, 4) == 0, f
        port.step(1.0 / 60.0, 4)
        gb, pb = gpu.bodies()[:, :cols], port.bodies()[:, :cols]
        bad = np.argwhere(gb.view(np.uint32) != pb.view(np.uint32))
        assert len(bad) == 0, "frame %d: body/field %s gpu %r port %r" % (f, bad[0].tolist(), gb[tuple(bad[0])],
                                                                           pb[tuple(bad[0])])
        assert np.array_equal(gpu.end_events(), port.end_events()), f
        assert np.array_equal(gpu.begin_events(), port.begin_events()), f
        if f % 5 == 0:
            assert compare_contacts(gpu, port) == [], f
            assert np.array_equal(gpu.color_counts(), port.color_counts()), f
            if sleep:
                assert gpu.counters()["awake_bodies"] == port.awake_body_count(), f
    gpu.close()
    port.close()


def test_gpu_type_and_enabled_getters(gpu_lib):
    """bodyGetType / bodyIsEnabled follow the calls; a disabled body neither
    moves nor collides, and moves again once enabled."""
    from forge2d_gb300.world import GpuWorld
    g = GpuWorld(scenes.world_def(enableSleep=0))
    lib = g.lib
    ground = g.create_body(scenes.body_def(type=0))
    g.create_box(ground, scenes.shape_def(), 10.0, 0.5)
    b = g.create_body(scenes.body_def(type=2, positionY=3.0))
    g.create_circle(b, scenes.shape_def(), 0.0, 0.0, 0.5)
    enabled = native.CODES["F2D_BODY_ENABLED"]
    assert lib.f2d_body_get_type(*b) == 2
    g.body_set_type(b, 1)
    assert lib.f2d_body_get_type(*b) == 1
    g.body_set_type(b, 2)
    g.body_disable(b)
    assert lib.f2d_body_get_param(b[0], b[1], enabled) == 0.0
    y0 = g.bodies()[1, 1]
    for _ in range(30):
        assert g.step() == 0
    assert g.bodies()[1, 1] == y0
    g.body_enable(b)
    assert lib.f2d_body_get_param(b[0], b[1], enabled) == 1.0
    for _ in range(120):
        assert g.step() == 0
    y = g.bodies()[1, 1]
    assert 0.9 < y < 1.1  # resting on the ground box
    g.close()
