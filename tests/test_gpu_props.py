"""The generic property calls on the GPU against the oracle (GPU only).

The same property script as the oracle's pin against the reference (joint
setters of every type, body damping / gravity scale / bullet / fixed
rotation / mass data, shape friction / restitution / density / event flags /
filters, chain friction) on the CUDA world and on the CPU restatement:
bodies bit for bit every frame, contacts, colours, every getter and shape
point tests every ten frames, with and without sleeping.
"""
from __future__ import annotations

import numpy as np
import pytest

from forge2d_gb300 import scenes

from parity import build_property_scene, compare_contacts, property_reads, property_script, point_answers

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("sleep", [0, 1])
def test_gpu_properties_match_port(gpu_lib, port_lib, sleep):
    from forge2d_gb300.world import GpuWorld
    wkw = dict(enableSleep=sleep, enableContinuous=1)
    gpu = GpuWorld(scenes.world_def(**wkw))
    port = port_lib.PortWorld(scenes.world_def(**wkw))
    nb, nj = build_property_scene(gpu)
    assert build_property_scene(port) == (nb, nj)
    ns = len(port.shapes()[1])
    cols = 12 if sleep else 9
    for f in range(1, 101):
        property_script(gpu, f, nb, nj)
        property_script(port, f, nb, nj)
        assert gpu.step(1.0 / 60.0, 4) == 0, f
        port.step(1.0 / 60.0, 4)
        gb, pb = gpu.bodies()[:, :cols], port.bodies()[:, :cols]
        bad = np.argwhere(gb.view(np.uint32) != pb.view(np.uint32))
        assert len(bad) == 0, "frame %d: body/field %s gpu %r port %r" % (f, bad[0].tolist(), gb[tuple(bad[0])],
                                                                           pb[tuple(bad[0])])
        assert np.array_equal(gpu.end_events(), port.end_events()), f
        if f % 10 == 0:
            assert compare_contacts(gpu, port) == [], f
            assert np.array_equal(gpu.color_counts(), port.color_counts()), f
            a = np.array(property_reads(gpu, nb, ns, nj), np.float64)
            b = np.array(property_reads(port, nb, ns, nj), np.float64)
            bad = np.flatnonzero(a.view(np.uint64) != b.view(np.uint64))
            assert len(bad) == 0, (f, bad[:5], a[bad[:5]], b[bad[:5]])
            assert point_answers(gpu) == point_answers(port), f
    gpu.close()
    port.close()


def test_gpu_body_lists_names_points(gpu_lib):
    """bodyGetShapes / bodyGetJoints in list order (newest first), names,
    world and local points, shape geometry and owner, joint bodies."""
    import ctypes as C
    from forge2d_gb300.world import GpuWorld
    g = GpuWorld(scenes.world_def(enableSleep=0))
    lib = g.lib
    ground = g.create_body(scenes.body_def(type=0))
    b = g.create_body(scenes.body_def(type=2, positionX=1.0, positionY=2.0, rotationCos=0.0, rotationSin=1.0))
    s1 = g.create_circle(b, scenes.shape_def(), 0.5, 0.0, 0.25)
    s2 = g.create_box(b, scenes.shape_def(), 0.5, 0.3)
    j1 = g.create_revolute(scenes.revolute_def(bodyA=ground, bodyB=b))
    j2 = g.create_revolute(scenes.revolute_def(bodyA=b, bodyB=ground))
    out = np.zeros(8, np.int32)
    ip = out.ctypes.data_as(C.POINTER(C.c_int32))
    assert lib.f2d_body_get_shapes(b[0], b[1], ip, 4) == 2
    assert [tuple(out[0:2]), tuple(out[2:4])] == [s2, s1]
    assert lib.f2d_body_get_joints(b[0], b[1], ip, 4) == 2
    assert [tuple(out[0:2]), tuple(out[2:4])] == [j2, j1]
    lib.f2d_body_set_name(b[0], b[1], b"crate-with-a-rather-long-name-0123456789")
    buf = C.create_string_buffer(64)
    assert lib.f2d_body_get_name(b[0], b[1], buf, 64) == 31
    assert buf.value == b"crate-with-a-rather-long-name-0"
    x, y = C.c_double(), C.c_double()
    lib.f2d_body_get_world_point(b[0], b[1], 1.0, 0.0, C.byref(x), C.byref(y))
    assert (x.value, y.value) == (1.0, 3.0)
    lib.f2d_body_get_local_point(b[0], b[1], 1.0, 3.0, C.byref(x), C.byref(y))
    assert (x.value, y.value) == (1.0, 0.0)
    geo = np.zeros(17, np.float64)
    gp = geo.ctypes.data_as(C.POINTER(C.c_double))
    assert lib.f2d_shape_get_geometry(s1[0], s1[1], 0, gp, 17) == 3  # circle
    assert tuple(geo[:3]) == (0.5, 0.0, 0.25)
    assert lib.f2d_shape_get_geometry(s2[0], s2[1], 0, gp, 17) == 0  # not a circle
    bi, bw = C.c_int32(), C.c_int32()
    assert lib.f2d_shape_get_body(s2[0], s2[1], C.byref(bi), C.byref(bw)) and (bi.value, bw.value) == b
    assert lib.f2d_joint_get_body(j1[0], j1[1], 1, C.byref(bi), C.byref(bw)) and (bi.value, bw.value) == b
    assert g.step() == 0
    aabb = np.zeros(4, np.float64)
    lib.f2d_shape_get_aabb(s1[0], s1[1], aabb.ctypes.data_as(C.POINTER(C.c_double)))
    assert aabb[0] < aabb[2] and aabb[1] < aabb[3]
    g.close()
