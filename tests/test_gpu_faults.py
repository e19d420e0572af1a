"""Host-side faults (GPU only: a world needs a device): stale and invalid
ids, definitions the reference's creation asserts stop on, calls on a
destroyed world. Every one is refused on the host with a return value or a
status bit; none reaches a kernel, so nothing here can fault the GPU.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np
import pytest

from forge2d_gb300 import native, scenes

pytestmark = pytest.mark.gpu


def _world(**kw):
    from forge2d_gb300.world import GpuWorld
    return GpuWorld(scenes.world_def(**kw))


def test_invalid_and_stale_ids_are_refused(gpu_lib):
    g = _world(enableSleep=1)
    lib = g.lib
    b = g.create_body(scenes.body_def(type=2, positionY=2.0))
    s = g.create_circle(b, scenes.shape_def(), 0.0, 0.0, 0.5)
    ground = g.create_body(scenes.body_def(type=0))
    g.create_box(ground, scenes.shape_def(), 5.0, 0.5)
    j = g.create_revolute(scenes.revolute_def(bodyA=ground, bodyB=b))
    assert g.step() == 0
    bad = [(0, b[1]), (-3, b[1]), (1 << 20, b[1]), (b[0], b[1] + (1 << 16)), (b[0], 0x7fff)]
    x, y = C.c_double(7.0), C.c_double(7.0)
    for i1, wg in bad:
        assert not lib.f2d_body_is_valid(i1, wg)
        lib.f2d_body_get_position(i1, wg, C.byref(x), C.byref(y))
        lib.f2d_body_set_linear_velocity(i1, wg, 1.0, 1.0)
        lib.f2d_destroy_body(i1, wg)
        assert not lib.f2d_shape_is_valid(i1, wg)
        lib.f2d_destroy_shape(i1, wg, 1)
        assert not lib.f2d_joint_is_valid(i1, wg)
        lib.f2d_destroy_joint(i1, wg)
        lib.f2d_destroy_chain(i1, wg)
    assert lib.f2d_body_is_valid(*b) and lib.f2d_shape_is_valid(*s) and lib.f2d_joint_is_valid(*j)
    # a destroyed handle stays invalid; destroying it again does nothing
    g.destroy_joint(j)
    assert not lib.f2d_joint_is_valid(*j)
    g.destroy_joint(j)
    g.destroy_body(b)
    assert not lib.f2d_body_is_valid(*b) and not lib.f2d_shape_is_valid(*s)
    g.destroy_body(b)
    g.destroy_shape(s)
    assert g.step() == 0 and g.sync() == 0
    c = g.counters()
    assert c["shapes"] == 1 and c["joints"] == 0
    # a body of another world is not a body of this one
    h = _world()
    hb = h.create_body(scenes.body_def(type=2))
    jd = scenes.revolute_def(bodyA=ground, bodyB=hb)
    assert g.create_revolute(jd) == -1
    h.close()
    g.close()


def test_invalid_definitions_are_refused(gpu_lib):
    g = _world()
    nan, inf = math.nan, math.inf
    for field, value in (("positionX", nan), ("positionY", inf), ("rotationCos", nan), ("rotationCos", 0.5),
                         ("linearVelocityX", nan), ("angularVelocity", inf), ("linearDamping", -1.0),
                         ("angularDamping", nan), ("sleepThreshold", -0.1), ("gravityScale", nan), ("type", 7)):
        d = dict(type=2)
        d[field] = value
        with pytest.raises(RuntimeError):
            g.create_body(scenes.body_def(**d))
    b = g.create_body(scenes.body_def(type=2))
    for field, value in (("density", -1.0), ("density", nan), ("friction", -0.5), ("restitution", inf),
                         ("rollingResistance", -1.0), ("tangentSpeed", nan)):
        assert g.create_circle(b, scenes.shape_def(**{field: value}), 0.0, 0.0, 0.5) == -1
    assert g.create_box(b, scenes.shape_def(), 0.5, 0.5, radius=-0.1) == -1
    assert g.create_polygon(b, scenes.shape_def(), [(0, 0), (1, 0), (0, 1)], radius=nan) == -1
    ground = g.create_body(scenes.body_def(type=0))
    bad_mat = ((0.6, -1.0, 0.0, 0.0, 0, 0),)
    assert g.create_chain(ground, [(0, 0), (1, 0), (2, 0), (3, 0)], materials=bad_mat) == -1
    assert g.counters()["shapes"] == 0
    assert g.step() == 0
    g.close()


def test_calls_on_a_destroyed_world(gpu_lib):
    g = _world()
    wid = g.id
    g.create_body(scenes.body_def(type=2))
    g.close()
    lib = native.lib()
    assert not lib.f2d_world_is_valid(wid)
    assert lib.f2d_world_step(wid, 1.0 / 60.0, 4) == 0x100  # F2D_STATUS_INVALID
    out = np.zeros(8, np.int32)
    lib.f2d_world_get_counters(wid, out.ctypes.data_as(C.POINTER(C.c_int32)))
    assert not out.any()
