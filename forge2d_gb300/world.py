"""Host-side mirror of forge2d's world API over the GPU C ABI.

``World`` / ``Body`` / ``Shape`` / ``Joint`` follow the names and argument
meaning of forge2d's public Dart API (packages/forge2d/lib/src/api/world.dart,
body.dart; the defs of defs.dart) and of the RawBox2D seam it sits on
(packages/forge2d/lib/src/backend/raw_box2d.dart). Ids are the seam's packed
pairs (index1, worldAndGeneration).

``GpuWorld`` is the flat builder the seeded scenes in ``scenes.py`` and the
parity tests drive; the oracle worlds expose the same methods.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import native
from .scenes import (BODY_DEFAULTS, JOINT_DEFAULTS, JOINT_DISTANCE, JOINT_FILTER, JOINT_MOTOR, JOINT_MOUSE,
                     JOINT_PRISMATIC, JOINT_WELD, JOINT_WHEEL, REVOLUTE_DEFAULTS, SHAPE_DEFAULTS, WORLD_DEFAULTS)

BODY_STRIDE = 12
CONTACT_INTS = 9
CONTACT_FLOATS = 25


def _fill(struct, values: dict):
    for k, v in values.items():
        if hasattr(struct, k):
            setattr(struct, k, v)
    return struct


def _fptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def _iptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


class GpuWorld:
    """Flat builder over the C ABI (one GPU world)."""

    def __init__(self, world_def: dict | None = None, workers: int = 1):
        self.lib = native.lib()
        wd = dict(WORLD_DEFAULTS)
        if world_def:
            wd.update(world_def)
        # current generation per index of each id kind (ids are reused)
        self._wg = {"body": {}, "shape": {}, "joint": {}, "chain": {}}
        self.id = self.lib.f2d_create_world(C.byref(_fill(native.WorldDef(), wd)))
        if self.id == 0:
            raise RuntimeError("f2d_create_world failed (no CUDA device?)")
        self._closed = False

    def close(self):
        if not self._closed:
            self.lib.f2d_destroy_world(self.id)
            self._closed = True

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def reserve(self, bodies=0, shapes=0, contacts=0, joints=0):
        self.lib.f2d_world_reserve(self.id, bodies, shapes, contacts, joints)

    # creation ---------------------------------------------------------
    def create_body(self, body_def: dict):
        bd = dict(BODY_DEFAULTS)
        bd.update(body_def)
        i1, wg = C.c_int32(0), C.c_int32(0)
        if not self.lib.f2d_create_body(self.id, C.byref(_fill(native.BodyDef(), bd)), C.byref(i1), C.byref(wg)):
            raise RuntimeError("createBody failed")
        self._wg["body"][i1.value - 1] = wg.value
        return (i1.value, wg.value)

    def _id(self, kind, x):
        """(index1, worldAndGeneration) of a handle or of a 0-based index."""
        if isinstance(x, (int, np.integer)):
            return (int(x) + 1, self._wg[kind][int(x)])
        return x

    def _body(self, body):
        return self._id("body", body)

    # destroy path ------------------------------------------------------
    def destroy_body(self, body):
        b = self._body(body)
        self.lib.f2d_destroy_body(b[0], b[1])

    def body_set_type(self, body, body_type):
        """b2Body_SetType; ``body`` is a creation handle or a body index."""
        b = self._body(body)
        self.lib.f2d_body_set_type(b[0], b[1], int(body_type))

    def body_disable(self, body):
        b = self._body(body)
        self.lib.f2d_body_disable(b[0], b[1])

    def body_enable(self, body):
        b = self._body(body)
        self.lib.f2d_body_enable(b[0], b[1])

    def destroy_shape(self, shape, update_mass=True):
        s = self._id("shape", shape)
        self.lib.f2d_destroy_shape(s[0], s[1], int(update_mass))

    def destroy_joint(self, joint):
        j = self._id("joint", joint)
        self.lib.f2d_destroy_joint(j[0], j[1])

    def destroy_chain(self, chain):
        c = self._id("chain", chain)
        self.lib.f2d_destroy_chain(c[0], c[1])

    # properties (generic get/set codes, native.CODES) ----------------
    def body_get(self, body, code):
        b = self._body(body)
        return self.lib.f2d_body_get_param(b[0], b[1], native.CODES[code] if isinstance(code, str) else code)

    def body_set(self, body, code, value):
        b = self._body(body)
        self.lib.f2d_body_set_param(b[0], b[1], native.CODES[code] if isinstance(code, str) else code, value)

    def body_set_mass_data(self, body, mass, inertia, cx, cy):
        b = self._body(body)
        self.lib.f2d_body_set_mass_data(b[0], b[1], mass, inertia, cx, cy)

    def body_apply_mass_from_shapes(self, body):
        b = self._body(body)
        self.lib.f2d_body_apply_mass_from_shapes(b[0], b[1])

    def shape_get(self, shape, code):
        s = self._id("shape", shape)
        return self.lib.f2d_shape_get_param(s[0], s[1], native.CODES[code] if isinstance(code, str) else code)

    def shape_set(self, shape, code, value, flag=0):
        s = self._id("shape", shape)
        self.lib.f2d_shape_set_param(s[0], s[1], native.CODES[code] if isinstance(code, str) else code, value,
                                     int(flag))

    def shape_set_filter(self, shape, category, mask, group):
        s = self._id("shape", shape)
        self.lib.f2d_shape_set_filter(s[0], s[1], category, mask, group)

    def shape_test_point(self, shape, x, y):
        s = self._id("shape", shape)
        return bool(self.lib.f2d_shape_test_point(s[0], s[1], x, y))

    def chain_set(self, chain, code, value):
        c = self._id("chain", chain)
        self.lib.f2d_chain_set_param(c[0], c[1], native.CODES[code] if isinstance(code, str) else code, value)

    def joint_get(self, joint, code):
        j = self._id("joint", joint)
        return self.lib.f2d_joint_get_param(j[0], j[1], native.CODES[code] if isinstance(code, str) else code)

    def joint_set(self, joint, code, value, value2=0.0):
        j = self._id("joint", joint)
        self.lib.f2d_joint_set_param(j[0], j[1], native.CODES[code] if isinstance(code, str) else code, value,
                                     value2)

    def set_collide_connected(self, joint, flag):
        j = self._id("joint", joint)
        self.lib.f2d_joint_set_collide_connected(j[0], j[1], int(flag))

    # sleeping ---------------------------------------------------------
    def set_awake(self, body, awake):
        """b2Body_SetAwake; ``body`` is a creation handle or a body index."""
        b = self._body(body)
        self.lib.f2d_body_set_awake(b[0], b[1], int(awake))

    def is_awake(self, body):
        b = self._body(body)
        return bool(self.lib.f2d_body_is_awake(b[0], b[1]))

    def enable_sleeping(self, enabled):
        self.lib.f2d_world_enable_sleeping(self.id, int(enabled))

    def awake_body_count(self):
        return self.counters()["awake_bodies"]

    def _sd(self, sd):
        d = dict(SHAPE_DEFAULTS)
        d.update(sd)
        return C.byref(_fill(native.ShapeDef(), d))

    def _ret(self, ok, i1, wg, kind="shape"):
        if not ok:
            return -1
        self._wg[kind][i1.value - 1] = wg.value
        return (i1.value, wg.value)

    def create_circle(self, body, sd, cx, cy, r):
        i1, wg = C.c_int32(0), C.c_int32(0)
        ok = self.lib.f2d_create_circle_shape(body[0], body[1], self._sd(sd), cx, cy, r, C.byref(i1), C.byref(wg))
        return self._ret(ok, i1, wg)

    def create_capsule(self, body, sd, x1, y1, x2, y2, r):
        i1, wg = C.c_int32(0), C.c_int32(0)
        ok = self.lib.f2d_create_capsule_shape(body[0], body[1], self._sd(sd), x1, y1, x2, y2, r, C.byref(i1),
                                               C.byref(wg))
        return self._ret(ok, i1, wg)

    def create_segment(self, body, sd, x1, y1, x2, y2):
        i1, wg = C.c_int32(0), C.c_int32(0)
        ok = self.lib.f2d_create_segment_shape(body[0], body[1], self._sd(sd), x1, y1, x2, y2, C.byref(i1),
                                               C.byref(wg))
        return self._ret(ok, i1, wg)

    def create_box(self, body, sd, hx, hy, cx=0.0, cy=0.0, c=1.0, s=0.0, radius=0.0):
        i1, wg = C.c_int32(0), C.c_int32(0)
        ok = self.lib.f2d_create_box_shape(body[0], body[1], self._sd(sd), hx, hy, cx, cy, c, s, radius,
                                           C.byref(i1), C.byref(wg))
        return self._ret(ok, i1, wg)

    def create_polygon(self, body, sd, points, radius=0.0):
        pts = np.ascontiguousarray(np.asarray(points, dtype=np.float64).reshape(-1))
        i1, wg = C.c_int32(0), C.c_int32(0)
        ok = self.lib.f2d_create_polygon_shape(body[0], body[1], self._sd(sd),
                                               pts.ctypes.data_as(C.POINTER(C.c_double)), len(pts) // 2, radius,
                                               C.byref(i1), C.byref(wg))
        return self._ret(ok, i1, wg)

    def create_revolute(self, jd: dict):
        d = dict(REVOLUTE_DEFAULTS)
        d.update(jd)
        a, b = self._body(d.pop("bodyA")), self._body(d.pop("bodyB"))
        rd = _fill(native.RevoluteDef(), d)
        rd.bodyAIndex1, rd.bodyAWorldAndGeneration = a
        rd.bodyBIndex1, rd.bodyBWorldAndGeneration = b
        i1, wg = C.c_int32(0), C.c_int32(0)
        ok = self.lib.f2d_create_revolute_joint(self.id, C.byref(rd), C.byref(i1), C.byref(wg))
        return self._ret(ok, i1, wg, "joint")

    def create_chain(self, body, points, materials=((0.6, 0.0, 0.0, 0.0, 0, 0),), categoryBits=1, maskBits=-1,
                     groupIndex=0, isLoop=False, enableSensorEvents=False):
        """Chain of one-sided segments on ``body`` (b2CreateChain); returns the
        chain id pair."""
        pts = np.ascontiguousarray(np.asarray(points, np.float64).reshape(-1))
        mats = np.ascontiguousarray(np.asarray(materials, np.float64).reshape(-1))
        i1, wg = C.c_int32(0), C.c_int32(0)
        ok = self.lib.f2d_create_chain(body[0], body[1], pts.ctypes.data_as(C.POINTER(C.c_double)), len(pts) // 2,
                                       mats.ctypes.data_as(C.POINTER(C.c_double)), len(mats) // 6, categoryBits,
                                       maskBits, groupIndex, int(isLoop), int(enableSensorEvents),
                                       C.byref(i1), C.byref(wg))
        chain = self._ret(ok, i1, wg, "chain")
        if ok:
            for s in self.chain_segments(chain):
                self._wg["shape"][s[0] - 1] = s[1]
        return chain

    def cast_ray(self, ox, oy, tx, ty, fn, cat=1, mask=-1):
        """b2World_CastRay: fn(shape, point(2), normal(2), fraction) -> float,
        0-based shape ids, hits in ascending fraction."""
        cb = native.CastResultFn(lambda s, sw, px, py, nx, ny, f, ctx: float(fn(s - 1, (px, py), (nx, ny), f)))
        return self.lib.f2d_world_cast_ray(self.id, ox, oy, tx, ty, cat, mask, cb, None)

    def explode(self, x, y, radius, falloff, impulse_per_length, mask=-1):
        """b2World_Explode: radial impulse on the dynamic shapes near (x, y)."""
        self.lib.f2d_world_explode(self.id, mask, x, y, radius, falloff, impulse_per_length)

    def set_custom_filter(self, fn):
        """fn(shapeA, shapeB) -> bool with 0-based shape ids (A has the smaller
        proxy key; for continuous collision A is the static shape); None
        removes the filter."""
        if fn is None:
            self._filter_cb = native.CustomFilterFn()
        else:
            self._filter_cb = native.CustomFilterFn(lambda a, aw, b, bw, ctx: int(bool(fn(a - 1, b - 1))))
        self.lib.f2d_world_set_custom_filter(self.id, self._filter_cb, None)

    def set_pre_solve(self, fn):
        """fn(shapeA, shapeB, ManifoldView) -> bool with 0-based shape ids;
        None removes the callback."""
        if fn is None:
            self._presolve_cb = native.PreSolveFn()
        else:
            self._presolve_cb = native.PreSolveFn(
                lambda a, aw, b, bw, m, ctx: int(bool(fn(a - 1, b - 1, m.contents))))
        self.lib.f2d_world_set_pre_solve(self.id, self._presolve_cb, None)

    def sensor_events(self):
        """This step's sensor (begin, end) events as (sensor shape, visitor
        shape) rows of 0-based shape ids, in the order they were produced."""
        cap = 1 << 16
        b = np.zeros((cap, 4), np.int32)
        e = np.zeros((cap, 4), np.int32)
        ne = C.c_int32(0)
        nb = self.lib.f2d_world_get_sensor_events(self.id, _iptr(b), _iptr(e), cap, C.byref(ne))
        return b[:nb][:, [0, 2]] - 1, e[:ne.value][:, [0, 2]] - 1

    def chain_segments(self, chain):
        out = np.zeros(2 * (1 << 16), np.int32)
        n = self.lib.f2d_chain_get_segments(chain[0], chain[1], _iptr(out), len(out) // 2)
        return [tuple(r) for r in out[:2 * n].reshape(-1, 2).tolist()]

    def create_joint(self, jd: dict):
        """Weld (type 2) or distance (type 3) joint from an f2d_joint_def dict."""
        d = dict(JOINT_DEFAULTS)
        d.update(jd)
        a, b = self._body(d.pop("bodyA")), self._body(d.pop("bodyB"))
        rd = _fill(native.JointDef(), d)
        rd.bodyAIndex1, rd.bodyAWorldAndGeneration = a
        rd.bodyBIndex1, rd.bodyBWorldAndGeneration = b
        i1, wg = C.c_int32(0), C.c_int32(0)
        ok = self.lib.f2d_create_joint(self.id, C.byref(rd), C.byref(i1), C.byref(wg))
        return self._ret(ok, i1, wg, "joint")

    def joint_constraint(self, joint):
        """(force.x, force.y, torque) of the last step."""
        out = np.zeros(3, np.float32)
        self.lib.f2d_joint_get_constraint(joint[0], joint[1], out.ctypes.data_as(C.POINTER(C.c_float)))
        return out

    def set_limits(self, joint, enable, lower, upper):
        """Limit of a revolute, prismatic or wheel joint."""
        self.lib.f2d_joint_set_limits(joint[0], joint[1], int(enable), lower, upper)

    def set_motor(self, joint, enable, speed, max_motor):
        """Motor of a revolute, prismatic, wheel or distance joint."""
        self.lib.f2d_joint_set_motor(joint[0], joint[1], int(enable), speed, max_motor)

    def mouse_set_target(self, joint, x, y):
        self.lib.f2d_mouse_joint_set_target(joint[0], joint[1], x, y)

    def autotune(self, dt=1.0 / 60.0, substeps=4, steps_per_candidate=3):
        """Steps through the launch configurations and keeps the fastest;
        returns (status, (solver variant, leaf-order period), steps taken)."""
        out = np.zeros(3, np.int32)
        st = self.lib.f2d_world_autotune(self.id, dt, substeps, steps_per_candidate, _iptr(out))
        return st, (int(out[0]), int(out[1])), int(out[2])

    def tuning(self):
        out = np.zeros(2, np.int32)
        self.lib.f2d_world_get_tuning(self.id, _iptr(out))
        return int(out[0]), int(out[1])

    # learned warm start ---------------------------------------------------
    def set_sample_recording(self, capacity):
        self.lib.f2d_world_set_sample_recording(self.id, int(capacity))

    def samples(self):
        n = self.lib.f2d_world_sample_count(self.id)
        out = np.zeros((max(n, 1), 14), np.float32)
        m = self.lib.f2d_world_get_samples(self.id, _fptr(out), n)
        return out[:m]

    def set_warm_start_model(self, model):
        """model: a WarmStartModel (or None to switch prediction off)."""
        self.lib.f2d_world_set_warm_start_model(self.id, model.handle if model is not None else 0)

    def begin_subworld(self, gx, gy):
        return self.lib.f2d_world_begin_subworld(self.id, gx, gy)

    # stepping ---------------------------------------------------------
    def step(self, dt=1.0 / 60.0, substeps=4):
        return self.lib.f2d_world_step(self.id, dt, substeps)

    def sync(self) -> int:
        return self.lib.f2d_world_sync(self.id)

    def last_step_ms(self) -> float:
        return self.lib.f2d_world_last_step_ms(self.id)

    def last_step_launches(self) -> int:
        return self.lib.f2d_world_last_step_launches(self.id)

    def set_profiling(self, enabled: bool):
        self.lib.f2d_world_set_profiling(self.id, int(enabled))

    def phase_ms(self) -> np.ndarray:
        out = np.zeros(6, np.float64)
        self.lib.f2d_world_get_phase_ms(self.id, out.ctypes.data_as(C.POINTER(C.c_double)))
        return out

    def rebuild_ms(self) -> float:
        """Profiling mode: the tree rebuild's time on its own stream."""
        return float(self.lib.f2d_world_get_rebuild_ms(self.id))

    def solver_latency(self, probe_barriers=2000):
        """(grid barriers of the last grid-wide solver launch, measured
        microseconds per grid barrier on its grid)."""
        out = np.zeros(2, np.float64)
        self.lib.f2d_world_get_solver_latency(self.id, probe_barriers, out.ctypes.data_as(C.POINTER(C.c_double)))
        return int(out[0]), float(out[1])

    def counters(self) -> dict:
        out = np.zeros(8, np.int32)
        self.lib.f2d_world_get_counters(self.id, _iptr(out))
        keys = ("awake_bodies", "contacts", "touching", "overflow", "active_colors", "color_rounds", "shapes",
                "joints")
        return {k: int(v) for k, v in zip(keys, out)}

    def set_contact_plan(self, plan):
        plan = np.ascontiguousarray(np.asarray(plan, dtype=np.int32).reshape(-1, 3))
        self.lib.f2d_world_set_contact_plan(self.id, _iptr(plan), len(plan))

    # dumps ------------------------------------------------------------
    def bodies(self) -> np.ndarray:
        n = self.lib.f2d_world_body_capacity(self.id)
        out = np.zeros((max(n, 1), BODY_STRIDE), np.float32)
        self.lib.f2d_world_get_bodies(self.id, _fptr(out), n)
        return out[:n]

    def contacts(self):
        n = self.lib.f2d_world_contact_capacity(self.id)
        ints = np.zeros((max(n, 1), CONTACT_INTS), np.int32)
        fl = np.zeros((max(n, 1), CONTACT_FLOATS), np.float32)
        m = self.lib.f2d_world_get_contacts(self.id, _iptr(ints), _fptr(fl), n)
        return ints[:m], fl[:m]

    def shapes(self):
        n = self.lib.f2d_world_shape_capacity(self.id)
        fl = np.zeros((max(n, 1), 8), np.float32)
        ints = np.zeros((max(n, 1), 4), np.int32)
        self.lib.f2d_world_get_shapes(self.id, _fptr(fl), _iptr(ints), n)
        return fl[:n], ints[:n]

    def mass(self) -> np.ndarray:
        n = self.lib.f2d_world_body_capacity(self.id)
        out = np.zeros((max(n, 1), 8), np.float32)
        self.lib.f2d_world_get_mass(self.id, _fptr(out), n)
        return out[:n]

    def color_counts(self) -> np.ndarray:
        out = np.zeros(12, np.int32)
        self.lib.f2d_world_get_color_counts(self.id, _iptr(out))
        return out

    def event_counts(self):
        out = np.zeros(4, np.int32)
        self.lib.f2d_world_get_event_counts(self.id, _iptr(out))
        return out

    def begin_events(self):
        n = int(self.event_counts()[0])
        out = np.zeros((max(n, 1), 4), np.int32)
        m = self.lib.f2d_world_get_begin_events(self.id, _iptr(out), n)
        return out[:m][:, [0, 2]] - 1

    def begin_manifolds(self):
        """Per begin event: normal (2), point count, then per point the world
        point (2) and separation (9 floats)."""
        n = int(self.event_counts()[0])
        out = np.zeros((max(n, 1), 9), np.float32)
        m = self.lib.f2d_world_get_begin_manifolds(self.id, out.ctypes.data_as(C.POINTER(C.c_float)), n)
        return out[:m]

    def end_events(self):
        n = int(self.event_counts()[1])
        out = np.zeros((max(n, 1), 4), np.int32)
        m = self.lib.f2d_world_get_end_events(self.id, _iptr(out), n)
        return out[:m][:, [0, 2]] - 1

    def hit_events(self):
        n = int(self.event_counts()[2])
        ints = np.zeros((max(n, 1), 4), np.int32)
        fl = np.zeros((max(n, 1), 5), np.float32)
        m = self.lib.f2d_world_get_hit_events(self.id, _iptr(ints), _fptr(fl), n)
        return ints[:m][:, [0, 2]] - 1, fl[:m]

    def move_events(self):
        n = int(self.event_counts()[3])
        ints = np.zeros((max(n, 1), 3), np.int32)
        fl = np.zeros((max(n, 1), 4), np.float32)
        m = self.lib.f2d_world_get_body_events(self.id, _iptr(ints), _fptr(fl), n)
        return ints[:m], fl[:m]

    def cast_ray_closest(self, ox, oy, tx, ty, cat=1, mask=-1):
        shape = np.zeros(2, np.int32)
        out = np.zeros(5, np.float32)
        hit = self.lib.f2d_world_cast_ray_closest(self.id, ox, oy, tx, ty, cat, mask, _iptr(shape), _fptr(out))
        if not hit:
            return None
        return int(shape[0]) - 1, out

    def overlap_aabb(self, lx, ly, ux, uy, cat=1, mask=-1):
        cap = 1 << 16
        out = np.zeros((cap, 2), np.int32)
        n = self.lib.f2d_world_overlap_aabb(self.id, lx, ly, ux, uy, cat, mask, _iptr(out), cap)
        return out[:min(n, cap), 0] - 1

    def overlap_aabb_noalloc(self, lx, ly, ux, uy, cat=1, mask=-1, capacity=1 << 16):
        """f2d_world_overlap_aabb_noalloc: returns (count or negative code,
        the written (index1, worldAndGeneration) rows)."""
        out = np.zeros((max(capacity, 1), 2), np.int32)
        n = self.lib.f2d_world_overlap_aabb_noalloc(self.id, lx, ly, ux, uy, cat, mask, _iptr(out), capacity)
        return n, out[:max(0, min(n, capacity))]


class WarmStartModel:
    """The learned warm-start MLP [12 -> 64 -> 64 -> 2] on the GPU: BF16
    weights, FP32 accumulation, trained with the library's own forward and
    backward kernels."""

    def __init__(self, seed=1):
        self.lib = native.lib()
        self.handle = self.lib.f2d_mlp_create(seed)
        if self.handle == 0:
            raise RuntimeError("f2d_mlp_create failed")
        self.n_params = self.lib.f2d_mlp_param_count()
        self.mean = np.zeros(14, np.float32)
        self.inv_std = np.ones(14, np.float32)

    def close(self):
        if self.handle:
            self.lib.f2d_mlp_destroy(self.handle)
            self.handle = 0

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self):
        out = np.zeros(self.n_params, np.float32)
        self.lib.f2d_mlp_get_params(self.handle, _fptr(out))
        return out

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        self.lib.f2d_mlp_set_params(self.handle, _fptr(p))

    def set_normalization(self, mean, inv_std):
        self.mean = np.ascontiguousarray(mean, np.float32)
        self.inv_std = np.ascontiguousarray(inv_std, np.float32)
        self.lib.f2d_mlp_set_normalization(self.handle, _fptr(self.mean), _fptr(self.inv_std))

    def fit_normalization(self, samples):
        s = np.asarray(samples, np.float64)
        mean = s.mean(0)
        std = s.std(0)
        std[std < 1e-6] = 1.0
        self.set_normalization(mean.astype(np.float32), (1.0 / std).astype(np.float32))

    def gradient(self, samples):
        s = np.ascontiguousarray(samples, np.float32)
        g = np.zeros(self.n_params, np.float32)
        loss = self.lib.f2d_mlp_gradient(self.handle, _fptr(s), len(s), _fptr(g))
        return g, loss

    def train(self, samples, epochs=4, batch=4096, lr=2e-3, seed=1):
        s = np.ascontiguousarray(samples, np.float32)
        return self.lib.f2d_mlp_train(self.handle, _fptr(s), len(s), epochs, batch, lr, seed)

    def predict(self, feats):
        f = np.ascontiguousarray(feats, np.float32)
        out = np.zeros((len(f), 2), np.float32)
        self.lib.f2d_mlp_predict(self.handle, _fptr(f), len(f), _fptr(out))
        return out


# ---------------------------------------------------------------------------
# forge2d-style object API
# ---------------------------------------------------------------------------
class Shape:
    def __init__(self, world, sid):
        self.world, self.id = world, sid

    @property
    def is_valid(self):
        return bool(self.world.lib.f2d_shape_is_valid(*self.id))

    @property
    def type(self):
        return self.world.lib.f2d_shape_get_type(*self.id)


class Body:
    def __init__(self, world, bid):
        self.world, self.id = world, bid

    @property
    def lib(self):
        return self.world.lib

    def create_box(self, half_width, half_height, center=(0.0, 0.0), rotation=(1.0, 0.0), radius=0.0, **sd):
        return Shape(self.world, self.world._w.create_box(self.id, sd, half_width, half_height, center[0], center[1],
                                                          rotation[0], rotation[1], radius))

    def create_circle(self, radius, center=(0.0, 0.0), **sd):
        return Shape(self.world, self.world._w.create_circle(self.id, sd, center[0], center[1], radius))

    def create_capsule(self, center1, center2, radius, **sd):
        return Shape(self.world, self.world._w.create_capsule(self.id, sd, center1[0], center1[1], center2[0],
                                                              center2[1], radius))

    def create_segment(self, point1, point2, **sd):
        return Shape(self.world, self.world._w.create_segment(self.id, sd, point1[0], point1[1], point2[0],
                                                              point2[1]))

    def create_polygon(self, points, radius=0.0, **sd):
        sid = self.world._w.create_polygon(self.id, sd, points, radius)
        if sid == -1:
            raise ValueError("The points do not form a valid convex hull: at least three distinct, "
                             "non-collinear points are required")
        return Shape(self.world, sid)

    @property
    def position(self):
        x, y = C.c_double(), C.c_double()
        self.lib.f2d_body_get_position(self.id[0], self.id[1], C.byref(x), C.byref(y))
        return (x.value, y.value)

    @property
    def rotation(self):
        c, s = C.c_double(), C.c_double()
        self.lib.f2d_body_get_rotation(self.id[0], self.id[1], C.byref(c), C.byref(s))
        return (c.value, s.value)

    @property
    def linear_velocity(self):
        x, y = C.c_double(), C.c_double()
        self.lib.f2d_body_get_linear_velocity(self.id[0], self.id[1], C.byref(x), C.byref(y))
        return (x.value, y.value)

    @linear_velocity.setter
    def linear_velocity(self, v):
        self.lib.f2d_body_set_linear_velocity(self.id[0], self.id[1], v[0], v[1])

    @property
    def angular_velocity(self):
        return self.lib.f2d_body_get_angular_velocity(self.id[0], self.id[1])

    @angular_velocity.setter
    def angular_velocity(self, w):
        self.lib.f2d_body_set_angular_velocity(self.id[0], self.id[1], w)

    def set_transform(self, position, rotation=(1.0, 0.0)):
        self.lib.f2d_body_set_transform(self.id[0], self.id[1], position[0], position[1], rotation[0], rotation[1])

    def apply_force(self, force, point, wake=True):
        self.lib.f2d_body_apply_force(self.id[0], self.id[1], force[0], force[1], point[0], point[1], int(wake))

    def apply_force_to_center(self, force, wake=True):
        self.lib.f2d_body_apply_force_to_center(self.id[0], self.id[1], force[0], force[1], int(wake))

    def apply_torque(self, torque, wake=True):
        self.lib.f2d_body_apply_torque(self.id[0], self.id[1], torque, int(wake))

    def apply_linear_impulse(self, impulse, point, wake=True):
        self.lib.f2d_body_apply_linear_impulse(self.id[0], self.id[1], impulse[0], impulse[1], point[0], point[1],
                                               int(wake))

    def apply_linear_impulse_to_center(self, impulse, wake=True):
        self.lib.f2d_body_apply_linear_impulse_to_center(self.id[0], self.id[1], impulse[0], impulse[1], int(wake))

    def apply_angular_impulse(self, impulse, wake=True):
        self.lib.f2d_body_apply_angular_impulse(self.id[0], self.id[1], impulse, int(wake))

    @property
    def is_awake(self):
        return bool(self.lib.f2d_body_is_awake(*self.id))

    def set_awake(self, awake):
        self.lib.f2d_body_set_awake(self.id[0], self.id[1], int(awake))

    @property
    def sleep_threshold(self):
        return self.lib.f2d_body_get_sleep_threshold(*self.id)

    @sleep_threshold.setter
    def sleep_threshold(self, value):
        self.lib.f2d_body_set_sleep_threshold(self.id[0], self.id[1], value)

    @property
    def is_sleep_enabled(self):
        return bool(self.lib.f2d_body_is_sleep_enabled(*self.id))

    def enable_sleep(self, enabled):
        self.lib.f2d_body_enable_sleep(self.id[0], self.id[1], int(enabled))

    @property
    def mass(self):
        return self.lib.f2d_body_get_mass(*self.id)

    @property
    def rotational_inertia(self):
        return self.lib.f2d_body_get_rotational_inertia(*self.id)

    @property
    def type(self):
        return self.lib.f2d_body_get_type(*self.id)

    @type.setter
    def type(self, value):
        self.lib.f2d_body_set_type(self.id[0], self.id[1], int(value))

    @property
    def is_enabled(self):
        return bool(self.lib.f2d_body_get_param(self.id[0], self.id[1], native.CODES["F2D_BODY_ENABLED"]))

    def set_enabled(self, flag):
        """Body.setEnabled: b2Body_Enable / b2Body_Disable."""
        (self.lib.f2d_body_enable if flag else self.lib.f2d_body_disable)(self.id[0], self.id[1])

    @property
    def is_valid(self):
        return bool(self.lib.f2d_body_is_valid(*self.id))


class Joint:
    def __init__(self, world, jid):
        self.world, self.id = world, jid

    @property
    def is_valid(self):
        return bool(self.world.lib.f2d_joint_is_valid(*self.id))

    def set_target(self, x, y):
        """MouseJoint.setTarget: takes effect at the next step."""
        self.world.lib.f2d_mouse_joint_set_target(self.id[0], self.id[1], x, y)


class World:
    """forge2d ``World``: step, createBody, createRevoluteJoint, events, queries."""

    def __init__(self, gravity=(0.0, -10.0), **world_def):
        wd = dict(gravityX=gravity[0], gravityY=gravity[1])
        wd.update(world_def)
        self._w = GpuWorld(wd)
        self.lib = self._w.lib

    @property
    def id(self):
        return self._w.id

    def destroy(self):
        self._w.close()

    def step(self, dt, sub_step_count=4):
        return self._w.step(dt, sub_step_count)

    def create_body(self, **body_def):
        return Body(self, self._w.create_body(body_def))

    def create_revolute_joint(self, body_a, body_b, **jd):
        jd = dict(jd)
        jd["bodyA"] = body_a.id
        jd["bodyB"] = body_b.id
        return Joint(self, self._w.create_revolute(jd))

    def create_weld_joint(self, body_a, body_b, **jd):
        jd = dict(jd, type=JOINT_WELD, bodyA=body_a.id, bodyB=body_b.id)
        return Joint(self, self._w.create_joint(jd))

    def create_distance_joint(self, body_a, body_b, **jd):
        jd = dict(jd, type=JOINT_DISTANCE, bodyA=body_a.id, bodyB=body_b.id)
        return Joint(self, self._w.create_joint(jd))

    def create_prismatic_joint(self, body_a, body_b, **jd):
        jd = dict(jd, type=JOINT_PRISMATIC, bodyA=body_a.id, bodyB=body_b.id)
        return Joint(self, self._w.create_joint(jd))

    def create_wheel_joint(self, body_a, body_b, **jd):
        jd = dict(jd, type=JOINT_WHEEL, bodyA=body_a.id, bodyB=body_b.id)
        return Joint(self, self._w.create_joint(jd))

    def create_motor_joint(self, body_a, body_b, **jd):
        jd = dict(jd, type=JOINT_MOTOR, bodyA=body_a.id, bodyB=body_b.id)
        return Joint(self, self._w.create_joint(jd))

    def create_mouse_joint(self, body_a, body_b, **jd):
        jd = dict(jd, type=JOINT_MOUSE, bodyA=body_a.id, bodyB=body_b.id)
        return Joint(self, self._w.create_joint(jd))

    def create_filter_joint(self, body_a, body_b):
        jd = dict(type=JOINT_FILTER, bodyA=body_a.id, bodyB=body_b.id)
        return Joint(self, self._w.create_joint(jd))

    @property
    def gravity(self):
        x, y = C.c_double(), C.c_double()
        self.lib.f2d_world_get_gravity(self.id, C.byref(x), C.byref(y))
        return (x.value, y.value)

    @gravity.setter
    def gravity(self, g):
        self.lib.f2d_world_set_gravity(self.id, g[0], g[1])

    def cast_ray_closest(self, origin, translation, category_bits=1, mask_bits=-1):
        return self._w.cast_ray_closest(origin[0], origin[1], translation[0], translation[1], category_bits,
                                        mask_bits)

    def overlap_aabb(self, lower, upper, category_bits=1, mask_bits=-1):
        return self._w.overlap_aabb(lower[0], lower[1], upper[0], upper[1], category_bits, mask_bits)

    def contact_events(self):
        return {"begin": self._w.begin_events(), "end": self._w.end_events(), "hit": self._w.hit_events()}

    def body_move_events(self):
        return self._w.move_events()
