"""ctypes front end of the two CPU oracles. TEST INFRASTRUCTURE ONLY.

* ``RefWorld`` drives the unmodified Box2D v3.1.1 C library that forge2d
  vendors (packages/forge2d/third_party/box2d), compiled into
  ``oracle/_ref/libbox2d_ref.so`` together with ``oracle/ref_harness.c``.
  It exists only where the reference checkout exists.
* ``PortWorld`` drives ``oracle/_build/libf2d_port.so``, the plain-C
  restatement in ``oracle/port/`` that travels with the repository and is the
  parity reference and CPU baseline on machines without the reference.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline arm may
import this module; the product package never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_SO = os.path.join(HERE, "_ref", "libbox2d_ref.so")
PORT_SO = os.path.join(HERE, "_build", "libf2d_port.so")


def reference_box2d_dir() -> str:
    """The reference's vendored Box2D tree: $F2D_REF_B2 when set, else the
    default of the build recipe (``REF_B2 ?=`` in oracle/Makefile)."""
    env = os.environ.get("F2D_REF_B2")
    if env:
        return env
    try:
        with open(os.path.join(HERE, "Makefile")) as f:
            for line in f:
                if line.startswith("REF_B2 ?="):
                    return line.split("?=", 1)[1].strip()
    except OSError:
        pass
    return ""


REF_B2 = reference_box2d_dir()

BODY_STRIDE = 12
CONTACT_INTS = 9
CONTACT_FLOATS = 25


class WorldDef(C.Structure):
    _fields_ = [
        ("gravityX", C.c_double), ("gravityY", C.c_double),
        ("restitutionThreshold", C.c_double), ("hitEventThreshold", C.c_double),
        ("contactHertz", C.c_double), ("contactDampingRatio", C.c_double),
        ("maxContactPushSpeed", C.c_double), ("maximumLinearSpeed", C.c_double),
        ("enableSleep", C.c_int32), ("enableContinuous", C.c_int32),
    ]


class BodyDef(C.Structure):
    _fields_ = [
        ("type", C.c_int32), ("pad0", C.c_int32),
        ("positionX", C.c_double), ("positionY", C.c_double),
        ("rotationCos", C.c_double), ("rotationSin", C.c_double),
        ("linearVelocityX", C.c_double), ("linearVelocityY", C.c_double),
        ("angularVelocity", C.c_double), ("linearDamping", C.c_double),
        ("angularDamping", C.c_double), ("gravityScale", C.c_double),
        ("sleepThreshold", C.c_double),
        ("enableSleep", C.c_int32), ("isAwake", C.c_int32),
        ("fixedRotation", C.c_int32), ("isBullet", C.c_int32),
        ("isEnabled", C.c_int32), ("allowFastRotation", C.c_int32),
    ]


class ShapeDef(C.Structure):
    _fields_ = [
        ("friction", C.c_double), ("restitution", C.c_double),
        ("rollingResistance", C.c_double), ("tangentSpeed", C.c_double),
        ("density", C.c_double),
        ("categoryBits", C.c_int64), ("maskBits", C.c_int64),
        ("groupIndex", C.c_int32), ("userMaterialId", C.c_int32),
        ("isSensor", C.c_int32), ("enableSensorEvents", C.c_int32),
        ("enableContactEvents", C.c_int32), ("enableHitEvents", C.c_int32),
        ("enablePreSolveEvents", C.c_int32), ("invokeContactCreation", C.c_int32),
        ("updateBodyMass", C.c_int32), ("pad0", C.c_int32),
    ]


class RevoluteDef(C.Structure):
    _fields_ = [
        ("bodyA", C.c_int32), ("bodyB", C.c_int32),
        ("localAnchorAX", C.c_double), ("localAnchorAY", C.c_double),
        ("localAnchorBX", C.c_double), ("localAnchorBY", C.c_double),
        ("referenceAngle", C.c_double), ("targetAngle", C.c_double),
        ("enableSpring", C.c_int32), ("pad0", C.c_int32),
        ("hertz", C.c_double), ("dampingRatio", C.c_double),
        ("enableLimit", C.c_int32), ("pad1", C.c_int32),
        ("lowerAngle", C.c_double), ("upperAngle", C.c_double),
        ("enableMotor", C.c_int32), ("pad2", C.c_int32),
        ("maxMotorTorque", C.c_double), ("motorSpeed", C.c_double),
        ("drawSize", C.c_double),
        ("collideConnected", C.c_int32), ("pad3", C.c_int32),
    ]


class ManifoldPointView(C.Structure):
    _fields_ = [(n, C.c_float) for n in ("pointX", "pointY", "anchorAX", "anchorAY", "anchorBX", "anchorBY",
                                        "separation")] + [("id", C.c_int32)]


class ManifoldView(C.Structure):
    """f2d_manifold_view: the manifold a pre-solve callback sees."""
    _fields_ = [("normalX", C.c_float), ("normalY", C.c_float), ("pointCount", C.c_int32), ("pad0", C.c_int32),
                ("points", ManifoldPointView * 2)]


FILTER_FN = C.CFUNCTYPE(C.c_int32, C.c_int32, C.c_int32, C.c_void_p)
CAST_FN = C.CFUNCTYPE(C.c_float, C.c_int32, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float, C.c_void_p)
PRESOLVE_FN = C.CFUNCTYPE(C.c_int32, C.c_int32, C.c_int32, C.POINTER(ManifoldView), C.c_void_p)


class JointDef(C.Structure):
    """f2d_joint_def: weld 2, distance 3, prismatic 4, wheel 5, motor 6,
    mouse 7 and filter 8 joints."""
    _fields_ = [
        ("type", C.c_int32), ("bodyA", C.c_int32), ("bodyB", C.c_int32), ("collideConnected", C.c_int32),
        ("localAnchorAX", C.c_double), ("localAnchorAY", C.c_double),
        ("localAnchorBX", C.c_double), ("localAnchorBY", C.c_double),
        ("referenceAngle", C.c_double),
        ("linearHertz", C.c_double), ("linearDampingRatio", C.c_double),
        ("angularHertz", C.c_double), ("angularDampingRatio", C.c_double),
        ("length", C.c_double), ("minLength", C.c_double), ("maxLength", C.c_double),
        ("hertz", C.c_double), ("dampingRatio", C.c_double),
        ("maxMotorForce", C.c_double), ("motorSpeed", C.c_double),
        ("enableSpring", C.c_int32), ("enableLimit", C.c_int32), ("enableMotor", C.c_int32), ("pad0", C.c_int32),
        ("localAxisAX", C.c_double), ("localAxisAY", C.c_double),
        ("targetTranslation", C.c_double), ("lowerTranslation", C.c_double), ("upperTranslation", C.c_double),
        ("maxMotorTorque", C.c_double),
        ("linearOffsetX", C.c_double), ("linearOffsetY", C.c_double), ("angularOffset", C.c_double),
        ("maxForce", C.c_double), ("maxTorque", C.c_double), ("correctionFactor", C.c_double),
        ("targetX", C.c_double), ("targetY", C.c_double),
    ]


def _fill(struct, values: dict):
    for k, v in values.items():
        setattr(struct, k, v)
    return struct


def build_ref(quiet=True) -> bool:
    """Compile the reference library in place (needs the reference tree)."""
    if not os.path.isdir(REF_B2):
        return os.path.exists(REF_SO)
    r = subprocess.run(["make", "-C", HERE, "ref", "-j8", "REF_B2=" + REF_B2], capture_output=quiet)
    return r.returncode == 0 and os.path.exists(REF_SO)


def build_port(quiet=True) -> bool:
    r = subprocess.run(["make", "-C", HERE, "port", "-j8"], capture_output=quiet)
    return r.returncode == 0 and os.path.exists(PORT_SO)


def ref_available() -> bool:
    return os.path.exists(REF_SO) or os.path.isdir(REF_B2)


_P = C.POINTER


def _bind(lib, prefix):
    d = C.c_double
    i = C.c_int
    sig = {
        "create_world": (i, [_P(WorldDef), i]),
        "destroy_world": (None, [i]),
        "world_step": (None, [i, d, i]),
        "world_step_timed": (d, [i, d, i, i]),
        "create_body": (i, [i, _P(BodyDef)]),
        "create_circle_shape": (i, [i, i, _P(ShapeDef), d, d, d]),
        "create_capsule_shape": (i, [i, i, _P(ShapeDef), d, d, d, d, d]),
        "create_segment_shape": (i, [i, i, _P(ShapeDef), d, d, d, d]),
        "create_chain": (i, [i, i, _P(d), i, _P(d), i, C.c_longlong, C.c_longlong, i, i, i]),
        "chain_get_segments": (i, [i, i, _P(i), i]),
        "get_sensor_events": (i, [i, _P(i), _P(i), i, _P(i)]),
        "set_custom_filter": (None, [i, FILTER_FN, C.c_void_p]),
        "set_pre_solve": (None, [i, PRESOLVE_FN, C.c_void_p]),
        "world_explode": (None, [i, C.c_longlong, d, d, d, d, d]),
        "joint_set_motor": (None, [i, i, i, d, d]),
        "joint_set_limits": (None, [i, i, i, d, d]),
        "joint_get_constraint": (None, [i, i, _P(C.c_float)]),
        "world_cast_ray": (i, [i, d, d, d, d, C.c_longlong, C.c_longlong, CAST_FN, C.c_void_p]),
        "create_box_shape": (i, [i, i, _P(ShapeDef), d, d, d, d, d, d, d]),
        "create_polygon_shape": (i, [i, i, _P(ShapeDef), _P(d), i, d]),
        "create_revolute_joint": (i, [i, _P(RevoluteDef)]),
        "body_capacity": (i, [i]),
        "get_bodies": (i, [i, _P(C.c_float), i]),
        "contact_capacity": (i, [i]),
        "get_contacts": (i, [i, _P(i), _P(C.c_float), i]),
        "shape_capacity": (i, [i]),
        "get_shapes": (i, [i, _P(C.c_float), _P(i), i]),
        "get_mass": (i, [i, _P(C.c_float), i]),
        "get_polygon": (i, [i, i, _P(C.c_float)]),
        "get_color_counts": (None, [i, _P(i)]),
        "awake_body_count": (i, [i]),
        "event_counts": (None, [i, _P(i)]),
        "get_begin_events": (i, [i, _P(i), i]),
        "get_end_events": (i, [i, _P(i), i]),
        "get_begin_manifolds": (i, [i, _P(C.c_float), i]),
        "get_hit_events": (i, [i, _P(i), _P(C.c_float), i]),
        "get_move_events": (i, [i, _P(i), _P(C.c_float), i]),
        "cast_ray_closest": (i, [i, d, d, d, d, C.c_longlong, C.c_longlong, _P(i), _P(C.c_float)]),
        "overlap_aabb": (i, [i, d, d, d, d, C.c_longlong, C.c_longlong, _P(i), i]),
        "joint_color": (i, [i, i]),
        "body_set_awake": (None, [i, i, i]),
        "create_joint": (i, [i, _P(JointDef)]),
        "mouse_joint_set_target": (None, [i, i, d, d]),
        "world_enable_sleeping": (None, [i, i]),
        "tree_order": (i, [i, i, _P(i), i]),
        "destroy_body": (None, [i, i]),
        "body_set_type": (None, [i, i, i]),
        "body_disable": (None, [i, i]),
        "body_enable": (None, [i, i]),
        "destroy_shape": (None, [i, i, i]),
        "destroy_joint": (None, [i, i]),
        "destroy_chain": (None, [i, i]),
        "tree_stats": (None, [i, i, _P(i)]),
        "tree_nodes": (i, [i, i, _P(i), _P(C.c_float), i]),
        "body_get_param": (d, [i, i, i]),
        "body_set_param": (None, [i, i, i, d]),
        "body_set_mass_data": (None, [i, i, d, d, d, d]),
        "body_apply_mass_from_shapes": (None, [i, i]),
        "shape_get_param": (d, [i, i, i]),
        "shape_set_param": (None, [i, i, i, d, i]),
        "shape_set_filter": (None, [i, i, C.c_longlong, C.c_longlong, i]),
        "shape_test_point": (i, [i, i, d, d]),
        "chain_set_param": (None, [i, i, i, d]),
        "joint_get_param": (d, [i, i, i]),
        "joint_set_param": (None, [i, i, i, d, d]),
    }
    out = {}
    for name, (res, args) in sig.items():
        fn = getattr(lib, prefix + name, None)
        if fn is None:
            continue
        fn.restype = res
        fn.argtypes = args
        out[name] = fn
    return out


def _fptr(a):
    return a.ctypes.data_as(_P(C.c_float))


def _iptr(a):
    return a.ctypes.data_as(_P(C.c_int))


class _CpuWorld:
    """Common driver for ref_* and orc_* libraries (same flat signatures)."""

    _lib = None
    _fns = None
    prefix = ""

    def __init__(self, world_def: dict, workers: int = 1):
        wd = _fill(WorldDef(), world_def)
        self.w = self._fns["create_world"](C.byref(wd), int(workers))
        if self.w < 0:
            raise RuntimeError("world table full")

    def cast_ray(self, ox, oy, tx, ty, fn, cat=1, mask=-1):
        """b2World_CastRay: fn(shape, point(2), normal(2), fraction) -> float."""
        cb = CAST_FN(lambda s, px, py, nx, ny, f, ctx: float(fn(s, (px, py), (nx, ny), f)))
        return self._fns["world_cast_ray"](self.w, ox, oy, tx, ty, cat, mask, cb, None)

    def joint_constraint(self, joint):
        """(force.x, force.y, torque) of the last step."""
        out = np.zeros(3, np.float32)
        self._fns["joint_get_constraint"](self.w, joint, out.ctypes.data_as(_P(C.c_float)))
        return out

    def set_limits(self, joint, enable, lower, upper):
        """Limit of a revolute, prismatic or wheel joint."""
        self._fns["joint_set_limits"](self.w, joint, int(enable), lower, upper)

    def set_motor(self, joint, enable, speed, max_motor):
        """Motor of a revolute, prismatic, wheel or distance joint."""
        self._fns["joint_set_motor"](self.w, joint, int(enable), speed, max_motor)

    def explode(self, x, y, radius, falloff, impulse_per_length, mask=-1):
        """b2World_Explode."""
        self._fns["world_explode"](self.w, mask, x, y, radius, falloff, impulse_per_length)

    def set_custom_filter(self, fn):
        """fn(shapeA, shapeB) -> bool, 0-based shape ids; None removes it."""
        self._filter_cb = FILTER_FN(lambda a, b, ctx: int(bool(fn(a, b)))) if fn else FILTER_FN()
        self._fns["set_custom_filter"](self.w, self._filter_cb, None)

    def set_pre_solve(self, fn):
        """fn(shapeA, shapeB, ManifoldView) -> bool; None removes it."""
        self._presolve_cb = PRESOLVE_FN(lambda a, b, m, ctx: int(bool(fn(a, b, m.contents)))) if fn else PRESOLVE_FN()
        self._fns["set_pre_solve"](self.w, self._presolve_cb, None)

    # properties (the product header's generic get/set codes) ----------
    @staticmethod
    def _code(code):
        if isinstance(code, str):
            from forge2d_gb300.native import CODES
            return CODES[code]
        return code

    def body_get(self, body, code):
        return self._fns["body_get_param"](self.w, body, self._code(code))

    def body_set(self, body, code, value):
        self._fns["body_set_param"](self.w, body, self._code(code), value)

    def body_set_mass_data(self, body, mass, inertia, cx, cy):
        self._fns["body_set_mass_data"](self.w, body, mass, inertia, cx, cy)

    def body_apply_mass_from_shapes(self, body):
        self._fns["body_apply_mass_from_shapes"](self.w, body)

    def shape_get(self, shape, code):
        return self._fns["shape_get_param"](self.w, shape, self._code(code))

    def shape_set(self, shape, code, value, flag=0):
        self._fns["shape_set_param"](self.w, shape, self._code(code), value, int(flag))

    def shape_set_filter(self, shape, category, mask, group):
        self._fns["shape_set_filter"](self.w, shape, category, mask, group)

    def shape_test_point(self, shape, x, y):
        return bool(self._fns["shape_test_point"](self.w, shape, x, y))

    def chain_set(self, chain, code, value):
        self._fns["chain_set_param"](self.w, chain, self._code(code), value)

    def joint_get(self, joint, code):
        return self._fns["joint_get_param"](self.w, joint, self._code(code))

    def joint_set(self, joint, code, value, value2=0.0):
        self._fns["joint_set_param"](self.w, joint, self._code(code), value, value2)

    # destroy path -----------------------------------------------------
    def body_set_type(self, body, body_type):
        self._fns["body_set_type"](self.w, body, body_type)

    def body_disable(self, body):
        self._fns["body_disable"](self.w, body)

    def body_enable(self, body):
        self._fns["body_enable"](self.w, body)

    def destroy_body(self, body):
        self._fns["destroy_body"](self.w, body)

    def destroy_shape(self, shape, update_mass=True):
        self._fns["destroy_shape"](self.w, shape, int(update_mass))

    def destroy_joint(self, joint):
        self._fns["destroy_joint"](self.w, joint)

    def destroy_chain(self, chain):
        self._fns["destroy_chain"](self.w, chain)

    def tree_order(self, body_type):
        """Leaf shape ids of the broadphase tree of ``body_type`` (0 static,
        1 kinematic, 2 dynamic) in depth-first visiting order."""
        out = np.zeros(self._fns["shape_capacity"](self.w) + 1, np.int32)
        n = self._fns["tree_order"](self.w, body_type, out.ctypes.data_as(_P(C.c_int)), len(out))
        return out[:n].copy()

    def tree_nodes(self, body_type):
        """Port only: every node of a tree as ints (child1, child2, parent,
        height, flags, shape) and boxes (lower, upper), by node id."""
        cap = self._fns["tree_nodes"](self.w, body_type, None, None, 0)
        ints = np.zeros((cap, 6), np.int32)
        boxes = np.zeros((cap, 4), np.float32)
        self._fns["tree_nodes"](self.w, body_type, _iptr(ints), _fptr(boxes), cap)
        return ints, boxes

    def tree_stats(self, body_type):
        """(nodeCount, nodeCapacity, proxyCount, height, root, freeList)."""
        out = np.zeros(6, np.int32)
        self._fns["tree_stats"](self.w, body_type, out.ctypes.data_as(_P(C.c_int)))
        return out

    def close(self):
        if self.w is not None and self.w >= 0:
            self._fns["destroy_world"](self.w)
            self.w = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # creation ---------------------------------------------------------
    def create_body(self, body_def: dict) -> int:
        return self._fns["create_body"](self.w, C.byref(_fill(BodyDef(), body_def)))

    def create_circle(self, body, sd, cx, cy, r):
        return self._fns["create_circle_shape"](self.w, body, C.byref(_fill(ShapeDef(), sd)), cx, cy, r)

    def create_capsule(self, body, sd, x1, y1, x2, y2, r):
        return self._fns["create_capsule_shape"](self.w, body, C.byref(_fill(ShapeDef(), sd)), x1, y1, x2, y2, r)

    def create_segment(self, body, sd, x1, y1, x2, y2):
        return self._fns["create_segment_shape"](self.w, body, C.byref(_fill(ShapeDef(), sd)), x1, y1, x2, y2)

    def create_chain(self, body, points, materials=((0.6, 0.0, 0.0, 0.0, 0, 0),), categoryBits=1, maskBits=-1,
                     groupIndex=0, isLoop=False, enableSensorEvents=False):
        """b2CreateChain: ``points`` (n, 2), ``materials`` one or n rows of
        (friction, restitution, rollingResistance, tangentSpeed,
        userMaterialId, customColor)."""
        pts = np.ascontiguousarray(np.asarray(points, np.float64).reshape(-1))
        mats = np.ascontiguousarray(np.asarray(materials, np.float64).reshape(-1))
        return self._fns["create_chain"](self.w, body, pts.ctypes.data_as(_P(C.c_double)), len(pts) // 2,
                                         mats.ctypes.data_as(_P(C.c_double)), len(mats) // 6, categoryBits,
                                         maskBits, groupIndex, int(isLoop), int(enableSensorEvents))

    def sensor_events(self):
        """This step's sensor (begin, end) events as (sensor shape, visitor
        shape) rows, in the order they were produced."""
        cap = 1 << 16
        b = np.zeros((cap, 2), np.int32)
        e = np.zeros((cap, 2), np.int32)
        ne = C.c_int(0)
        nb = self._fns["get_sensor_events"](self.w, b.ctypes.data_as(_P(C.c_int)), e.ctypes.data_as(_P(C.c_int)),
                                             cap, C.byref(ne))
        return b[:nb].copy(), e[:ne.value].copy()

    def chain_segments(self, chain):
        out = np.zeros(1 << 16, np.int32)
        n = self._fns["chain_get_segments"](self.w, chain, out.ctypes.data_as(_P(C.c_int)), len(out))
        return out[:n].copy()

    def create_box(self, body, sd, hx, hy, cx=0.0, cy=0.0, c=1.0, s=0.0, radius=0.0):
        return self._fns["create_box_shape"](self.w, body, C.byref(_fill(ShapeDef(), sd)), hx, hy, cx, cy, c, s, radius)

    def create_polygon(self, body, sd, points, radius=0.0):
        pts = np.ascontiguousarray(np.asarray(points, dtype=np.float64).reshape(-1))
        return self._fns["create_polygon_shape"](self.w, body, C.byref(_fill(ShapeDef(), sd)),
                                                 pts.ctypes.data_as(_P(C.c_double)), len(pts) // 2, radius)

    def create_revolute(self, jd: dict) -> int:
        return self._fns["create_revolute_joint"](self.w, C.byref(_fill(RevoluteDef(), jd)))

    # stepping ---------------------------------------------------------
    def step(self, dt=1.0 / 60.0, substeps=4):
        self._fns["world_step"](self.w, dt, substeps)

    def step_timed(self, dt, substeps, steps) -> float:
        return self._fns["world_step_timed"](self.w, dt, substeps, steps)

    # dumps ------------------------------------------------------------
    def bodies(self) -> np.ndarray:
        n = self._fns["body_capacity"](self.w)
        out = np.zeros((max(n, 1), BODY_STRIDE), np.float32)
        self._fns["get_bodies"](self.w, _fptr(out), n)
        return out[:n]

    def contacts(self):
        n = self._fns["contact_capacity"](self.w)
        ints = np.zeros((max(n, 1), CONTACT_INTS), np.int32)
        fl = np.zeros((max(n, 1), CONTACT_FLOATS), np.float32)
        m = self._fns["get_contacts"](self.w, _iptr(ints), _fptr(fl), n)
        return ints[:m], fl[:m]

    def shapes(self):
        n = self._fns["shape_capacity"](self.w)
        fl = np.zeros((max(n, 1), 8), np.float32)
        ints = np.zeros((max(n, 1), 4), np.int32)
        self._fns["get_shapes"](self.w, _fptr(fl), _iptr(ints), n)
        return fl[:n], ints[:n]

    def mass(self) -> np.ndarray:
        n = self._fns["body_capacity"](self.w)
        out = np.zeros((max(n, 1), 8), np.float32)
        self._fns["get_mass"](self.w, _fptr(out), n)
        return out[:n]

    def polygon(self, shape) -> np.ndarray:
        out = np.zeros(36, np.float32)
        self._fns["get_polygon"](self.w, shape, _fptr(out))
        return out

    def color_counts(self) -> np.ndarray:
        out = np.zeros(24, np.int32)
        self._fns["get_color_counts"](self.w, _iptr(out))
        return out[:12]

    def event_counts(self):
        out = np.zeros(4, np.int32)
        self._fns["event_counts"](self.w, _iptr(out))
        return out

    def begin_events(self):
        n = int(self.event_counts()[0])
        out = np.zeros((max(n, 1), 2), np.int32)
        m = self._fns["get_begin_events"](self.w, _iptr(out), n)
        return out[:m]

    def begin_manifolds(self):
        """Per begin event: normal (2), point count, then per point the world
        point (2) and separation (9 floats)."""
        n = int(self.event_counts()[0])
        out = np.zeros((max(n, 1), 9), np.float32)
        m = self._fns["get_begin_manifolds"](self.w, _fptr(out), n)
        return out[:m]

    def end_events(self):
        n = int(self.event_counts()[1])
        out = np.zeros((max(n, 1), 2), np.int32)
        m = self._fns["get_end_events"](self.w, _iptr(out), n)
        return out[:m]

    def hit_events(self):
        n = int(self.event_counts()[2])
        ints = np.zeros((max(n, 1), 2), np.int32)
        fl = np.zeros((max(n, 1), 5), np.float32)
        m = self._fns["get_hit_events"](self.w, _iptr(ints), _fptr(fl), n)
        return ints[:m], fl[:m]

    def move_events(self):
        n = int(self.event_counts()[3])
        ints = np.zeros((max(n, 1), 2), np.int32)
        fl = np.zeros((max(n, 1), 4), np.float32)
        m = self._fns["get_move_events"](self.w, _iptr(ints), _fptr(fl), n)
        return ints[:m], fl[:m]

    def cast_ray_closest(self, ox, oy, tx, ty, cat=1, mask=-1):
        shape = C.c_int(-1)
        out = np.zeros(5, np.float32)
        hit = self._fns["cast_ray_closest"](self.w, ox, oy, tx, ty, cat, mask, C.byref(shape), _fptr(out))
        if not hit:
            return None
        return shape.value, out

    def overlap_aabb(self, lx, ly, ux, uy, cat=1, mask=-1):
        cap = 4096
        out = np.zeros(cap, np.int32)
        n = self._fns["overlap_aabb"](self.w, lx, ly, ux, uy, cat, mask, _iptr(out), cap)
        return out[:min(n, cap)]

    def joint_color(self, j):
        return self._fns["joint_color"](self.w, j)

    def awake_body_count(self):
        return self._fns["awake_body_count"](self.w)

    def create_joint(self, jd: dict) -> int:
        """Weld or distance joint from a scenes.joint_def dict."""
        return self._fns["create_joint"](self.w, C.byref(_fill(JointDef(), jd)))

    def mouse_set_target(self, joint, x, y):
        self._fns["mouse_joint_set_target"](self.w, joint, x, y)

    def set_awake(self, body, awake):
        self._fns["body_set_awake"](self.w, body, int(awake))

    def enable_sleeping(self, enabled):
        self._fns["world_enable_sleeping"](self.w, int(enabled))


class RefWorld(_CpuWorld):
    prefix = "ref_"

    def __init__(self, world_def, workers=1):
        if RefWorld._lib is None:
            if not os.path.exists(REF_SO) and not build_ref():
                raise RuntimeError("reference library unavailable")
            RefWorld._lib = C.CDLL(REF_SO)
            RefWorld._fns = _bind(RefWorld._lib, "ref_")
        super().__init__(world_def, workers)


class PortWorld(_CpuWorld):
    prefix = "orc_"

    def __init__(self, world_def, workers=1):
        if PortWorld._lib is None:
            if not os.path.exists(PORT_SO) and not build_port():
                raise RuntimeError("port library failed to build")
            PortWorld._lib = C.CDLL(PORT_SO)
            PortWorld._fns = _bind(PortWorld._lib, "orc_")
            lib = PortWorld._lib
            lib.orc_set_contact_plan.restype = None
            lib.orc_set_contact_plan.argtypes = [C.c_int, _P(C.c_int), C.c_int]
        super().__init__(world_def, workers)

    def begin_subworld(self, gx, gy):
        """Batched form: later bodies form a new sub-world with this gravity."""
        fn = PortWorld._lib.orc_begin_subworld
        fn.restype = C.c_int
        fn.argtypes = [C.c_int, C.c_double, C.c_double]
        return fn(self.w, gx, gy)

    def set_contact_plan(self, plan: np.ndarray):
        """Parity mode: contacts created during the next step take the given
        ids. ``plan`` rows are (contactId, shapeIdA, shapeIdB)."""
        plan = np.ascontiguousarray(plan, dtype=np.int32).reshape(-1, 3)
        PortWorld._lib.orc_set_contact_plan(self.w, _iptr(plan), len(plan))
