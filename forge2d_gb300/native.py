"""ctypes binding of the C ABI in include/forge2d_gb300.h.

The library is built in-tree by ``forge2d_gb300.build`` into
``forge2d_gb300/_build/libforge2d_gb300.so``. There is no CPU fallback: if
the library is missing or cannot be loaded, ``lib()`` raises.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libforge2d_gb300.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "forge2d_gb300.h")


def _codes():
    """The property codes of the generic get/set calls, read from the C
    header (F2D_BODY_*, F2D_SHAPE_*, F2D_JP_*)."""
    import re
    out = {}
    with open(HEADER) as f:
        for m in re.finditer(r"^#define (F2D_(?:BODY|SHAPE|JP)_[A-Z_]+) (\d+)", f.read(), re.M):
            out[m.group(1)] = int(m.group(2))
    return out


CODES = _codes()

_P = C.POINTER
_lib = None


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
        ("bodyAIndex1", C.c_int32), ("bodyAWorldAndGeneration", C.c_int32),
        ("bodyBIndex1", C.c_int32), ("bodyBWorldAndGeneration", C.c_int32),
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


class JointDef(C.Structure):
    """f2d_joint_def: weld 2, distance 3, prismatic 4, wheel 5, motor 6,
    mouse 7 and filter 8 joints."""
    _fields_ = [
        ("type", C.c_int32),
        ("bodyAIndex1", C.c_int32), ("bodyAWorldAndGeneration", C.c_int32),
        ("bodyBIndex1", C.c_int32), ("bodyBWorldAndGeneration", C.c_int32),
        ("collideConnected", C.c_int32),
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


class ManifoldPointView(C.Structure):
    _fields_ = [(n, C.c_float) for n in ("pointX", "pointY", "anchorAX", "anchorAY", "anchorBX", "anchorBY",
                                        "separation")] + [("id", C.c_int32)]


class ManifoldView(C.Structure):
    """f2d_manifold_view: the new manifold a pre-solve callback sees."""
    _fields_ = [("normalX", C.c_float), ("normalY", C.c_float), ("pointCount", C.c_int32), ("pad0", C.c_int32),
                ("points", ManifoldPointView * 2)]


CastResultFn = C.CFUNCTYPE(C.c_float, C.c_int32, C.c_int32, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float,
                           C.c_void_p)
CustomFilterFn = C.CFUNCTYPE(C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_void_p)
PreSolveFn = C.CFUNCTYPE(C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.POINTER(ManifoldView),
                         C.c_void_p)


# (name, restype, argtypes)
_i, _d, _f, _i64 = C.c_int32, C.c_double, C.c_float, C.c_int64
_SIGS = [
    ("f2d_create_world", _i, [_P(WorldDef)]),
    ("f2d_destroy_world", None, [_i]),
    ("f2d_world_is_valid", _i, [_i]),
    ("f2d_world_step", _i, [_i, _d, _i]),
    ("f2d_world_sync", _i, [_i]),
    ("f2d_world_set_gravity", None, [_i, _d, _d]),
    ("f2d_world_get_gravity", None, [_i, _P(_d), _P(_d)]),
    ("f2d_world_begin_subworld", _i, [_i, _d, _d]),
    ("f2d_world_subworld_count", _i, [_i]),
    ("f2d_world_enable_sleeping", None, [_i, _i]),
    ("f2d_world_is_sleeping_enabled", _i, [_i]),
    ("f2d_world_enable_continuous", None, [_i, _i]),
    ("f2d_world_is_continuous_enabled", _i, [_i]),
    ("f2d_create_body", _i, [_i, _P(BodyDef), _P(_i), _P(_i)]),
    ("f2d_body_is_valid", _i, [_i, _i]),
    ("f2d_destroy_body", None, [_i, _i]),
    ("f2d_destroy_shape", None, [_i, _i, _i]),
    ("f2d_destroy_chain", None, [_i, _i]),
    ("f2d_destroy_joint", None, [_i, _i]),
    ("f2d_joint_set_collide_connected", None, [_i, _i, _i]),
    ("f2d_joint_get_collide_connected", _i, [_i, _i]),
    ("f2d_body_get_param", _d, [_i, _i, _i]),
    ("f2d_body_set_param", None, [_i, _i, _i, _d]),
    ("f2d_body_get_world_point", None, [_i, _i, _d, _d, _P(_d), _P(_d)]),
    ("f2d_body_get_local_point", None, [_i, _i, _d, _d, _P(_d), _P(_d)]),
    ("f2d_body_set_mass_data", None, [_i, _i, _d, _d, _d, _d]),
    ("f2d_body_apply_mass_from_shapes", None, [_i, _i]),
    ("f2d_body_set_name", None, [_i, _i, C.c_char_p]),
    ("f2d_body_get_name", _i, [_i, _i, C.c_char_p, _i]),
    ("f2d_body_get_shapes", _i, [_i, _i, _P(_i), _i]),
    ("f2d_body_get_joints", _i, [_i, _i, _P(_i), _i]),
    ("f2d_shape_get_param", _d, [_i, _i, _i]),
    ("f2d_shape_set_param", None, [_i, _i, _i, _d, _i]),
    ("f2d_shape_get_body", _i, [_i, _i, _P(_i), _P(_i)]),
    ("f2d_shape_set_filter", None, [_i, _i, _i64, _i64, _i]),
    ("f2d_shape_test_point", _i, [_i, _i, _d, _d]),
    ("f2d_shape_get_geometry", _i, [_i, _i, _i, _P(_d), _i]),
    ("f2d_shape_get_aabb", None, [_i, _i, _P(_d)]),
    ("f2d_chain_is_valid", _i, [_i, _i]),
    ("f2d_chain_get_param", _d, [_i, _i, _i]),
    ("f2d_chain_set_param", None, [_i, _i, _i, _d]),
    ("f2d_joint_get_param", _d, [_i, _i, _i]),
    ("f2d_joint_set_param", None, [_i, _i, _i, _d, _d]),
    ("f2d_joint_get_body", _i, [_i, _i, _i, _P(_i), _P(_i)]),
    ("f2d_joint_wake_bodies", None, [_i, _i]),
    ("f2d_world_get_solver_latency", None, [_i, _i, _P(_d)]),
    ("f2d_body_get_position", None, [_i, _i, _P(_d), _P(_d)]),
    ("f2d_body_get_rotation", None, [_i, _i, _P(_d), _P(_d)]),
    ("f2d_body_set_transform", None, [_i, _i, _d, _d, _d, _d]),
    ("f2d_body_get_linear_velocity", None, [_i, _i, _P(_d), _P(_d)]),
    ("f2d_body_set_linear_velocity", None, [_i, _i, _d, _d]),
    ("f2d_body_get_angular_velocity", _d, [_i, _i]),
    ("f2d_body_set_angular_velocity", None, [_i, _i, _d]),
    ("f2d_body_apply_force", None, [_i, _i, _d, _d, _d, _d, _i]),
    ("f2d_body_apply_force_to_center", None, [_i, _i, _d, _d, _i]),
    ("f2d_body_apply_torque", None, [_i, _i, _d, _i]),
    ("f2d_body_apply_linear_impulse", None, [_i, _i, _d, _d, _d, _d, _i]),
    ("f2d_body_apply_linear_impulse_to_center", None, [_i, _i, _d, _d, _i]),
    ("f2d_body_apply_angular_impulse", None, [_i, _i, _d, _i]),
    ("f2d_body_get_mass", _d, [_i, _i]),
    ("f2d_body_get_rotational_inertia", _d, [_i, _i]),
    ("f2d_body_get_type", _i, [_i, _i]),
    ("f2d_body_is_awake", _i, [_i, _i]),
    ("f2d_body_set_awake", None, [_i, _i, _i]),
    ("f2d_body_set_type", None, [_i, _i, _i]),
    ("f2d_body_disable", None, [_i, _i]),
    ("f2d_body_enable", None, [_i, _i]),
    ("f2d_body_is_sleep_enabled", _i, [_i, _i]),
    ("f2d_body_enable_sleep", None, [_i, _i, _i]),
    ("f2d_body_get_sleep_threshold", _d, [_i, _i]),
    ("f2d_body_set_sleep_threshold", None, [_i, _i, _d]),
    ("f2d_create_circle_shape", _i, [_i, _i, _P(ShapeDef), _d, _d, _d, _P(_i), _P(_i)]),
    ("f2d_create_capsule_shape", _i, [_i, _i, _P(ShapeDef), _d, _d, _d, _d, _d, _P(_i), _P(_i)]),
    ("f2d_create_segment_shape", _i, [_i, _i, _P(ShapeDef), _d, _d, _d, _d, _P(_i), _P(_i)]),
    ("f2d_create_box_shape", _i, [_i, _i, _P(ShapeDef), _d, _d, _d, _d, _d, _d, _d, _P(_i), _P(_i)]),
    ("f2d_create_polygon_shape", _i, [_i, _i, _P(ShapeDef), _P(_d), _i, _d, _P(_i), _P(_i)]),
    ("f2d_shape_is_valid", _i, [_i, _i]),
    ("f2d_shape_get_type", _i, [_i, _i]),
    ("f2d_create_revolute_joint", _i, [_i, _P(RevoluteDef), _P(_i), _P(_i)]),
    ("f2d_create_joint", _i, [_i, _P(JointDef), _P(_i), _P(_i)]),
    ("f2d_mouse_joint_set_target", None, [_i, _i, _d, _d]),
    ("f2d_joint_set_motor", None, [_i, _i, _i, _d, _d]),
    ("f2d_joint_set_limits", None, [_i, _i, _i, _d, _d]),
    ("f2d_joint_get_constraint", None, [_i, _i, _P(_f)]),
    ("f2d_create_chain", _i, [_i, _i, _P(_d), _i, _P(_d), _i, _i64, _i64, _i, _i, _i, _P(_i), _P(_i)]),
    ("f2d_chain_get_segments", _i, [_i, _i, _P(_i), _i]),
    ("f2d_world_get_sensor_events", _i, [_i, _P(_i), _P(_i), _i, _P(_i)]),
    ("f2d_world_set_custom_filter", None, [_i, CustomFilterFn, C.c_void_p]),
    ("f2d_world_set_pre_solve", None, [_i, PreSolveFn, C.c_void_p]),
    ("f2d_world_explode", None, [_i, _i64, _d, _d, _d, _d, _d]),
    ("f2d_world_cast_ray", _i, [_i, _d, _d, _d, _d, _i64, _i64, CastResultFn, C.c_void_p]),
    ("f2d_joint_is_valid", _i, [_i, _i]),
    ("f2d_world_get_event_counts", None, [_i, _P(_i)]),
    ("f2d_world_get_begin_events", _i, [_i, _P(_i), _i]),
    ("f2d_world_get_begin_manifolds", _i, [_i, _P(_f), _i]),
    ("f2d_world_get_end_events", _i, [_i, _P(_i), _i]),
    ("f2d_world_get_hit_events", _i, [_i, _P(_i), _P(_f), _i]),
    ("f2d_world_get_body_events", _i, [_i, _P(_i), _P(_f), _i]),
    ("f2d_world_cast_ray_closest", _i, [_i, _d, _d, _d, _d, _i64, _i64, _P(_i), _P(_f)]),
    ("f2d_world_overlap_aabb", _i, [_i, _d, _d, _d, _d, _i64, _i64, _P(_i), _i]),
    ("f2d_world_overlap_aabb_noalloc", _i, [_i, _d, _d, _d, _d, _i64, _i64, _P(_i), _i]),
    ("f2d_world_body_capacity", _i, [_i]),
    ("f2d_world_get_bodies", _i, [_i, _P(_f), _i]),
    ("f2d_world_contact_capacity", _i, [_i]),
    ("f2d_world_get_contacts", _i, [_i, _P(_i), _P(_f), _i]),
    ("f2d_world_shape_capacity", _i, [_i]),
    ("f2d_world_get_shapes", _i, [_i, _P(_f), _P(_i), _i]),
    ("f2d_world_get_mass", _i, [_i, _P(_f), _i]),
    ("f2d_world_get_color_counts", None, [_i, _P(_i)]),
    ("f2d_world_set_contact_plan", None, [_i, _P(_i), _i]),
    ("f2d_world_last_step_ms", _d, [_i]),
    ("f2d_world_last_step_launches", _i, [_i]),
    ("f2d_world_reserve", None, [_i, _i, _i, _i, _i]),
    ("f2d_world_autotune", _i, [_i, _d, _i, _i, _P(_i)]),
    ("f2d_world_set_sample_recording", None, [_i, _i]),
    ("f2d_world_sample_count", _i, [_i]),
    ("f2d_world_get_samples", _i, [_i, _P(_f), _i]),
    ("f2d_world_set_warm_start_model", _i, [_i, _i]),
    ("f2d_mlp_create", _i, [C.c_uint32]),
    ("f2d_mlp_destroy", None, [_i]),
    ("f2d_mlp_param_count", _i, []),
    ("f2d_mlp_get_params", None, [_i, _P(_f)]),
    ("f2d_mlp_set_params", None, [_i, _P(_f)]),
    ("f2d_mlp_set_normalization", None, [_i, _P(_f), _P(_f)]),
    ("f2d_mlp_gradient", _f, [_i, _P(_f), _i, _P(_f)]),
    ("f2d_mlp_train", _f, [_i, _P(_f), _i, _i, _i, _f, C.c_uint32]),
    ("f2d_mlp_predict", None, [_i, _P(_f), _i, _P(_f)]),
    ("f2d_world_get_tuning", None, [_i, _P(_i)]),
    ("f2d_world_set_profiling", None, [_i, _i]),
    ("f2d_world_get_phase_ms", None, [_i, _P(_d)]),
    ("f2d_world_get_rebuild_ms", _d, [_i]),
    ("f2d_world_get_counters", None, [_i, _P(_i)]),
]

SYMBOLS = [s[0] for s in _SIGS]


def header_symbols(path=None):
    """Names of every F2D_API entry point declared in include/forge2d_gb300.h."""
    import re
    if path is None:
        path = os.path.join(os.path.dirname(HERE), "include", "forge2d_gb300.h")
    text = open(path).read()
    return re.findall(r"F2D_API\s+[\w\s\*]+?\b(f2d_\w+)\s*\(", text)


def load(path: str = LIB_PATH):
    """Load the native library (raises when it is absent)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(
            "forge2d_gb300 native library not built (%s); run __graft_entry__.build() "
            "or python forge2d_gb300/build.py" % path)
    lib = C.CDLL(path)
    for name, res, args in _SIGS:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def lib():
    return load()
