"""Lock-step helpers shared by the parity tests.

``lockstep(ref, other, steps)`` steps a reference-side world and a
candidate world together; before each candidate step it hands the candidate
the contact ids the reference created in that step (parity mode), so that
colour assignment and every downstream result can be compared bit for bit.
"""
from __future__ import annotations

import numpy as np


def new_contacts(prev: set, ints: np.ndarray):
    cur = set((int(a), int(b), int(c)) for a, b, c in ints[:, :3])
    return cur, sorted(cur - prev)


def body_rows(world) -> np.ndarray:
    return world.bodies()[:, :9]


def first_mismatch(a: np.ndarray, b: np.ndarray):
    bad = np.argwhere(~((a == b) | (np.isnan(a) & np.isnan(b))))
    return None if len(bad) == 0 else bad[0].tolist()


def contact_table(world):
    ints, fl = world.contacts()
    return {int(r[0]): (r, f) for r, f in zip(ints, fl)}


def compare_contacts(a, b):
    """Contacts keyed by id: shape pair, colour, point count, point ids and
    every manifold float must agree. Returns a list of differences."""
    ta, tb = contact_table(a), contact_table(b)
    diffs = []
    if set(ta) != set(tb):
        diffs.append(("ids", sorted(set(ta) ^ set(tb))[:5]))
        return diffs
    for cid in ta:
        ra, fa = ta[cid]
        rb, fb = tb[cid]
        if not (np.array_equal(ra[[1, 2, 3, 4, 7, 8]], rb[[1, 2, 3, 4, 7, 8]]) and np.array_equal(fa, fb)):
            diffs.append((cid, ra.tolist(), rb.tolist()))
            if len(diffs) > 5:
                break
    return diffs


# User callbacks of the callback parity cases: pure functions of the shape
# ids and the manifold, so every world that installs them decides alike.
def filter_rule(a, b):
    """Custom filter: pairs whose shape ids sum to a multiple of 5 never
    collide."""
    return (a + b) % 5 != 0


def pre_solve_rule(a, b, m):
    """Pre-solve: contacts whose shape ids sum to a multiple of 4 are one-way
    (solved only while the normal does not point down)."""
    if (a + b) % 4 == 0:
        return m.normalY > -0.2
    return True


BLASTS = {150: (-1.5, 2.0, 3.0, 2.0, 2.5, -1), 250: (-0.5, 2.0, 3.0, 2.0, 2.5, -1), 330: (0.3, 2.0, 3.0, 0.0, 4.0, 1)}


def blast(world, f):
    """The explosions of the explode parity cases (frame -> x, y, radius,
    falloff, impulse per length, mask)."""
    if f in BLASTS:
        x, y, r, fo, ipl, mask = BLASTS[f]
        world.explode(x, y, r, fo, ipl, mask=mask)


def ray_answers(world, rays):
    """Closest hit through a closest-hit callback, and every hit through an
    all-hits callback (sorted), per ray."""
    out = []
    for o, t in rays:
        best = {}

        def closest(s, p, n, f):
            if f == 0.0:
                return -1.0
            best["r"] = (s, tuple(np.float32(v).view(np.uint32).item() for v in (*p, *n, f)))
            return f

        hits = []

        def every(s, p, n, f):
            hits.append((s, np.float32(f).view(np.uint32).item()))
            return 1.0

        world.cast_ray(o[0], o[1], t[0], t[1], closest)
        world.cast_ray(o[0], o[1], t[0], t[1], every)
        out.append((best.get("r"), sorted(hits)))
    return out


# frame -> (enable, speed, max) applied to every motorised joint of joint_rigs
MOTOR_EDITS = {100: (1, 3.0, 40.0), 160: (0, 3.0, 40.0), 220: (1, -1.5, 15.0), 280: (1, 0.5, 90.0)}


# frame -> (enable, lower, upper) for the same joints' limits
LIMIT_EDITS = {120: (1, -0.5, 0.8), 190: (0, -0.5, 0.8), 240: (1, 0.6, -0.2), 300: (1, -0.1, 0.1)}


def edit_motors(world, motors, f):
    if f in LIMIT_EDITS:
        enable, lo, hi = LIMIT_EDITS[f]
        for j in motors:
            world.set_limits(j, enable, lo, hi)
    if f in MOTOR_EDITS:
        enable, speed, mx = MOTOR_EDITS[f]
        for k, j in enumerate(motors):
            world.set_motor(j, enable, speed * (1.0 + 0.25 * (k % 3)), mx)


def install_callbacks(world):
    world.set_custom_filter(filter_rule)
    world.set_pre_solve(pre_solve_rule)


def touching_pair(world):
    """Body ids of the first touching contact between two dynamic bodies."""
    ints, _ = world.contacts()
    _, sh = world.shapes()
    mass = world.mass()
    for r in ints:
        if r[4] > 0 and ( r[5] & 1 ):
            a, b = int(sh[r[1], 1]), int(sh[r[2], 1])
            if a != b and mass[a, 2] > 0 and mass[b, 2] > 0:
                return a, b
    return None


def destroy_script(world, f, ids):
    """Destroys and re-creates between steps, the same calls on every world
    (bodies, shapes, joints and chains picked by id from the scene built by
    scenes.build(..., "pyramids_chains", pyramids=2, rows=8, chains=4,
    links=10) plus two chain shapes): ``ids`` holds the picks."""
    from forge2d_gb300 import scenes
    if f == 30:
        world.destroy_body(ids["box"])          # a box inside a pyramid
        world.destroy_body(ids["link"])         # a chain link: two joints go
    elif f == 50:
        world.destroy_shape(ids["shape"], True)  # one of two shapes of a body
        world.destroy_joint(ids["joint"])
    elif f == 70:
        world.destroy_chain(ids["chain"])
        # new bodies take the freed ids; the proxies take freed tree nodes
        for k in range(3):
            b = world.create_body(scenes.body_def(type=2, positionX=-3.0 + 1.1 * k, positionY=12.0 + k))
            world.create_circle(b, scenes.shape_def(enableContactEvents=1), 0.0, 0.0, 0.35)
    elif f == 90:
        pair = ids.get("touch")
        if pair is not None:
            # a joint between touching bodies ends their contacts
            world.create_revolute(scenes.revolute_def(bodyA=pair[0], bodyB=pair[1], collideConnected=0))
    elif f == 110:
        world.destroy_body(ids["last"])
        world.destroy_shape(ids["twin_box"], False)


def type_script(world, f):
    """Body type changes, disables and enables between steps, the same calls
    on every world, on the scene of build_destroy_scene (ground 0, pyramid
    boxes 1-72, chains of an anchor and ten links at 73, 84, 95 and 106, the
    two-shape body 117): dynamic <-> static <-> kinematic with and without
    joints, static anchors made dynamic, disabled bodies with joints, a type
    change while disabled. No call turns a static body holding two joints of
    the constraint graph non-static (the one colour deviation, see
    test_port_type_change_colour_deviation)."""
    calls = {
        15: [("body_set_type", 12, 0)],      # a pyramid box becomes static
        20: [("body_set_type", 78, 1)],      # a chain link (two joints) kinematic
        25: [("body_set_type", 117, 1)],     # the two-shape body kinematic
        35: [("body_set_type", 84, 2)],      # a static anchor (joint, no shapes) dynamic
        40: [("body_set_type", 78, 2), ("body_set_type", 12, 2)],
        50: [("body_disable", 89), ("body_disable", 30)],
        55: [("body_set_type", 30, 1)],      # type change while disabled
        65: [("body_set_type", 117, 2)],
        70: [("body_enable", 89), ("body_enable", 30)],
        80: [("body_set_type", 100, 0)],     # static between two dynamic links
        85: [("body_set_type", 101, 0)],     # its neighbour too: a joint between statics
        95: [("body_set_type", 101, 2)],     # static -> dynamic: one joint re-coloured, one from the static set
        100: [("body_set_type", 20, 1)],     # a box of a sleeping pyramid (with sleeping on) turns kinematic
        105: [("body_disable", 50)],         # a box of the other sleeping pyramid is disabled
        110: [("body_disable", 106)],        # a static anchor with a joint
        112: [("body_enable", 50), ("body_set_type", 20, 2)],
        120: [("body_enable", 106), ("body_set_type", 30, 2)],
        130: [("body_disable", 40), ("body_set_type", 60, 0)],
        135: [("body_enable", 40), ("body_set_type", 60, 2)],
    }
    for call in calls.get(f, ()):
        getattr(world, call[0])(*call[1:])


class _JointCounter:
    """Builder proxy that counts the joints created through it."""

    def __init__(self, b):
        self.b, self.joints = b, 0

    def create_joint(self, d):
        self.joints += 1
        return self.b.create_joint(d)

    def create_revolute(self, d):
        self.joints += 1
        return self.b.create_revolute(d)

    def __getattr__(self, name):
        return getattr(self.b, name)


def build_property_scene(w):
    """Every joint type (weld and distance rigs, prismatic / wheel / motor /
    mouse / filter rigs, revolute gallery) side by side over one ground, a
    small mixed pile and a chain strip, for the property script. Returns
    (bodies, joints)."""
    from forge2d_gb300 import scenes
    c = _JointCounter(w)
    scenes.joint_zoo(c, copies=2)
    scenes.joint_rigs(scenes._PileOffset(c, 0.0, 40.0), copies=2)
    scenes.joint_gallery(scenes._PileOffset(c, 0.0, 80.0), copies=2)
    scenes.pile(scenes._PileOffset(c, 150.0, 0.0), count=120, seed=11, width=20.0, height=30.0)
    ground = w.create_body(scenes.body_def(type=0, positionX=-120.0, positionY=-3.0))
    w.create_chain(ground, [(-20.0, 0.0), (-10.0, -1.0), (0.0, 0.0), (10.0, -1.0), (20.0, 0.0)])
    return len(w.bodies()), c.joints


# codes read back from every joint after the script's edits
JOINT_READS = ("F2D_JP_TYPE", "F2D_JP_LOCAL_ANCHOR_AX", "F2D_JP_LOCAL_ANCHOR_BY", "F2D_JP_SPRING_ENABLED",
               "F2D_JP_SPRING_HERTZ", "F2D_JP_SPRING_DAMPING", "F2D_JP_TARGET", "F2D_JP_LIMIT_ENABLED",
               "F2D_JP_LOWER", "F2D_JP_UPPER", "F2D_JP_MOTOR_ENABLED", "F2D_JP_MOTOR_SPEED", "F2D_JP_MAX_MOTOR",
               "F2D_JP_MOTOR_EFFORT", "F2D_JP_LENGTH", "F2D_JP_MIN_LENGTH", "F2D_JP_MAX_LENGTH", "F2D_JP_CURRENT",
               "F2D_JP_SPEED", "F2D_JP_LINEAR_HERTZ", "F2D_JP_LINEAR_DAMPING", "F2D_JP_ANGULAR_HERTZ",
               "F2D_JP_ANGULAR_DAMPING", "F2D_JP_LINEAR_OFFSET_X", "F2D_JP_LINEAR_OFFSET_Y",
               "F2D_JP_ANGULAR_OFFSET", "F2D_JP_MAX_FORCE", "F2D_JP_MAX_TORQUE", "F2D_JP_CORRECTION",
               "F2D_JP_TARGET_X", "F2D_JP_TARGET_Y")
BODY_READS = ("F2D_BODY_LINEAR_DAMPING", "F2D_BODY_ANGULAR_DAMPING", "F2D_BODY_GRAVITY_SCALE", "F2D_BODY_BULLET",
              "F2D_BODY_FIXED_ROTATION", "F2D_BODY_ENABLED", "F2D_BODY_TYPE", "F2D_BODY_LOCAL_CENTER_X",
              "F2D_BODY_LOCAL_CENTER_Y", "F2D_BODY_WORLD_CENTER_X", "F2D_BODY_WORLD_CENTER_Y")
SHAPE_READS = ("F2D_SHAPE_DENSITY", "F2D_SHAPE_FRICTION", "F2D_SHAPE_RESTITUTION", "F2D_SHAPE_SENSOR",
               "F2D_SHAPE_SENSOR_EVENTS", "F2D_SHAPE_CONTACT_EVENTS", "F2D_SHAPE_HIT_EVENTS",
               "F2D_SHAPE_PRESOLVE_EVENTS", "F2D_SHAPE_CATEGORY", "F2D_SHAPE_MASK", "F2D_SHAPE_GROUP")


def property_reads(world, nb, ns, nj):
    """Every getter code of every body, shape and joint (a flat list)."""
    out = []
    for b in range(nb):
        out += [world.body_get(b, c) for c in BODY_READS]
    for s in range(ns):
        out += [world.shape_get(s, c) for c in SHAPE_READS]
    for j in range(nj):
        out += [world.joint_get(j, c) for c in JOINT_READS]
    return out


def property_script(world, f, nb, nj):
    """Setters of every kind between steps, the same calls on every world:
    joint springs, limits, motors, targets, lengths, offsets and stiffness
    by type; body damping, gravity scale, bullet, fixed rotation and mass
    data; shape friction, restitution, density, event flags and filters;
    chain friction. Bodies are picked among the dynamic ones by index."""
    if f == 20:
        for j in range(nj):
            t = int(world.joint_get(j, "F2D_JP_TYPE"))
            if t == 5:  # revolute
                world.joint_set(j, "F2D_JP_SPRING_ENABLED", 1)
                world.joint_set(j, "F2D_JP_SPRING_HERTZ", 2.5)
                world.joint_set(j, "F2D_JP_SPRING_DAMPING", 0.4)
                world.joint_set(j, "F2D_JP_TARGET", 0.3)
                world.joint_set(j, "F2D_JP_LIMIT_ENABLED", 1)
                world.joint_set(j, "F2D_JP_LOWER", 0.6, -0.4)
            elif t == 4:  # prismatic
                world.joint_set(j, "F2D_JP_SPRING_ENABLED", 1 - world.joint_get(j, "F2D_JP_SPRING_ENABLED"))
                world.joint_set(j, "F2D_JP_SPRING_HERTZ", 2.0)
                world.joint_set(j, "F2D_JP_TARGET", 0.5)
                world.joint_set(j, "F2D_JP_LOWER", -1.0, 2.0)
                world.joint_set(j, "F2D_JP_MOTOR_SPEED", -0.5)
                world.joint_set(j, "F2D_JP_MAX_MOTOR", 40.0)
            elif t == 7:  # wheel
                world.joint_set(j, "F2D_JP_SPRING_HERTZ", 6.0)
                world.joint_set(j, "F2D_JP_SPRING_DAMPING", 0.9)
                world.joint_set(j, "F2D_JP_LOWER", -0.3, 0.2)
                world.joint_set(j, "F2D_JP_MOTOR_SPEED", 3.0)
                world.joint_set(j, "F2D_JP_MAX_MOTOR", 12.0)
            elif t == 0:  # distance
                world.joint_set(j, "F2D_JP_LENGTH", 2.5)
                world.joint_set(j, "F2D_JP_MIN_LENGTH", 3.2, 1.2)
                world.joint_set(j, "F2D_JP_SPRING_ENABLED", 1 - world.joint_get(j, "F2D_JP_SPRING_ENABLED"))
                world.joint_set(j, "F2D_JP_SPRING_HERTZ", 3.0)
                world.joint_set(j, "F2D_JP_MOTOR_SPEED", -1.0)
            elif t == 6:  # weld
                world.joint_set(j, "F2D_JP_LINEAR_HERTZ", 4.0)
                world.joint_set(j, "F2D_JP_LINEAR_DAMPING", 0.3)
                world.joint_set(j, "F2D_JP_ANGULAR_HERTZ", 2.0)
                world.joint_set(j, "F2D_JP_ANGULAR_DAMPING", 0.8)
            elif t == 2:  # motor
                world.joint_set(j, "F2D_JP_LINEAR_OFFSET_X", world.joint_get(j, "F2D_JP_LINEAR_OFFSET_X") - 2.0, 3.0)
                world.joint_set(j, "F2D_JP_ANGULAR_OFFSET", -0.4)
                world.joint_set(j, "F2D_JP_MAX_FORCE", 50.0)
                world.joint_set(j, "F2D_JP_MAX_TORQUE", -5.0)  # clamped to 0
                world.joint_set(j, "F2D_JP_CORRECTION", 1.5)  # clamped to 1
            elif t == 3:  # mouse
                world.joint_set(j, "F2D_JP_SPRING_HERTZ", 3.0)
                world.joint_set(j, "F2D_JP_SPRING_DAMPING", 0.5)
                world.joint_set(j, "F2D_JP_MAX_FORCE", 150.0)
    dyn = [b for b in range(nb) if int(world.body_get(b, "F2D_BODY_TYPE")) == 2]
    if f == 30:
        for j in range(nj):
            t = int(world.joint_get(j, "F2D_JP_TYPE"))
            if t in (4, 5, 7, 0):
                world.joint_set(j, "F2D_JP_MOTOR_ENABLED", 1 - world.joint_get(j, "F2D_JP_MOTOR_ENABLED"))
            if t in (4, 7):
                world.joint_set(j, "F2D_JP_LIMIT_ENABLED", 1 - world.joint_get(j, "F2D_JP_LIMIT_ENABLED"))
        world.body_set(dyn[3], "F2D_BODY_LINEAR_DAMPING", 0.5)
        world.body_set(dyn[4], "F2D_BODY_ANGULAR_DAMPING", 0.3)
        world.body_set(dyn[5], "F2D_BODY_GRAVITY_SCALE", -0.5)
        world.body_set(dyn[6], "F2D_BODY_BULLET", 1)
        world.body_set(dyn[-7], "F2D_BODY_FIXED_ROTATION", 1)
        world.body_set_mass_data(dyn[-9], 4.0, 1.5, 0.1, -0.05)
    if f == 40:
        ns = len(world.shapes()[1])
        pile_shapes = range(ns - 130, ns - 10)
        for k, s in enumerate(pile_shapes):
            if k % 7 == 0:
                world.shape_set(s, "F2D_SHAPE_FRICTION", 0.1)
            if k % 7 == 1:
                world.shape_set(s, "F2D_SHAPE_RESTITUTION", 0.7)
            if k % 7 == 2:
                world.shape_set(s, "F2D_SHAPE_DENSITY", 3.0, 1)
            if k % 7 == 3:
                world.shape_set(s, "F2D_SHAPE_CONTACT_EVENTS", 1)
                world.shape_set(s, "F2D_SHAPE_HIT_EVENTS", 1)
            if k % 7 == 4:
                world.shape_set_filter(s, 2, -1, 0)  # new category: proxy re-created
            if k % 7 == 5:
                world.shape_set_filter(s, 1, ~2, 0)  # mask only: proxy moves
            if k % 7 == 6:
                world.shape_set(s, "F2D_SHAPE_DENSITY", 0.5, 0)
        world.chain_set(0, "F2D_SHAPE_FRICTION", 0.05)
    if f == 60:
        world.body_set(dyn[-7], "F2D_BODY_FIXED_ROTATION", 0)
        world.body_apply_mass_from_shapes(dyn[-9])
        for j in range(nj):
            if int(world.joint_get(j, "F2D_JP_TYPE")) == 5:
                world.joint_set(j, "F2D_JP_LOWER", -0.4, 0.6)  # the same bounds: no change
                world.joint_set(j, "F2D_JP_LIMIT_ENABLED", 0)


def point_answers(world):
    """b2Shape_TestPoint of every third shape at a point near its body's
    origin (the answers, in shape order)."""
    bodies = world.bodies()
    _, sh = world.shapes()
    out = []
    for s in range(0, len(sh), 3):
        b = int(sh[s, 1])
        if b < 0:
            continue
        out.append(world.shape_test_point(s, float(bodies[b, 0]) + 0.25, float(bodies[b, 1]) - 0.1))
    return out


def rounded_scene(w):
    """Rounded boxes and rounded polygons over a rounded ground, for ray
    casts that take the shape-cast path (geometry.c:879-888)."""
    from forge2d_gb300 import scenes
    rng = np.random.default_rng(21)
    ground = w.create_body(scenes.body_def(type=0, positionY=-1.0))
    w.create_box(ground, scenes.shape_def(), 20.0, 0.5, radius=0.25)
    for k in range(48):
        b = w.create_body(scenes.body_def(type=2, positionX=float(rng.uniform(-15, 15)),
                                          positionY=float(rng.uniform(1, 12))))
        r = float(rng.uniform(0.05, 0.3))
        if k % 2 == 0:
            w.create_box(b, scenes.shape_def(), float(rng.uniform(0.2, 0.6)), float(rng.uniform(0.2, 0.6)), radius=r)
        else:
            ang = np.sort(rng.uniform(0, 2 * np.pi, 5))
            pts = [(0.5 * np.cos(a), 0.5 * np.sin(a)) for a in ang]
            w.create_polygon(b, scenes.shape_def(), pts, radius=r)


def rounded_rays(n=200, seed=4):
    rng = np.random.default_rng(seed)
    return [(rng.uniform(-18, 18, 2) + [0.0, 6.0], rng.uniform(-20, 20, 2)) for _ in range(n)]


def multishape_scene(w):
    """Bodies of two or three shapes each over a ground, for explosions whose
    impulses on one body add up over several shapes (the order of the
    dynamic tree's query fixes the sum's last bits)."""
    from forge2d_gb300 import scenes
    rng = np.random.default_rng(12)
    ground = w.create_body(scenes.body_def(type=0, positionY=-1.0))
    w.create_box(ground, scenes.shape_def(), 30.0, 1.0)
    for k in range(90):
        b = w.create_body(scenes.body_def(type=2, positionX=float(rng.uniform(-12, 12)),
                                          positionY=float(rng.uniform(1, 14))))
        w.create_box(b, scenes.shape_def(), 0.35, 0.25)
        w.create_circle(b, scenes.shape_def(density=2.0), 0.4, 0.1, 0.2)
        if k % 2:
            w.create_capsule(b, scenes.shape_def(), -0.3, -0.2, 0.0, -0.4, 0.12)


# frame -> blasts (x, y, radius, falloff, impulse per length, mask) into the
# multi-shape scene: through sleeping sets late, with and without falloff
MULTI_BLASTS = {60: (0.0, 2.0, 4.0, 2.0, 3.0, -1), 150: (5.0, 1.0, 3.0, 0.0, 6.0, -1),
                260: (-4.0, 1.5, 5.0, 3.0, 4.0, 0x1)}
