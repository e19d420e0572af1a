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
