"""Seeded synthetic scenes for the benchmark workloads and parity cases.

Each generator drives a *builder* with the flat creation calls that forge2d's
RawBox2D seam exposes (createBody / createBoxShape / createCircleShape /
createCapsuleShape / createPolygonShape / createRevoluteJoint,
packages/forge2d/lib/src/backend/raw_box2d.dart:71-91, :320-385, :~700).
The same generator therefore builds bit-identical scenes in the GPU world
and in any CPU world that offers the same calls: every number is drawn once
as a Python float and rounded to float32 by the callee, as forge2d's FFI
backend does when it fills b2BodyDef / b2ShapeDef.

Scenes:

* ``pyramid``      -- 40-row pyramid of 820 unit boxes on a 100x2 static box.
* ``pile``         -- mixed circles / capsules / convex polygons dropped into a
                      static U-shaped container (the 100k-body pile and its
                      scaled-down parity variants).
* ``pyramids_chains`` -- side-by-side pyramids plus revolute-joint capsule
                      chains hanging from static anchors.
* ``joint_gallery`` -- revolute limits, motors, springs, dynamic-dynamic
                      hinges and collideConnected joints.
* ``batched``      -- thousands of independent sub-worlds (pyramids, piles,
                      chains) with tilted gravity, stepped as one world.
"""
from __future__ import annotations

import math

import numpy as np

WORLD_DEFAULTS = dict(
    gravityX=0.0, gravityY=-10.0, restitutionThreshold=1.0, hitEventThreshold=1.0,
    contactHertz=30.0, contactDampingRatio=10.0, maxContactPushSpeed=3.0,
    maximumLinearSpeed=400.0, enableSleep=1, enableContinuous=1,
)

BODY_DEFAULTS = dict(
    type=0, positionX=0.0, positionY=0.0, rotationCos=1.0, rotationSin=0.0,
    linearVelocityX=0.0, linearVelocityY=0.0, angularVelocity=0.0,
    linearDamping=0.0, angularDamping=0.0, gravityScale=1.0, sleepThreshold=0.05,
    enableSleep=1, isAwake=1, fixedRotation=0, isBullet=0, isEnabled=1,
    allowFastRotation=0,
)

SHAPE_DEFAULTS = dict(
    friction=0.6, restitution=0.0, rollingResistance=0.0, tangentSpeed=0.0,
    density=1.0, categoryBits=1, maskBits=-1, groupIndex=0, userMaterialId=0,
    isSensor=0, enableSensorEvents=0, enableContactEvents=0, enableHitEvents=0,
    enablePreSolveEvents=0, invokeContactCreation=1, updateBodyMass=1,
)

REVOLUTE_DEFAULTS = dict(
    bodyA=0, bodyB=0, localAnchorAX=0.0, localAnchorAY=0.0, localAnchorBX=0.0,
    localAnchorBY=0.0, referenceAngle=0.0, targetAngle=0.0, enableSpring=0,
    hertz=0.0, dampingRatio=0.0, enableLimit=0, lowerAngle=0.0, upperAngle=0.0,
    enableMotor=0, maxMotorTorque=0.0, motorSpeed=0.0, drawSize=0.25,
    collideConnected=0,
)

STATIC, KINEMATIC, DYNAMIC = 0, 1, 2
JOINT_WELD, JOINT_DISTANCE, JOINT_PRISMATIC, JOINT_WHEEL, JOINT_MOTOR, JOINT_MOUSE, JOINT_FILTER = 2, 3, 4, 5, 6, 7, 8

JOINT_DEFAULTS = dict(
    type=JOINT_WELD, bodyA=0, bodyB=0, collideConnected=0,
    localAnchorAX=0.0, localAnchorAY=0.0, localAnchorBX=0.0, localAnchorBY=0.0,
    referenceAngle=0.0, linearHertz=0.0, linearDampingRatio=0.0, angularHertz=0.0, angularDampingRatio=0.0,
    length=1.0, minLength=0.0, maxLength=100000.0, hertz=0.0, dampingRatio=0.0,
    maxMotorForce=0.0, motorSpeed=0.0, enableSpring=0, enableLimit=0, enableMotor=0,
    localAxisAX=1.0, localAxisAY=0.0, targetTranslation=0.0, lowerTranslation=0.0, upperTranslation=0.0,
    maxMotorTorque=0.0, linearOffsetX=0.0, linearOffsetY=0.0, angularOffset=0.0,
    maxForce=1.0, maxTorque=1.0, correctionFactor=0.3, targetX=0.0, targetY=0.0,
)


def joint_def(**kw):
    d = dict(JOINT_DEFAULTS)
    d.update(kw)
    return d


def world_def(**kw):
    d = dict(WORLD_DEFAULTS)
    d.update(kw)
    return d


def body_def(**kw):
    d = dict(BODY_DEFAULTS)
    d.update(kw)
    return d


def shape_def(**kw):
    d = dict(SHAPE_DEFAULTS)
    d.update(kw)
    return d


def revolute_def(**kw):
    d = dict(REVOLUTE_DEFAULTS)
    d.update(kw)
    return d


def pyramid(b, rows=40, x0=None, y0=0.0, ground=True, half=0.5, friction=0.6,
            density=1.0, restitution=0.0, **shape_kw):
    """The 40-row pyramid layout: row r has rows-r boxes, spacing 1.0, offset
    0.5 per row, resting on a static box 100x2 centred at y=-1."""
    ids = []
    if ground:
        g = b.create_body(body_def(type=STATIC, positionX=0.0 if x0 is None else x0 + rows / 2 - 0.5,
                                   positionY=y0 - 1.0))
        b.create_box(g, shape_def(), 50.0, 1.0)
    if x0 is None:
        x0 = -(rows - 1) * 0.5
    sd = shape_def(friction=friction, density=density, restitution=restitution, **shape_kw)
    for r in range(rows):
        for i in range(rows - r):
            body = b.create_body(body_def(type=DYNAMIC, positionX=x0 + 0.5 * r + i,
                                          positionY=y0 + 0.5 + r))
            b.create_box(body, sd, half, half)
            ids.append(body)
    return ids


def _polygon_points(rng, n, radius):
    """n vertices on a jittered circle (angles perturbed, CCW)."""
    base = np.linspace(0.0, 2.0 * math.pi, n, endpoint=False)
    jitter = rng.uniform(-0.3, 0.3, n) * (2.0 * math.pi / n)
    ang = np.sort(base + jitter)
    rad = radius * rng.uniform(0.85, 1.0, n)
    return [(float(rad[k] * math.cos(ang[k])), float(rad[k] * math.sin(ang[k]))) for k in range(n)]


def pile(b, count=100_000, seed=1234, width=400.0, height=800.0, wall_height=None,
         frac_circle=0.4, frac_capsule=0.3, with_container=True, enable_hit_events=False,
         enable_contact_events=False, filters=False, sensor_visitors=False, presolve=False):
    """The mixed pile: ``count`` bodies drawn from ``seed`` -- 40% circles
    r~U[0.25,0.75], 30% capsules (half-length U[0.2,0.8], r U[0.15,0.4]),
    30% convex polygons with 3-8 vertices on a jittered circle r~U[0.3,0.8];
    uniform spawn in a width x height region above a static U-shaped
    container of three boxes; density 1, friction 0.6, restitution U[0,0.3].
    ``filters`` gives the shapes collision filters by index: categories
    1, 2, 4 in turn, every 5th shape's mask excludes the next category,
    every 7th shape is in group -1 (never collides within the group), every
    11th in group 2 (always collides within the group), every 13th is a
    sensor. ``sensor_visitors`` turns on sensor events for three shapes in
    four, in categories 1 and 2 alternately. ``presolve`` turns on pre-solve
    events for every third shape."""
    rng = np.random.default_rng(seed)
    hw = 0.5 * width
    if wall_height is None:
        wall_height = 0.5 * height
    if with_container:
        c = b.create_body(body_def(type=STATIC))
        sd = shape_def()
        b.create_box(c, sd, hw + 5.0, 1.0, 0.0, -1.0, 1.0, 0.0, 0.0)          # floor
        b.create_box(c, sd, 1.0, wall_height, -hw - 1.0, wall_height, 1.0, 0.0, 0.0)  # left wall
        b.create_box(c, sd, 1.0, wall_height, hw + 1.0, wall_height, 1.0, 0.0, 0.0)   # right wall
    kinds = rng.random(count)
    xs = rng.uniform(-hw + 1.0, hw - 1.0, count)
    ys = rng.uniform(1.0, 1.0 + height, count)
    angles = rng.uniform(-math.pi, math.pi, count)
    rest = rng.uniform(0.0, 0.3, count)
    ids = []
    for k in range(count):
        a = float(angles[k])
        body = b.create_body(body_def(type=DYNAMIC, positionX=float(xs[k]), positionY=float(ys[k]),
                                      rotationCos=math.cos(a), rotationSin=math.sin(a)))
        extra = {}
        if filters:
            cat = 1 << (k % 3)
            extra["categoryBits"] = cat
            if k % 5 == 0:
                extra["maskBits"] = -1 ^ (1 << ((k + 1) % 3))
            if k % 7 == 0:
                extra["groupIndex"] = -1
            elif k % 11 == 0:
                extra["groupIndex"] = 2
            if k % 13 == 0:
                extra["isSensor"] = 1
        if presolve:
            extra["enablePreSolveEvents"] = int(k % 3 == 0)
        if sensor_visitors:
            extra["enableSensorEvents"] = int(k % 4 != 0)
            extra["categoryBits"] = 1 << (k % 2)
        sd = shape_def(restitution=float(rest[k]), enableHitEvents=int(enable_hit_events),
                       enableContactEvents=int(enable_contact_events), **extra)
        u = kinds[k]
        if u < frac_circle:
            b.create_circle(body, sd, 0.0, 0.0, float(rng.uniform(0.25, 0.75)))
        elif u < frac_circle + frac_capsule:
            hl = float(rng.uniform(0.2, 0.8))
            r = float(rng.uniform(0.15, 0.4))
            b.create_capsule(body, sd, -hl, 0.0, hl, 0.0, r)
        else:
            n = int(rng.integers(3, 9))
            pts = _polygon_points(rng, n, float(rng.uniform(0.3, 0.8)))
            if b.create_polygon(body, sd, pts, 0.0) == -1:
                b.create_circle(body, sd, 0.0, 0.0, 0.5)
        ids.append(body)
    return ids


def chain(b, anchor_x, anchor_y, links=50, half_length=0.25, radius=0.1, density=1.0):
    """A chain of capsule links hanging from a static anchor by revolute
    joints; the first joint pins link 0 to the anchor body."""
    anchor = b.create_body(body_def(type=STATIC, positionX=anchor_x, positionY=anchor_y))
    sd = shape_def(density=density)
    prev = anchor
    prev_anchor = (0.0, 0.0)
    pitch = 2.0 * half_length
    for k in range(links):
        x = anchor_x + half_length + k * pitch
        body = b.create_body(body_def(type=DYNAMIC, positionX=x, positionY=anchor_y))
        b.create_capsule(body, sd, -half_length, 0.0, half_length, 0.0, radius)
        b.create_revolute(revolute_def(bodyA=prev, bodyB=body, localAnchorAX=prev_anchor[0],
                                       localAnchorAY=prev_anchor[1], localAnchorBX=-half_length,
                                       localAnchorBY=0.0))
        prev = body
        prev_anchor = (half_length, 0.0)
    return anchor


def pyramids_chains(b, pyramids=64, rows=40, chains=200, links=50, gap=2.0):
    """Stacking plus joints: ``pyramids`` copies of the 40-row pyramid side by
    side ``gap`` units apart plus ``chains`` revolute chains of ``links``
    capsule links (half-length 0.25, r 0.1) fixed to static anchors."""
    pitch = rows + gap
    g = b.create_body(body_def(type=STATIC, positionX=0.0, positionY=-1.0))
    total = pyramids * pitch
    b.create_box(g, shape_def(), 0.5 * total + 10.0, 1.0)
    left = -0.5 * total
    for p in range(pyramids):
        pyramid(b, rows=rows, x0=left + p * pitch + 0.5, ground=False)
    span = total / max(chains, 1)
    for c in range(chains):
        chain(b, left + (c + 0.25) * span, rows + 20.0 + 1.0 * (c % 2), links=links)


def joint_gallery(b, copies=4):
    """Revolute features side by side, ``copies`` times: a pendulum held by
    an angle limit, a motor-driven wheel against a torque cap with a box
    resting on it, a spring-loaded arm with a target angle, a two-body
    hinge between dynamic boxes (limit + motor), and a joint with
    collideConnected set, over a ground box."""
    g = b.create_body(body_def(type=STATIC, positionY=-1.0))
    b.create_box(g, shape_def(), 20.0 * copies, 1.0)
    for k in range(copies):
        x0 = -20.0 * copies + 10.0 + 20.0 * k
        # limited pendulum
        anchor = b.create_body(body_def(type=STATIC, positionX=x0, positionY=8.0))
        bob = b.create_body(body_def(type=DYNAMIC, positionX=x0 + 2.0, positionY=8.0))
        b.create_capsule(bob, shape_def(), -1.0, 0.0, 1.0, 0.0, 0.2)
        b.create_revolute(revolute_def(bodyA=anchor, bodyB=bob, localAnchorBX=-2.0, enableLimit=1,
                                       lowerAngle=-0.5 - 0.1 * k, upperAngle=0.25))
        # motor wheel carrying a box
        wheel = b.create_body(body_def(type=DYNAMIC, positionX=x0 + 5.0, positionY=1.0))
        b.create_circle(wheel, shape_def(friction=0.9), 0.0, 0.0, 1.0)
        hub = b.create_body(body_def(type=STATIC, positionX=x0 + 5.0, positionY=1.0))
        b.create_revolute(revolute_def(bodyA=hub, bodyB=wheel, enableMotor=1, motorSpeed=2.0 + k,
                                       maxMotorTorque=50.0))
        load = b.create_body(body_def(type=DYNAMIC, positionX=x0 + 5.0, positionY=2.6))
        b.create_box(load, shape_def(), 0.5, 0.5)
        # spring arm
        base = b.create_body(body_def(type=STATIC, positionX=x0 + 9.0, positionY=4.0))
        arm = b.create_body(body_def(type=DYNAMIC, positionX=x0 + 10.0, positionY=4.0))
        b.create_box(arm, shape_def(), 1.0, 0.1)
        b.create_revolute(revolute_def(bodyA=base, bodyB=arm, localAnchorBX=-1.0, enableSpring=1,
                                       hertz=2.0 + k, dampingRatio=0.3, targetAngle=0.4))
        # dynamic-dynamic hinge with limit and motor, dropping onto the ground
        p = b.create_body(body_def(type=DYNAMIC, positionX=x0 + 13.0, positionY=3.0))
        b.create_box(p, shape_def(), 1.0, 0.25)
        q = b.create_body(body_def(type=DYNAMIC, positionX=x0 + 15.0, positionY=3.0, angularVelocity=1.0))
        b.create_box(q, shape_def(), 1.0, 0.25)
        b.create_revolute(revolute_def(bodyA=p, bodyB=q, localAnchorAX=1.0, localAnchorBX=-1.0, enableLimit=1,
                                       lowerAngle=-1.0, upperAngle=1.0, enableMotor=1, motorSpeed=-1.0,
                                       maxMotorTorque=5.0, referenceAngle=0.1))
        # overlapping bodies that keep colliding through their joint
        r1 = b.create_body(body_def(type=DYNAMIC, positionX=x0 + 17.0, positionY=2.0))
        b.create_box(r1, shape_def(), 0.5, 0.5)
        r2 = b.create_body(body_def(type=DYNAMIC, positionX=x0 + 17.6, positionY=2.0))
        b.create_box(r2, shape_def(), 0.5, 0.5)
        b.create_revolute(revolute_def(bodyA=r1, bodyB=r2, localAnchorAX=0.3, localAnchorBX=-0.3,
                                       collideConnected=1))


def overflow_heap(b, platforms=6, per=24, long_count=160, spokes=16):
    """Bodies with more constraints than the graph has colours: ``platforms``
    dynamic planks each carrying a row of ``per`` circles (r 0.25) with a
    second row on top, one long plank under ``long_count`` circles (one body
    whose overflow contacts form a single long chain), and a hub with
    ``spokes`` revolute spokes (overflow joints), over a static ground."""
    g = b.create_body(body_def(type=STATIC, positionY=-1.0))
    b.create_box(g, shape_def(), 200.0 + 0.5 * long_count, 1.0)
    x = -150.0
    for k in range(platforms):
        hx = 0.25 * per
        plank = b.create_body(body_def(type=DYNAMIC, positionX=x + hx, positionY=0.3))
        b.create_box(plank, shape_def(), hx, 0.25)
        for row in range(2):
            for i in range(per - row):
                c = b.create_body(body_def(type=DYNAMIC, positionX=x + 0.25 + 0.5 * i + 0.25 * row,
                                           positionY=0.8 + 0.45 * row + 0.01 * k))
                b.create_circle(c, shape_def(friction=0.4), 0.0, 0.0, 0.25)
        x += 2.0 * hx + 3.0
    hx = 0.25 * long_count
    plank = b.create_body(body_def(type=DYNAMIC, positionX=x + hx, positionY=0.3))
    b.create_box(plank, shape_def(), hx, 0.25)
    for i in range(long_count):
        c = b.create_body(body_def(type=DYNAMIC, positionX=x + 0.25 + 0.5 * i, positionY=0.8))
        b.create_circle(c, shape_def(), 0.0, 0.0, 0.25)
    x += 2.0 * hx + 5.0
    hub = b.create_body(body_def(type=DYNAMIC, positionX=x, positionY=3.0))
    b.create_circle(hub, shape_def(), 0.0, 0.0, 0.5)
    for k in range(spokes):
        a = 2.0 * math.pi * k / spokes
        sx, sy = x + 1.5 * math.cos(a), 3.0 + 1.5 * math.sin(a)
        s = b.create_body(body_def(type=DYNAMIC, positionX=sx, positionY=sy,
                                   rotationCos=math.cos(a), rotationSin=math.sin(a)))
        b.create_box(s, shape_def(), 0.3, 0.15)
        b.create_revolute(revolute_def(bodyA=hub, bodyB=s, localAnchorBX=-1.5,
                                       enableSpring=1, hertz=4.0, dampingRatio=0.5))


def joint_zoo(b, copies=3):
    """Weld and distance joints side by side, ``copies`` times over a ground
    box: a cantilever of six boxes welded end to end (stiff on even copies,
    soft linear/angular springs on odd ones), a rigid distance pendulum, a
    box hanging on a damped distance spring between length limits, and two
    boxes pushed apart by a distance motor."""
    g = b.create_body(body_def(type=STATIC, positionY=-1.0))
    b.create_box(g, shape_def(), 30.0 * copies, 1.0)
    for k in range(copies):
        x0 = -30.0 * copies + 10.0 + 30.0 * k
        soft = k % 2 == 1
        wall = b.create_body(body_def(type=STATIC, positionX=x0, positionY=6.0))
        b.create_box(wall, shape_def(), 0.25, 1.0)
        prev, prev_x = wall, x0
        for i in range(6):
            x = x0 + 0.75 + 1.0 * i
            seg = b.create_body(body_def(type=DYNAMIC, positionX=x, positionY=6.0))
            b.create_box(seg, shape_def(), 0.5, 0.125)
            b.create_joint(joint_def(type=JOINT_WELD, bodyA=prev, bodyB=seg,
                                     localAnchorAX=0.25 if i == 0 else 0.5, localAnchorBX=-0.5,
                                     linearHertz=5.0 if soft else 0.0, linearDampingRatio=0.7,
                                     angularHertz=3.0 if soft else 0.0, angularDampingRatio=0.5,
                                     referenceAngle=0.05 * k))
            prev, prev_x = seg, x
        anchor = b.create_body(body_def(type=STATIC, positionX=x0 + 10.0, positionY=8.0))
        bob = b.create_body(body_def(type=DYNAMIC, positionX=x0 + 13.0, positionY=8.0))
        b.create_circle(bob, shape_def(), 0.0, 0.0, 0.4)
        b.create_joint(joint_def(type=JOINT_DISTANCE, bodyA=anchor, bodyB=bob, length=3.0))
        hook = b.create_body(body_def(type=STATIC, positionX=x0 + 17.0, positionY=9.0))
        weight = b.create_body(body_def(type=DYNAMIC, positionX=x0 + 17.5, positionY=6.5))
        b.create_box(weight, shape_def(), 0.4, 0.4)
        b.create_joint(joint_def(type=JOINT_DISTANCE, bodyA=hook, bodyB=weight, length=2.0, minLength=1.0,
                                 maxLength=3.5, enableSpring=1, hertz=2.0 + k, dampingRatio=0.3,
                                 enableLimit=1, localAnchorBY=0.3))
        p1 = b.create_body(body_def(type=DYNAMIC, positionX=x0 + 22.0, positionY=1.0))
        b.create_box(p1, shape_def(), 0.5, 0.5)
        p2 = b.create_body(body_def(type=DYNAMIC, positionX=x0 + 24.0, positionY=1.0))
        b.create_box(p2, shape_def(), 0.5, 0.5)
        b.create_joint(joint_def(type=JOINT_DISTANCE, bodyA=p1, bodyB=p2, length=2.0, enableSpring=1,
                                 hertz=0.0, enableMotor=1, maxMotorForce=20.0, motorSpeed=1.0 + k,
                                 enableLimit=1, minLength=1.5, maxLength=4.0))


def chain_terrain(b, count=400, seed=5, width=40.0, height=40.0, bumps=6, materials=None):
    """Chain shapes: a closed loop container (clockwise, so the one-sided
    segments face inwards) with a wavy floor of convex and concave
    vertices, an open bumpy ramp (its end points ghosts only) and the mixed
    pile's shapes (``count`` from ``seed``) dropped on them."""
    g = b.create_body(body_def(type=STATIC))
    hw = 0.5 * width + 1.0
    top = height + 6.0
    pts = [(-hw, top), (hw, top), (hw, 0.0)]
    n = 8 * bumps
    for i in range(1, n):
        x = hw - 2.0 * hw * i / n
        pts.append((x, 0.6 * math.sin(bumps * math.pi * x / hw) + 0.25 * math.cos(3.1 * x)))
    pts.append((-hw, 0.0))
    mats = materials if materials is not None else [(0.6, 0.0, 0.0, 0.0, 0, 0)]
    b.create_chain(g, pts, materials=mats, isLoop=True)
    ramp = [(0.6 * hw + 2.0, 0.45 * top + 3.0)]
    for i in range(7):
        x = 0.6 * hw - 1.2 * hw * i / 6.0
        ramp.append((x, 0.45 * top - 0.25 * (0.6 * hw - x) + 0.4 * math.sin(2.0 * x)))
    ramp.append((-0.6 * hw - 2.0, 0.45 * top - 0.35 * hw - 1.5))
    b.create_chain(g, ramp, materials=[(0.4, 0.1, 0.0, 0.0, 0, 0)], isLoop=False)
    return pile(b, count=count, seed=seed, width=width - 2.0, height=height, with_container=False)


def sensor_field(b, count=300, seed=8, width=30.0, height=40.0):
    """Sensor shapes: four static sensor zones across the container (one
    masks out category 2, one has its events off), a kinematic body sweeping
    a sensor circle through the pile, and a falling box carrying a larger
    sensor circle on its own body; the mixed pile's shapes (``count`` from
    ``seed``) as visitors, three in four with sensor events on."""
    hw = 0.5 * width
    zones = b.create_body(body_def(type=STATIC))
    for i in range(4):
        x = -hw + width * (i + 0.5) / 4.0
        extra = {}
        if i == 1:
            extra["maskBits"] = -1 ^ 2
        b.create_box(zones, shape_def(isSensor=1, enableSensorEvents=int(i != 3), **extra), 2.5, 1.5 + i,
                     x, 4.0 + 2.0 * i, 1.0, 0.0, 0.0)
    sweeper = b.create_body(body_def(type=KINEMATIC, positionX=-hw, positionY=3.0, linearVelocityX=3.0,
                                     angularVelocity=0.5))
    b.create_circle(sweeper, shape_def(isSensor=1, enableSensorEvents=1), 0.0, 0.0, 2.0)
    carrier = b.create_body(body_def(type=DYNAMIC, positionX=0.3, positionY=height + 8.0))
    b.create_box(carrier, shape_def(enableSensorEvents=1), 0.6, 0.6)
    b.create_circle(carrier, shape_def(isSensor=1, enableSensorEvents=1), 0.0, 0.0, 1.8)
    return pile(b, count=count, seed=seed, width=width, height=height, sensor_visitors=True)


def joint_rigs(b, copies=3, motors=None):
    """Prismatic, wheel, motor, mouse and filter joints, ``copies`` times over
    a ground box: an elevator (vertical prismatic with limits and a motor)
    carrying a box, a horizontal prismatic spring, a two-wheeled cart on
    sprung, limited, motored wheel joints, a box led by a motor joint, a box
    held up by a mouse joint, and two overlapping boxes a filter joint keeps
    from colliding. Returns the mouse joints' ids; the ids of the motorised
    joints (lift, wheels) are appended to ``motors`` when given."""
    g = b.create_body(body_def(type=STATIC, positionY=-1.0))
    b.create_box(g, shape_def(), 30.0 * copies, 1.0)
    mice = []
    for k in range(copies):
        x0 = -30.0 * copies + 5.0 + 30.0 * k
        base = b.create_body(body_def(type=STATIC, positionX=x0, positionY=0.5))
        b.create_box(base, shape_def(), 0.2, 0.2)
        lift = b.create_body(body_def(type=DYNAMIC, positionX=x0, positionY=1.0))
        b.create_box(lift, shape_def(), 1.0, 0.1)
        jid = b.create_joint(joint_def(type=JOINT_PRISMATIC, bodyA=base, bodyB=lift, localAnchorAY=0.5,
                                       localAxisAX=0.0, localAxisAY=1.0, enableLimit=1, lowerTranslation=0.0,
                                       upperTranslation=3.0 + k, enableMotor=1, maxMotorForce=60.0,
                                       motorSpeed=1.0 + 0.5 * k))
        if motors is not None:
            motors.append(jid)
        cargo = b.create_body(body_def(type=DYNAMIC, positionX=x0 + 0.2, positionY=1.5))
        b.create_box(cargo, shape_def(), 0.3, 0.3)
        slider = b.create_body(body_def(type=DYNAMIC, positionX=x0 + 4.0, positionY=3.0))
        b.create_box(slider, shape_def(), 0.4, 0.2)
        b.create_joint(joint_def(type=JOINT_PRISMATIC, bodyA=base, bodyB=slider, localAnchorAX=3.0,
                                 localAnchorAY=2.5, localAxisAX=1.0, localAxisAY=0.2 * k, referenceAngle=0.1,
                                 enableSpring=1, hertz=1.5, dampingRatio=0.2, targetTranslation=1.0))
        cx, cy = x0 + 9.0, 1.5
        chassis = b.create_body(body_def(type=DYNAMIC, positionX=cx, positionY=cy))
        b.create_box(chassis, shape_def(), 1.2, 0.25)
        for side in (-1.0, 1.0):
            wheel = b.create_body(body_def(type=DYNAMIC, positionX=cx + 0.9 * side, positionY=cy - 0.6))
            b.create_circle(wheel, shape_def(friction=0.9), 0.0, 0.0, 0.35)
            jid = b.create_joint(joint_def(type=JOINT_WHEEL, bodyA=chassis, bodyB=wheel, localAnchorAX=0.9 * side,
                                           localAnchorAY=-0.6, localAxisAX=0.0, localAxisAY=1.0, enableSpring=1,
                                           hertz=4.0, dampingRatio=0.7, enableLimit=1, lowerTranslation=-0.25,
                                           upperTranslation=0.25, enableMotor=1, maxMotorTorque=8.0,
                                           motorSpeed=-2.0 - k))
            if motors is not None:
                motors.append(jid)
        led = b.create_body(body_def(type=DYNAMIC, positionX=x0 + 15.0, positionY=0.5))
        b.create_box(led, shape_def(), 0.5, 0.5)
        b.create_joint(joint_def(type=JOINT_MOTOR, bodyA=g, bodyB=led, linearOffsetX=x0 + 16.0,
                                 linearOffsetY=4.0, angularOffset=0.5 + 0.2 * k, maxForce=80.0, maxTorque=20.0,
                                 correctionFactor=0.3))
        held = b.create_body(body_def(type=DYNAMIC, positionX=x0 + 20.0, positionY=0.5))
        b.create_box(held, shape_def(), 0.4, 0.6)
        mice.append(b.create_joint(joint_def(type=JOINT_MOUSE, bodyA=g, bodyB=held, targetX=x0 + 20.3,
                                             targetY=3.0, hertz=5.0, dampingRatio=0.7, maxForce=200.0)))
        under = b.create_body(body_def(type=DYNAMIC, positionX=x0 + 25.0, positionY=0.5))
        b.create_box(under, shape_def(), 0.5, 0.5)
        over = b.create_body(body_def(type=DYNAMIC, positionX=x0 + 25.2, positionY=1.2))
        b.create_box(over, shape_def(), 0.5, 0.5)
        b.create_joint(joint_def(type=JOINT_FILTER, bodyA=under, bodyB=over))
    return mice


def batched(b, worlds=4096, seed=7, tile=220.0, columns=64, only=None):
    """The batched scene: ``worlds`` independent sub-worlds of uneven size,
    each drawn from ``seed`` as a pyramid (rows U{5..30}), a random pile
    (20-500 shapes with the mixed pile's shape mix, in a U container sized to the
    count) or a revolute chain (10-100 links), with gravity (0, -10) tilted
    by U[-15, 15] degrees. World k sits in its own ``tile`` x ``tile`` cell of
    a ``columns``-wide grid; sub-worlds never interact even when bodies
    leave their cell. The builder needs ``begin_subworld(gx, gy)``; with
    ``only=k`` just world k is built (same draws), as a plain world when the
    builder has no ``begin_subworld``."""
    rng = np.random.default_rng(seed)
    kinds = rng.integers(0, 3, worlds)
    tilts = np.radians(rng.uniform(-15.0, 15.0, worlds))
    sizes = rng.random(worlds)
    seeds = rng.integers(0, 2 ** 31 - 1, worlds)
    for k in range(worlds):
        if only is not None and k != only:
            continue
        t = float(tilts[k])
        if hasattr(b, "begin_subworld"):
            b.begin_subworld(10.0 * math.sin(t), -10.0 * math.cos(t))
        ox = (k % columns) * tile
        oy = (k // columns) * tile
        if kinds[k] == 0:
            rows = 5 + int(sizes[k] * 26)
            g = b.create_body(body_def(type=STATIC, positionX=ox, positionY=oy - 1.0))
            b.create_box(g, shape_def(), 0.5 * rows + 10.0, 1.0)
            pyramid(b, rows=rows, x0=ox - 0.5 * (rows - 1), y0=oy, ground=False)
        elif kinds[k] == 1:
            n = 20 + int(sizes[k] * 481)
            width = max(8.0, 1.6 * math.sqrt(n))
            height = 2.5 * n / width + 4.0
            w0 = b.create_body(body_def(type=STATIC, positionX=ox, positionY=oy))
            sub = _PileOffset(b, ox, oy)
            pile(sub, count=n, seed=int(seeds[k]), width=width, height=height, with_container=False)
            hw = 0.5 * width
            sd = shape_def()
            b.create_box(w0, sd, hw + 2.0, 1.0, 0.0, -1.0, 1.0, 0.0, 0.0)
            b.create_box(w0, sd, 1.0, height, -hw - 1.0, height, 1.0, 0.0, 0.0)
            b.create_box(w0, sd, 1.0, height, hw + 1.0, height, 1.0, 0.0, 0.0)
        else:
            links = 10 + int(sizes[k] * 91)
            chain(b, ox - 0.25 * links, oy + 0.6 * tile, links=links)


def batched_gravity(k, worlds=4096, seed=7):
    """Gravity of sub-world k of ``batched(worlds=worlds, seed=seed)``."""
    rng = np.random.default_rng(seed)
    rng.integers(0, 3, worlds)
    t = float(np.radians(rng.uniform(-15.0, 15.0, worlds))[k])
    return 10.0 * math.sin(t), -10.0 * math.cos(t)


class _PileOffset:
    """Builder proxy that shifts every body created through it by (ox, oy)."""

    def __init__(self, b, ox, oy):
        self.b, self.ox, self.oy = b, ox, oy

    def create_body(self, d):
        d = dict(d)
        d["positionX"] = d.get("positionX", 0.0) + self.ox
        d["positionY"] = d.get("positionY", 0.0) + self.oy
        return self.b.create_body(d)

    def __getattr__(self, name):
        return getattr(self.b, name)


def build(b, name, **kw):
    if name == "pyramid":
        return pyramid(b, **kw)
    if name == "pile":
        return pile(b, **kw)
    if name == "pyramids_chains":
        return pyramids_chains(b, **kw)
    if name == "joint_gallery":
        return joint_gallery(b, **kw)
    if name == "batched":
        return batched(b, **kw)
    if name == "overflow_heap":
        return overflow_heap(b, **kw)
    if name == "joint_zoo":
        return joint_zoo(b, **kw)
    if name == "joint_rigs":
        return joint_rigs(b, **kw)
    if name == "chain_terrain":
        return chain_terrain(b, **kw)
    if name == "sensor_field":
        return sensor_field(b, **kw)
    raise ValueError(name)
