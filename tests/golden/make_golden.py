"""Generates the golden fixtures in tests/golden/ from the reference itself.

Runs the unmodified Box2D v3.1.1 sources vendored by forge2d (compiled into
oracle/_ref/libbox2d_ref.so by oracle/Makefile) on seeded scenes from
forge2d_gb300/scenes.py and records, per frame, the contact ids the
reference created (so a candidate can reproduce its contact order) and,
at checkpoint frames, every body's position, rotation, linear and angular
velocity and centre of mass, the colour occupancy and a contact dump; for
the full-size workloads, a digest of the bodies and colours of every frame.

Usage: python tests/golden/make_golden.py   (needs the reference checkout)
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from forge2d_gb300 import scenes  # noqa: E402
from oracle.oracle import RefWorld  # noqa: E402
from parity import install_callbacks  # noqa: E402

CASES = {
    "pyramid": dict(world=dict(enableSleep=0), scene=("pyramid", dict()), frames=256, checkpoints=[1, 8, 32, 64, 256]),
    "pile": dict(world=dict(enableSleep=0, enableContinuous=1),
                 scene=("pile", dict(count=300, seed=11, width=30.0, height=40.0)), frames=256,
                 checkpoints=[1, 30, 60, 120, 256]),
    "chains": dict(world=dict(enableSleep=0), scene=("pyramids_chains", dict(pyramids=2, rows=10, chains=6, links=20)),
                   frames=256, checkpoints=[1, 64, 256]),
    "joints": dict(world=dict(enableSleep=0), scene=("joint_gallery", dict()), frames=256,
                   checkpoints=[1, 64, 256]),
    "joint_zoo": dict(world=dict(enableSleep=0), scene=("joint_zoo", dict()), frames=256,
                      checkpoints=[1, 64, 256]),
    "joint_rigs": dict(world=dict(enableSleep=0), scene=("joint_rigs", dict()), frames=256,
                       checkpoints=[1, 64, 256]),
    "joint_rigs_sleep": dict(world=dict(enableSleep=1), scene=("joint_rigs", dict()), frames=300,
                             checkpoints=[1, 100, 200, 300]),
    "chain_terrain": dict(world=dict(enableSleep=0, enableContinuous=0), scene=("chain_terrain", dict(count=300)),
                          frames=256, checkpoints=[1, 64, 256]),
    # custom filter and pre-solve callbacks (tests/parity.py rules)
    "pile_callbacks": dict(world=dict(enableSleep=1, enableContinuous=1),
                           scene=("pile", dict(count=400, seed=6, width=20.0, height=40.0, presolve=True)),
                           frames=300, checkpoints=[1, 100, 200, 300], callbacks=True),
    # sensor events every frame (rows: frame, sensor shape, visitor shape)
    "sensor_field": dict(world=dict(enableSleep=1, enableContinuous=1), scene=("sensor_field", dict()), frames=300,
                         checkpoints=[1, 100, 300], sensors=True),
    # sleeping on: islands, sleeping solver sets, island splits
    "pyramid_sleep": dict(world=dict(enableSleep=1), scene=("pyramid", dict(rows=12)), frames=120,
                          checkpoints=[1, 30, 44, 60, 120]),
    "pile_sleep": dict(world=dict(enableSleep=1, enableContinuous=1),
                       scene=("pile", dict(count=300, seed=3, width=20.0, height=30.0)), frames=360,
                       checkpoints=[1, 100, 250, 300, 360]),
}


# Full-size workloads, recorded as per-frame digests (the states themselves
# would be hundreds of megabytes): the 100k-body mixed pile (its first 60
# frames: free fall, first contacts, the first dense frames) and the 64
# pyramids plus 200 fifty-link chains (10k revolute joints, deep overflow
# colours). The reference runs with a thread pool (its results do not depend
# on the worker count with sleeping off).
DIGEST_CASES = {
    "pile100k": dict(world=dict(enableSleep=0, enableContinuous=1), scene=("pile", dict(count=100_000, seed=1234)),
                     frames=60),
    "stack_chains": dict(world=dict(enableSleep=0), scene=("pyramids_chains", dict()), frames=64),
}


def frame_digest(world):
    """SHA-256 (first 128 bits) of every body row (position, rotation,
    linear and angular velocity, centre of mass) and the colour counts."""
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(world.bodies()[:, :9], np.float32).tobytes())
    h.update(np.ascontiguousarray(world.color_counts(), np.int32).tobytes())
    return h.hexdigest()[:32]


def record_digests(name, spec, workers=8):
    w = RefWorld(scenes.world_def(**spec["world"]), workers=workers)
    scene, kw = spec["scene"]
    scenes.build(w, scene, **kw)
    digests, contacts = [], []
    for _ in range(spec["frames"]):
        w.step(1.0 / 60.0, 4)
        digests.append(frame_digest(w))
        contacts.append(int(len(w.contacts()[0])))
    with open(os.path.join(HERE, name + "_digests_ref.json"), "w") as f:
        json.dump({"world": spec["world"], "scene": scene, "kw": kw, "digests": digests, "contacts": contacts}, f,
                  indent=0)
    w.close()


def record(name, spec):
    w = RefWorld(scenes.world_def(**spec["world"]))
    scene, kw = spec["scene"]
    scenes.build(w, scene, **kw)
    if spec.get("callbacks"):
        install_callbacks(w)
    prev = set()
    plan_rows = []
    out = {}
    sensor_rows = ([], [])
    for f in range(1, spec["frames"] + 1):
        w.step(1.0 / 60.0, 4)
        if spec.get("sensors"):
            for rows, ev in zip(sensor_rows, w.sensor_events()):
                rows.extend((f, int(r[0]), int(r[1])) for r in ev)
        ints, fl = w.contacts()
        cur = set((int(a), int(b), int(c)) for a, b, c in ints[:, :3])
        for row in sorted(cur - prev):
            plan_rows.append((f,) + row)
        prev = cur
        if f in spec["checkpoints"]:
            b = w.bodies()
            out["bodies_%d" % f] = b[:, :9].copy()
            # solver set (0 static, 2 awake, 3.. sleeping set id) and sleep time
            out["sets_%d" % f] = b[:, 10].copy()
            out["sleep_%d" % f] = b[:, 11].copy()
            out["colors_%d" % f] = w.color_counts().copy()
            if f == spec["checkpoints"][0]:
                out["contact_ints_%d" % f] = ints.copy()
                out["contact_floats_%d" % f] = fl.copy()
    out["plan"] = np.array(plan_rows, np.int32).reshape(-1, 4)
    if spec.get("sensors"):
        out["sensor_begin"] = np.array(sensor_rows[0], np.int32).reshape(-1, 3)
        out["sensor_end"] = np.array(sensor_rows[1], np.int32).reshape(-1, 3)
    out["checkpoints"] = np.array(spec["checkpoints"], np.int32)
    np.savez_compressed(os.path.join(HERE, name + "_ref.npz"), **out)
    w.close()


def frame_stats(world, mass):
    """Per-frame max penetration (-min touching separation, 0 if none) and
    kinetic energy sum(0.5 m v^2 + 0.5 I w^2) over dynamic bodies."""
    b = world.bodies()
    m = mass[:, 0].astype(np.float64)
    inertia = mass[:, 1].astype(np.float64)
    v = b[:, 4:6].astype(np.float64)
    w = b[:, 6].astype(np.float64)
    ke = float(np.sum(0.5 * m * (v * v).sum(1) + 0.5 * inertia * w * w))
    ints, fl = world.contacts()
    pen = 0.0
    if len(ints):
        sep = []
        for k in range(2):
            ok = ints[:, 4] > k
            sep.append(fl[ok, 3 + 11 * k + 6])
        s = np.concatenate(sep)
        if len(s):
            pen = float(max(0.0, -s.min()))
    return pen, ke


def record_stats(name, world_kw, scene, kw, frames):
    w = RefWorld(scenes.world_def(**world_kw))
    scenes.build(w, scene, **kw)
    mass = w.mass()
    rows = []
    for _ in range(frames):
        w.step(1.0 / 60.0, 4)
        rows.append(frame_stats(w, mass))
    np.save(os.path.join(HERE, name + "_stats_ref.npy"), np.array(rows, np.float64))
    w.close()


def hull_kats():
    """Convex hull / polygon / mass known answers from the reference create path."""
    rng = np.random.default_rng(5)
    rows = []
    w = RefWorld(scenes.world_def(enableSleep=0))
    for k in range(40):
        n = int(rng.integers(3, 9))
        pts = rng.uniform(-1.0, 1.0, (n, 2)).tolist()
        b = w.create_body(scenes.body_def(type=2, positionX=float(k * 3), positionY=0.0))
        s = w.create_polygon(b, scenes.shape_def(), pts, 0.0)
        poly = w.polygon(s).tolist() if s >= 0 else None
        rows.append({"points": pts, "shape": s, "polygon": poly, "mass": w.mass()[b].tolist()})
    w.close()
    with open(os.path.join(HERE, "hull_ref.json"), "w") as f:
        json.dump(rows, f)


def api_cases():
    """Behaviour cases of forge2d's own tests, measured on the reference:
    box drop (F2D/test/ffi/smoke_test.dart:36-47, world_test.dart:56-74),
    ray cast (events_test.dart:152-167), overlapAabb (:227-240)."""
    res = {}
    # box dropped 10 m onto a 50x1 ground box, 200 steps at 1/60 with 4 substeps
    w = RefWorld(scenes.world_def())
    g = w.create_body(scenes.body_def(type=0, positionY=-1.0))
    w.create_box(g, scenes.shape_def(), 50.0, 1.0)
    b = w.create_body(scenes.body_def(type=2, positionY=10.0))
    w.create_box(b, scenes.shape_def(), 0.5, 0.5)
    for _ in range(200):
        w.step(1.0 / 60.0, 4)
    res["drop"] = {"position": w.bodies()[b][:2].tolist(), "awake_bodies": w.awake_body_count()}
    w.close()
    # ray cast against a box at x=2 from the origin to x=10
    w = RefWorld(scenes.world_def(gravityY=0.0))
    bb = w.create_body(scenes.body_def(type=0, positionX=2.0))
    s = w.create_box(bb, scenes.shape_def(), 0.5, 0.5)
    hit = w.cast_ray_closest(0.0, 0.0, 10.0, 0.0)
    res["ray"] = {"shape": s, "hit": None if hit is None else [hit[0]] + hit[1].tolist()}
    # overlap query: one shape inside the box, one outside
    c1 = w.create_body(scenes.body_def(type=0, positionX=-5.0, positionY=5.0))
    s1 = w.create_circle(c1, scenes.shape_def(), 0.0, 0.0, 0.5)
    c2 = w.create_body(scenes.body_def(type=0, positionX=20.0, positionY=20.0))
    w.create_circle(c2, scenes.shape_def(), 0.0, 0.0, 0.5)
    res["overlap"] = {"inside": s1, "result": sorted(int(x) for x in w.overlap_aabb(-6.0, 4.0, -4.0, 6.0))}
    w.close()
    with open(os.path.join(HERE, "api_ref.json"), "w") as f:
        json.dump(res, f, indent=1)


if __name__ == "__main__":
    only = sys.argv[1:]
    for name, spec in CASES.items():
        if not only or name in only:
            record(name, spec)
    for name, spec in DIGEST_CASES.items():
        if not only or name in only:
            record_digests(name, spec)
    if only:
        sys.exit(0)
    record_stats("pyramid", dict(enableSleep=0), "pyramid", dict(), 256)
    record_stats("pile", dict(enableSleep=0, enableContinuous=1), "pile",
                 dict(count=300, seed=11, width=30.0, height=40.0), 256)
    hull_kats()
    api_cases()
    for fn in sorted(os.listdir(HERE)):
        print(fn, os.path.getsize(os.path.join(HERE, fn)))
