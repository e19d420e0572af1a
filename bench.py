"""Benchmark of the GPU world step: body-steps/s on one GB300.

Workload (default): the 100k-body mixed pile -- 40% circles, 30% capsules,
30% convex polygons from seed 1234, uniform spawn in a 400x800 region above a
static U-shaped container, density 1, friction 0.6, restitution U[0,0.3],
dt=1/60, 4 substeps, sleep off, continuous collision on (synthetic scene
generated by forge2d_gb300/scenes.py; no dataset exists for this metric).

A step is one world step (b2World_Step). Timing: W warm-up steps, then K
steps bracketed by a barrier and torch.cuda.synchronize(); each timed step is
preceded by an untimed 512 MB write that flushes the 129 MB L2, and is timed
with CUDA events recorded by the library on its own launching stream. The
e2e figure times the same steps through the C ABI with host buffers: step,
then read every body's transform into host memory.

--impl reference times the CPU restatement of the reference step (oracle/,
plain C, all host threads it uses) on the same scene and frames; it is the
reference arm because the reference's Box2D sources are not available on
the GPU host.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "body-steps/s on 1 GB300: plain vs batched/learned-warm-start at equal penetration"
HBM_FALLBACK = 6800.0

WORKLOADS = {
    "pile100k": dict(scene="pile", kw=dict(count=100_000, seed=1234), frames=600,
                     desc="100k mixed circles/capsules/polygons (40/30/30), spawn 400x800 above a static U container, "
                          "density 1, friction 0.6, restitution U[0,0.3], dt=1/60, 4 substeps, 600 frames"),
    "pile25k": dict(scene="pile", kw=dict(count=25_000, seed=1234, width=200.0, height=400.0), frames=600,
                    desc="25k-body variant of pile100k (same mix and seed, 200x400 spawn region); the ncu "
                         "capture case of the solver kernel"),
    "pyramid": dict(scene="pyramid", kw=dict(), frames=256,
                    desc="40-row pyramid of 820 unit boxes on a 100x2 static box, dt=1/60, 4 substeps, 256 frames"),
    "pyramids_chains": dict(scene="pyramids_chains", kw=dict(), frames=512,
                            desc="64 pyramids (52,480 boxes) + 200 revolute chains of 50 capsules (10k joints), "
                                 "dt=1/60, 4 substeps, 512 frames"),
}


def timed_frames(total, warmup, steps):
    """The K timed frames, spread evenly over frames warmup..total-1 of the
    scene (every frame when K covers them), so that a short run samples the
    sparse early frames and the dense late ones alike. Frames are numbered
    from 0; the other frames are stepped untimed."""
    span = total - warmup
    if steps >= span:
        return list(range(warmup, warmup + steps))
    if steps == 1:
        return [warmup + span // 2]
    return sorted(set(warmup + round(k * (span - 1) / (steps - 1)) for k in range(steps)))


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return HBM_FALLBACK, "fallback"


def ncu_traffic_ratio(kernel="k_solve", workload="pile25k"):
    """DRAM bytes (read + write) per algorithmic byte of the dominant kernel,
    from the committed ncu summary of a captured launch
    (profiles/<kernel>_<workload>.md, line 'dram_bytes_per_algorithmic_byte: R').
    The capture runs a smaller pile than the bench; the kernel's traffic
    scales with the contacts and bodies it processes, so the bench's
    per-launch traffic is R x its own algorithmic bytes."""
    path = os.path.join(ROOT, "profiles", "%s_%s.md" % (kernel, workload))
    try:
        for line in open(path):
            if line.strip().startswith("dram_bytes_per_algorithmic_byte:"):
                return float(line.split(":", 1)[1].strip())
    except Exception:
        pass
    return None


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=2)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for k, name in enumerate(names):
                if parts[5 + k].lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def solver_bytes(c):
    """Algorithmic bytes of one launch of the persistent solver kernel
    (substeps x {warm start, solve, relax} per touching contact, body
    integration, restitution and impulse storage): per touching contact and
    substep 100 + 24 B warm start, 204 + 52 B solve, 204 + 52 B relax, then
    112 B restitution and 72 B impulse store; per awake body and substep
    56 B velocity and 44 B position integration."""
    sub = 4
    per_contact = sub * (100 + 24 + 204 + 52 + 204 + 52) + 112 + 72
    per_body = sub * (56 + 44)
    return c["touching"] * per_contact + c["awake_bodies"] * per_body


def reduce_over_ranks(ms_total, world, device):
    """The job's timed milliseconds: the maximum over ranks (every replica
    runs the same number of steps, so the slowest rank bounds the job)."""
    if world is None:
        return ms_total, 1
    import torch
    t = torch.tensor([ms_total], dtype=torch.float64, device=device)
    world.all_reduce(t, op=world.ReduceOp.MAX)
    return float(t.item()), world.get_world_size()


def reduce_seconds_over_ranks(seconds, world):
    """Host-clock seconds of the slowest rank."""
    if world is None:
        return seconds
    import torch
    t = torch.tensor([seconds], dtype=torch.float64, device="cuda")
    world.all_reduce(t, op=world.ReduceOp.MAX)
    return float(t.item())


def job_throughput(nranks, bodies_per_rank, steps, ms_total):
    """Body-steps per second of the whole job (weak scaling: every rank
    steps its own replica of the workload)."""
    return nranks * bodies_per_rank * steps / (ms_total * 1e-3)


def run_gpu(args, rank, world):
    import torch

    from forge2d_gb300 import scenes
    from forge2d_gb300.world import GpuWorld

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
    spec = WORKLOADS[args.workload]
    wd = scenes.world_def(enableSleep=1 if args.sleep else 0, enableContinuous=1)
    g = GpuWorld(wd)
    scenes.build(g, spec["scene"], **spec["kw"])
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    frames = timed_frames(spec["frames"], args.warmup, args.steps)
    for _ in range(args.warmup):
        st = g.step(1.0 / 60.0, 4)
    st = g.sync()
    counters = g.counters()
    bodies = counters["awake_bodies"]

    # ---- device-timed value -------------------------------------------
    if world is not None:
        world.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", 0)))
    clocks.start()
    total_ms = 0.0
    status = 0
    launches = 0
    t0 = time.perf_counter()
    torch.cuda.nvtx.range_push("timed_steps")
    frame = args.warmup
    untimed_s = 0.0
    for target in frames:
        if frame < target:
            u0 = time.perf_counter()
            while frame < target:   # untimed frames between two timed ones
                status |= g.step(1.0 / 60.0, 4)
                frame += 1
            status |= g.sync()
            untimed_s += time.perf_counter() - u0
        flush.fill_(1.0)
        torch.cuda.synchronize()
        status |= g.step(1.0 / 60.0, 4)
        status |= g.sync()
        frame += 1
        total_ms += g.last_step_ms()
        launches += g.last_step_launches()
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    wall = time.perf_counter() - t0
    if world is not None:
        world.barrier()
    clk = clocks.stop()
    counters_after = g.counters()

    # ---- e2e through the C ABI with host buffers ----------------------
    # a second copy of the scene steps the same frames (W warm-up, then the
    # K timed ones), each step followed by the read of every body row into
    # a host buffer, timed on the host clock
    import ctypes as C

    import numpy as np

    g2 = GpuWorld(wd)
    scenes.build(g2, spec["scene"], **spec["kw"])
    for _ in range(args.warmup):
        g2.step(1.0 / 60.0, 4)
    g2.sync()
    n = g2.lib.f2d_world_body_capacity(g2.id)
    host = torch.empty((max(n, 1), 12), dtype=torch.float32, pin_memory=True)
    ptr = C.cast(host.data_ptr(), C.POINTER(C.c_float))
    e2e_steps = len(frames)
    rows = 0
    if world is not None:
        world.barrier()
    torch.cuda.synchronize()
    e2e_s = 0.0
    frame = args.warmup
    for target in frames:
        while frame < target:
            status |= g2.lib.f2d_world_step(g2.id, 1.0 / 60.0, 4)
            frame += 1
        status |= g2.sync()
        t1 = time.perf_counter()
        status |= g2.lib.f2d_world_step(g2.id, 1.0 / 60.0, 4)
        rows = g2.lib.f2d_world_get_bodies(g2.id, ptr, n)
        e2e_s += time.perf_counter() - t1
        frame += 1
    status |= g2.sync()
    e2e_s = reduce_seconds_over_ranks(e2e_s, world)
    g2.close()

    # ---- live roofline of the dominant kernel (profiled steps) ---------
    # three more steps of the first world after the timed frames, at the
    # scene's densest state, with per-phase events
    g.set_profiling(True)
    reps = 3
    solve_ms, alg_bytes = [], []
    phases = np.zeros(6)
    rebuild = 0.0
    for _ in range(reps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        g.step(1.0 / 60.0, 4)
        g.sync()
        p = g.phase_ms()
        phases += p
        rebuild += g.rebuild_ms() / reps
        solve_ms.append(p[4])
        alg_bytes.append(solver_bytes(g.counters()))
    g.set_profiling(False)
    phases /= reps
    # latency floor of the solver: its grid barriers x the measured cost of one
    barriers, us_per_barrier = g.solver_latency(2000)
    solve_avg = sum(solve_ms) / len(solve_ms)
    alg = sum(alg_bytes) / len(alg_bytes)
    peak, peak_kind = measured_peaks()
    achieved = alg / (solve_avg * 1e-3) / 1e9 if solve_avg > 0 else None
    ratio = ncu_traffic_ratio()
    traffic = ratio * alg if ratio is not None else None

    # ---- reduce over ranks -------------------------------------------
    ms_total, nranks = reduce_over_ranks(total_ms, world, "cuda")
    value = job_throughput(nranks, bodies, len(frames), ms_total)
    e2e_value = nranks * bodies * e2e_steps / e2e_s
    result = {
        "metric": METRIC,
        "value": value,
        "unit": "body-steps/s",
        "n_gpus": nranks,
        "steps": len(frames),
        "warmup": args.warmup,
        "ms_per_step": ms_total / len(frames),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded scene generator, forge2d_gb300/scenes.py)",
        "config": {"workload": args.workload, "description": spec["desc"], "bodies_per_gpu": bodies,
                   "frames": "%d timed frames spread over frames %d..%d of the scene's %d (first %d, last %d), "
                             "the others stepped untimed" % (len(frames), args.warmup, spec["frames"] - 1,
                                                             spec["frames"], frames[0], frames[-1]),
                   "sleep": bool(args.sleep), "continuous": True, "substeps": 4,
                   "l2": "flushed before every timed step (512 MB write, untimed)",
                   "parallelism": "replicas" if nranks > 1 else "single world",
                   "contacts_live_end": counters_after["contacts"],
                   "touching_end": counters_after["touching"]},
        "e2e": {"value": e2e_value, "unit": "body-steps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": int(rows * 12 * 4),
                "what": "f2d_world_step + f2d_world_get_bodies (every body row: transform, velocities, "
                        "to a pinned host buffer) on a second copy of the scene over the same frames, host clock",
                "steps": len(frames)},
        "roofline": {"kernel": "k_solve (persistent cooperative solver)", "bound": "hbm",
                     "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": (achieved / peak) if achieved else None, "traffic": traffic,
                     "peak_source": peak_kind, "algorithmic_bytes_per_launch": alg,
                     "avg_launch_ms": solve_avg,
                     "traffic_source": "ncu dram bytes per algorithmic byte of a captured pile25k launch "
                                       "(profiles/k_solve_pile25k.md) x this run's algorithmic bytes",
                     "profiled_steps": [{"solve_ms": a, "algorithmic_bytes": b}
                                        for a, b in zip(solve_ms, alg_bytes)],
                     "latency": {"barriers_per_launch": barriers, "us_per_barrier": us_per_barrier,
                                 "floor_ms": barriers * us_per_barrier * 1e-3,
                                 "floor_frac_of_launch": (barriers * us_per_barrier * 1e-3 / solve_avg)
                                 if solve_avg > 0 else None,
                                 "what": "the solver's stages are separated by grid-wide barriers; the floor is "
                                         "their count in the last launch times the cost of one barrier measured "
                                         "by a launch of 2000 bare barriers on the same grid"}},
        "phases_ms": {"broadphase": phases[0], "narrowphase": phases[1], "colouring": phases[2],
                      "solver_setup": phases[3], "solver_kernel": phases[4], "finalize": phases[5],
                      "tree_rebuild_beside": rebuild},
        "gpu_launches": launches,
        "clocks": clk,
        "status": status,
        "wall_s_timed_region": wall,
    }
    forms = {}
    if args.sleep_form:
        forms["sleep_on"] = run_sleep_on(args, torch, frames, flush, bodies)
    if args.batched:
        forms["batched"] = run_batched(args, torch)
    if args.learned:
        forms["learned_warm_start"] = run_learned(args, torch)
    if forms:
        result["forms"] = forms
    if rank == 0 and args.cpu_baseline:
        result["cpu_baseline"] = cpu_baseline(args, bodies_hint=bodies)
    return result, rank


def run_sleep_on(args, torch, frames, flush, bodies):
    """The same workload and frames with sleeping on, forge2d's default
    (islands, sleeping sets and their bookkeeping kept every step): device
    time of the same timed frames, L2 flushed before each."""
    from forge2d_gb300 import scenes
    from forge2d_gb300.world import GpuWorld
    spec = WORKLOADS[args.workload]
    g = GpuWorld(scenes.world_def(enableSleep=1, enableContinuous=1))
    scenes.build(g, spec["scene"], **spec["kw"])
    frame, total_ms, status = 0, 0.0, 0
    for target in frames:
        while frame < target:
            status |= g.step(1.0 / 60.0, 4)
            frame += 1
        status |= g.sync()
        flush.fill_(1.0)
        torch.cuda.synchronize()
        status |= g.step(1.0 / 60.0, 4)
        status |= g.sync()
        frame += 1
        total_ms += g.last_step_ms()
    c = g.counters()
    g.close()
    ms = total_ms / len(frames)
    return {"what": "the main workload with sleeping on (islands and sleeping sets kept on the device), "
                    "the same timed frames; value counts the main line's bodies", "ms_per_step": ms,
            "value": bodies * 1e3 / ms if ms > 0 else None, "unit": "body-steps/s",
            "awake_end": c["awake_bodies"], "status": status}


class _SubRecorder:
    """Builder proxy that records the sub-world of every body it creates."""

    def __init__(self, g):
        self.g = g
        self.body_sub = []
        self.sub = -1

    def begin_subworld(self, gx, gy):
        self.sub = self.g.begin_subworld(gx, gy)
        return self.sub

    def create_body(self, d):
        h = self.g.create_body(d)
        self.body_sub.append(self.sub)
        return h

    def __getattr__(self, name):
        return getattr(self.g, name)


class _PlainBuilder:
    """Builder proxy without sub-worlds (a plain world)."""

    def __init__(self, g):
        self.g = g

    def create_body(self, d):
        return self.g.create_body(d)

    def create_box(self, *a, **k):
        return self.g.create_box(*a, **k)

    def create_circle(self, *a, **k):
        return self.g.create_circle(*a, **k)

    def create_capsule(self, *a, **k):
        return self.g.create_capsule(*a, **k)

    def create_polygon(self, *a, **k):
        return self.g.create_polygon(*a, **k)

    def create_revolute(self, *a, **k):
        return self.g.create_revolute(*a, **k)


def max_penetration(world, group_of_shape=None, groups=0):
    """Max penetration (-min separation of touching manifold points), overall
    or per group of shapes."""
    import numpy as np
    ints, fl = world.contacts()
    if len(ints) == 0:
        return 0.0 if group_of_shape is None else np.zeros(groups)
    sep = np.full(len(ints), np.inf, np.float64)
    for k in range(2):
        ok = ints[:, 4] > k
        sep[ok] = np.minimum(sep[ok], fl[ok, 3 + 11 * k + 6])
    pen = np.maximum(0.0, -sep)
    pen[~np.isfinite(pen)] = 0.0
    if group_of_shape is None:
        return float(pen.max())
    out = np.zeros(groups)
    np.maximum.at(out, group_of_shape[ints[:, 1]], pen)
    return out


def run_batched(args, torch):
    """The batched form: 4096 sub-worlds stepped as one
    world after the autotuner picked the launch shapes, against the same
    worlds stepped one at a time as plain worlds (a seeded sample), at the
    same frame, with max penetration compared."""
    import numpy as np

    from forge2d_gb300 import scenes
    from forge2d_gb300.world import GpuWorld

    worlds, seed = args.batch_worlds, 7
    wd = scenes.world_def(enableSleep=0, enableContinuous=1)
    g = GpuWorld(wd)
    rec = _SubRecorder(g)
    scenes.batched(rec, worlds=worlds, seed=seed)
    body_sub = np.array(rec.body_sub, np.int32)
    _, sh = g.shapes()
    shape_sub = body_sub[sh[:, 1]]
    for _ in range(3):
        g.step(1.0 / 60.0, 4)
    st, chosen, taken = g.autotune(1.0 / 60.0, 4, 2)
    frames = 3 + taken
    # untimed frames up to the config's last ones, then the timed steps
    while frames < args.batch_frames - args.batch_steps:
        st |= g.step(1.0 / 60.0, 4)
        frames += 1
    torch.cuda.synchronize()
    ms = []
    for _ in range(args.batch_steps):
        st |= g.step(1.0 / 60.0, 4)
        st |= g.sync()
        ms.append(g.last_step_ms())
    frames += args.batch_steps
    c = g.counters()
    pen_b = max_penetration(g, shape_sub, worlds)
    bms = float(np.mean(ms))
    g.close()
    # plain: a seeded sample of the same worlds, each its own world
    rng = np.random.default_rng(3)
    sample = sorted(rng.choice(worlds, size=min(args.batch_sample, worlds), replace=False).tolist())
    pms, pen_p = [], []
    for k in sample:
        gx, gy = scenes.batched_gravity(k, worlds, seed)
        p = GpuWorld(scenes.world_def(enableSleep=0, enableContinuous=1, gravityX=gx, gravityY=gy))
        scenes.batched(_PlainBuilder(p), worlds=worlds, seed=seed, only=k)
        t = []
        for f in range(frames):
            p.step(1.0 / 60.0, 4)
            if f >= frames - args.batch_steps:
                p.sync()
                t.append(p.last_step_ms())
        pms.append(float(np.mean(t)))
        pen_p.append(max_penetration(p))
        p.close()
    plain_ws = 1000.0 / float(np.mean(pms))
    batched_ws = worlds * 1000.0 / bms
    return {
        "workload": "%d sub-worlds (pyramids rows U{5..30}, piles of 20-500 mixed shapes, chains of 10-100 "
                    "links; gravity tilted U[-15,15] deg; seed %d), dt=1/60, 4 substeps" % (worlds, seed),
        "worlds": worlds, "bodies": c["awake_bodies"], "touching": c["touching"], "joints": c["joints"],
        "ms_per_step": bms, "world_steps_per_s": batched_ws, "body_steps_per_s": c["awake_bodies"] * 1000.0 / bms,
        "autotune": {"solver_variant": ["auto", "cluster", "grid512", "grid256"][chosen[0]],
                     "leaf_order_period": chosen[1], "tuning_steps": taken},
        "frame": frames, "status": st,
        "plain": {"sample_worlds": len(sample), "ms_per_world_step": float(np.mean(pms)),
                  "world_steps_per_s": plain_ws,
                  "max_penetration_sample": float(np.max(pen_p)),
                  "mean_max_penetration_sample": float(np.mean(pen_p))},
        "max_penetration_batched_sample": float(np.max(pen_b[sample])),
        "mean_max_penetration_batched_sample": float(np.mean(pen_b[sample])),
        "max_penetration_batched_all": float(pen_b.max()),
        "world_steps_ratio_vs_plain": batched_ws / plain_ws,
    }


def kinetic_energy(world, mass):
    import numpy as np
    b = world.bodies()
    m = mass[:, 0].astype(np.float64)
    inertia = mass[:, 1].astype(np.float64)
    v = b[:, 4:6].astype(np.float64)
    w = b[:, 6].astype(np.float64)
    return float(np.sum(0.5 * m * (v * v).sum(1) + 0.5 * inertia * w * w))


def run_learned(args, torch):
    """The learned warm start: samples recorded by the
    plain solver on seeded scenes of configs 2-4, the MLP trained on the GPU,
    then the mixed pile at 200k bodies stepped plain at 4 and 2 substeps
    and with the learned warm start at 2 and 4 substeps: max penetration,
    kinetic-energy drift against plain at 4 substeps, world-steps/s."""
    import numpy as np

    from forge2d_gb300 import scenes
    from forge2d_gb300.world import GpuWorld, WarmStartModel

    wd = scenes.world_def(enableSleep=0, enableContinuous=1)
    t0 = time.perf_counter()
    samples = []
    for name, kw, frames in (("pile", dict(count=20000, seed=21, width=100.0, height=200.0), 240),
                             ("batched", dict(worlds=256, seed=22), 240),
                             ("pyramids_chains", dict(pyramids=4, rows=30, chains=40, links=30), 240)):
        g = GpuWorld(wd)
        scenes.build(g, name, **kw)
        g.set_sample_recording(args.learn_samples)
        for _ in range(frames):
            g.step(1.0 / 60.0, 4)
        samples.append(g.samples())
        g.close()
    samples = np.concatenate(samples)
    rec_s = time.perf_counter() - t0
    model = WarmStartModel(seed=3)
    model.fit_normalization(samples)
    loss0 = model.gradient(samples)[1]
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    loss = model.train(samples, epochs=args.learn_epochs, batch=4096, lr=2e-3)
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t1

    kw = dict(count=args.learn_bodies, seed=1234, width=400.0 * math.sqrt(args.learn_bodies / 1e5),
              height=800.0 * math.sqrt(args.learn_bodies / 1e5))
    runs = {}
    ke_ref = None
    for label, sub, use in (("plain_4", 4, False), ("plain_2", 2, False), ("learned_2", 2, True),
                            ("learned_4", 4, True)):
        g = GpuWorld(wd)
        scenes.build(g, "pile", **kw)
        mass = g.mass()
        if use:
            g.set_warm_start_model(model)
        pens, kes, ms = [], [], []
        for f in range(args.learn_frames):
            g.step(1.0 / 60.0, sub)
            if f % 20 == 19:
                g.sync()
                ms.append(g.last_step_ms())
                pens.append(max_penetration(g))
                kes.append(kinetic_energy(g, mass))
        g.close()
        kes = np.array(kes)
        if ke_ref is None:
            ke_ref = kes
        runs[label] = {"substeps": sub, "ms_per_step": float(np.median(ms)),
                       "world_steps_per_s": 1000.0 / float(np.median(ms)),
                       "mean_max_penetration": float(np.mean(pens)), "max_penetration": float(np.max(pens)),
                       "ke_drift_vs_plain_4": float(np.mean(np.abs(kes - ke_ref) / np.maximum(ke_ref, 1e-9)))}
    model.close()
    return {
        "workload": "mixed pile at %d bodies (seed 1234), %d frames, dt=1/60; samples from a 20k pile, "
                    "256 batched sub-worlds and a pyramids+chains scene (4 substeps, 240 frames each)"
                    % (args.learn_bodies, args.learn_frames),
        "samples": int(len(samples)), "record_s": rec_s, "train_s": train_s, "epochs": args.learn_epochs,
        "loss_initial": float(loss0), "loss_final": float(loss), "network": "MLP 12-64-64-2, BF16 weights, "
        "FP32 accumulation, mma.sync m16n8k16 tensor-core kernels (forward, backward, Adam)",
        "runs": runs,
    }


def cpu_baseline(args, bodies_hint=None, budget_s=None):
    """The CPU restatement on this host's cores, timed on the same frames as
    the GPU arm (the frames between them stepped untimed), stopping early
    if the whole run passes the wall-clock budget."""
    from forge2d_gb300 import scenes
    from oracle.oracle import PortWorld

    spec = WORKLOADS[args.workload]
    wd = scenes.world_def(enableSleep=0, enableContinuous=1)
    p = PortWorld(wd)
    scenes.build(p, spec["scene"], **spec["kw"])
    frames = timed_frames(spec["frames"], args.warmup, args.steps)
    budget = args.cpu_budget if budget_s is None else budget_s
    t_start = time.perf_counter()
    for _ in range(args.warmup):
        p.step(1.0 / 60.0, 4)
    frame, spent, done = args.warmup, 0.0, []
    for target in frames:
        while frame < target:
            p.step(1.0 / 60.0, 4)
            frame += 1
        if time.perf_counter() - t_start > budget:
            break
        spent += p.step_timed(1.0 / 60.0, 4, 1)
        frame += 1
        done.append(target)
    bodies = p.awake_body_count()
    threads = int(os.environ.get("OMP_NUM_THREADS", "0")) or (os.cpu_count() or 1)
    value = bodies * len(done) / spent
    p.close()
    return {"value": value, "unit": "body-steps/s", "cores": port_threads(threads), "kind": "port",
            "calibration": "the port takes 1.20x the reference library's time per frame on this scene "
                           "(same frames, 8 threads each, x86 host with the reference checkout)",
            "sample": "%d timed frames (first %d, last %d) of the %s scene's %d, the frames between them "
                      "stepped untimed; %.1f s of timed CPU step time" % (
                          len(done), done[0], done[-1], args.workload, spec["frames"], spent)}


def port_threads(default):
    try:
        from oracle.oracle import PortWorld  # noqa
        import ctypes
        lib = ctypes.CDLL(os.path.join(ROOT, "oracle", "_build", "libf2d_port.so"))
        fn = getattr(lib, "orc_thread_count", None)
        if fn is None:
            return 1
        fn.restype = ctypes.c_int
        return int(fn())
    except Exception:
        return 1


def run_reference(args, rank):
    if rank != 0:
        return None
    base = cpu_baseline(args, budget_s=args.cpu_budget)
    line = {"metric": METRIC, "value": base["value"], "unit": "body-steps/s", "n_gpus": 0,
            "steps": len(timed_frames(WORKLOADS[args.workload]["frames"], args.warmup, args.steps)),
            "warmup": args.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (seeded scene generator, forge2d_gb300/scenes.py)",
            "config": {"workload": args.workload, "description": WORKLOADS[args.workload]["desc"]},
            "impl": "reference", "cpu_baseline": base,
            "e2e": {"value": base["value"], "unit": "body-steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    return line


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=595)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--workload", default="pile100k", choices=sorted(WORKLOADS))
    ap.add_argument("--cpu-budget", type=float, default=150.0,
                    help="wall-clock seconds after which the CPU arm stops taking timed frames")
    ap.add_argument("--no-cpu-baseline", dest="cpu_baseline", action="store_false")
    ap.add_argument("--sleep", action="store_true",
                    help="create the main workload's worlds with sleeping on (profiling of the island path)")
    ap.add_argument("--no-sleep-form", dest="sleep_form", action="store_false",
                    help="skip the sleeping-on measurement of the main workload")
    ap.add_argument("--no-batched", dest="batched", action="store_false",
                    help="skip the batched form (4096 sub-worlds) beside the headline workload")
    ap.add_argument("--batch-worlds", type=int, default=4096)
    ap.add_argument("--batch-steps", type=int, default=30)
    ap.add_argument("--batch-frames", type=int, default=1000,
                    help="frames the batched form runs (its last batch-steps timed)")
    ap.add_argument("--batch-sample", type=int, default=16)
    ap.add_argument("--no-learned", dest="learned", action="store_false",
                    help="skip the learned warm start (200k pile) beside the headline workload")
    ap.add_argument("--learn-bodies", type=int, default=200_000)
    ap.add_argument("--learn-frames", type=int, default=240)
    ap.add_argument("--learn-epochs", type=int, default=10)
    ap.add_argument("--learn-samples", type=int, default=1_000_000)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3

    rank = int(os.environ.get("RANK", 0))
    wsize = int(os.environ.get("WORLD_SIZE", 1))
    world = None
    if args.impl == "reference":
        line = run_reference(args, rank)
        if line is not None:
            print(json.dumps(line), flush=True)
        return
    if wsize > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("nccl" if args.gpus > 1 else "gloo")
        world = dist
    result, rank = run_gpu(args, rank, world)
    if rank == 0:
        print(json.dumps(result), flush=True)
    if world is not None:
        world.destroy_process_group()


if __name__ == "__main__":
    main()
