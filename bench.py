#!/usr/bin/env python
"""Benchmark of the GB300 cloth step: cloth vertex-steps/s.

Default workload (the one the metric "batched vs plain" is quoted on): 256
garments in one batch, garment side ~ U{32..256} vertices (a 1 m sheet with the
structural / shear / bend spring lists, k = 2000 / 1000 / 500, two corners pinned),
each over its own icosphere (subdivision ~ U{3..6}, radius ~ U[0.2, 0.4] m, centred
0.5 m below the sheet), seeded synthetic data, timed from the draped state the
sheets reach after `--settle` steps.  A "step" is one pass of the fused step kernel
over every garment (integrate + springs + first-hit collision); the physics uses 4
steps per 1e-3 s frame (at 2 steps the heavier sheets blow up once they touch their
spheres; at 1 the step is linearly unstable).

Reported (one JSON line, rank 0):
  value       batched vertex-steps/s, device-resident inputs, CUDA events on the
              launching stream around K steps (graph replay), max over ranks
  e2e         the same through the C ABI with host buffers: every step uploads the
              pinned-vertex targets from pinned host memory, steps, and reads all
              positions back into pinned host memory (the read of step k overlaps
              steps k + 1 and k + 2; the timed region ends when the last read has
              landed),
              with the host link's own device-to-host rate for the same bytes
              (its ceiling: every step moves all positions over the link)
  plain_loop  the same garments as 256 plain simulators stepped one after another,
              each autotuned on its own draped state (visg_autotune)
  roofline    the fused step kernel: algorithmic bytes per launch / its launch time
              (CUDA events around each launch, 10 steps as one chain after the timed
              region; the same over the whole step is kept beside it)
  cpu_baseline the CPU restatement (OpenMP) on the same garments, bounded sample
  moving_body_configs  the plain configurations whose body moves (LBVH rebuilt
              every step), over their stated durations
  config0_plain  the 64 x 64 sheet over its sphere for its 200 frames, on the GPU
              and, beside it, the CPU restatement on the host cores
  adjoint_config  2,000 FP64 forward steps (0.5 s; checkpoint every 50) + the
              backward sweep on a 128 x 128 sheet with a stiffness per spring
`--impl reference` times the reference's step logic on the host cores (the
oracle port; the reference itself is CUDA only) on the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

PEAKS_FILE = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM = 6800.0
TRAFFIC_FILE = os.path.join(ROOT, "profiles", "fused_step_batched.md")
METRIC = "cloth vertex-steps/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--garments", type=int, default=256)
    ap.add_argument("--substeps", type=int, default=4)
    ap.add_argument("--settle", type=int, default=2400, help="untimed steps before the warm-up (draping)")
    ap.add_argument("--cpu-garments", type=int, default=16, help="garments in the CPU baseline's sample")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--scaling", default="weak", choices=["weak", "strong"],
                    help="weak: every rank its own batch (seed + rank); strong: one batch sharded by vertex count")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain per-garment loop")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--no-moving", action="store_true", help="skip the moving-body plain configs")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the differentiable (adjoint) config")
    ap.add_argument("--moving-only", action="store_true",
                    help="only the moving-body plain configs (one JSON object; for profiling the LBVH rebuild)")
    ap.add_argument("--rebuilds", type=int, default=0,
                    help="only N LBVH rebuilds of the noisy sphere's body, timed (one JSON object; profiling runs)")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--launch", default=None, help="block,ctas_per_sm instead of autotuning (profiling runs)")
    ap.add_argument("--stage", type=int, default=None, help="stage_neighbours with --launch (profiling runs)")
    ap.add_argument("--chains", type=int, default=2, choices=[1, 2],
                    help="step chains per step: 2 overlapping garment groups (default) or 1 (profiling runs)")
    return ap.parse_args()


# ---------------------------------------------------------------------------------------
def build_workload(n_garments: int, seed: int):
    from simulator_gb300 import scenes
    items = scenes.garment_batch(n_garments, seed=seed)
    nv = sum(len(c.xyz) for c, _ in items)
    ne = sum(sum(sl.n_entries for sl in c.lists) for c, _ in items)
    nt = sum(len(b.tris) for _, b in items)
    return items, nv, ne, nt


def workload_name(args):
    return (f"batched: {args.garments} garments, side ~ U{{32..256}} (1 m sheet, structural/shear/bend lists, "
            f"2 corners pinned), own icosphere subdiv ~ U{{3..6}}, r ~ U[0.2,0.4] m centred 0.5 m below; "
            f"{args.substeps} steps per 1e-3 s frame; timed from the draped state after {args.settle} steps")


def peak_hbm():
    try:
        with open(PEAKS_FILE) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM, "fallback"


STEP_SOURCES = [os.path.join(ROOT, "simulator_gb300", "csrc", f)
                for f in ("visg_step.cu", "visg_math.cuh", "visg_internal.cuh")]


def step_kernel_build():
    """Identity of the fused step kernel's source: the first 16 hex digits of the
    SHA-256 of the files it is compiled from."""
    import hashlib
    h = hashlib.sha256()
    for f in STEP_SOURCES:
        with open(f, "rb") as fh:
            h.update(fh.read())
    return h.hexdigest()[:16]


def committed_traffic():
    """DRAM bytes of the fused step kernel per step (all its launches) from the
    committed ncu summary, with where they come from.  The summary records the
    kernel build it was captured on; a figure captured on another build is not
    reported (traffic None, and the provenance says why)."""
    try:
        text = open(TRAFFIC_FILE).read()
    except OSError:
        return None, {"file": os.path.relpath(TRAFFIC_FILE, ROOT), "note": "missing"}
    fields = dict(re.findall(r"^(traffic_[a-z_]+):\s*(.+?)\s*$", text, re.M))
    src = {"file": os.path.relpath(TRAFFIC_FILE, ROOT), "captured_on": fields.get("traffic_capture"),
           "scale": fields.get("traffic_scale"), "kernel_build": fields.get("traffic_build"),
           "current_build": step_kernel_build()}
    if "traffic_bytes_per_step" not in fields:
        src["note"] = "no figure in the summary"
        return None, src
    if src["kernel_build"] != src["current_build"]:
        src["note"] = "stale: captured on another build of the step kernel, not reported"
        return None, src
    return float(fields["traffic_bytes_per_step"]), src


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms in the background."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,utilization.gpu,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []
        self.t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(self.index)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        if self.t:
            self.t.join(timeout=2)
        rows = []
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 10:
                continue
            try:
                rows.append(dict(sm=float(f[1]), smax=float(f[2]), util=float(f[4]), hw=f[6], hwt=f[7], swt=f[8],
                                 pcap=f[9]))
            except ValueError:
                continue
        if not rows:
            return None
        load = [r for r in rows if r["util"] >= 50.0] or rows
        reasons = set()
        for r in load:
            if r["hw"] == "Active":
                reasons.add("hw_slowdown")
            if r["hwt"] == "Active":
                reasons.add("hw_thermal_slowdown")
            if r["swt"] == "Active":
                reasons.add("sw_thermal_slowdown")
            if r["pcap"] == "Active":
                reasons.add("sw_power_cap")
        return {"sm_mhz": statistics.median(r["sm"] for r in load), "sm_max_mhz": max(r["smax"] for r in rows),
                "reasons": sorted(reasons), "samples": len(rows), "samples_under_load": len(load)}


def cpu_baseline(items, params, seconds: float, states=None, settle: int = 0):
    """The oracle (the reference's step restated in C++, float, OpenMP over the
    vertices of each garment) stepping a sample of the same garments from the same
    draped state: `states` (x, x_old, normal per garment) when given, else reached by
    stepping the oracle `settle` times (its trajectory is bit-identical to the GPU's)."""
    from oracle.ffi import OracleSim, num_threads
    threads = num_threads(0)
    sims = [OracleSim(params, c.xyz, c.lists, b.xyz, b.tris, b.normals, prec=4, pinned=c.pinned) for c, b in items]
    nv = sum(s.n for s in sims)
    for k, s in enumerate(sims):
        if states is not None:
            s.set_state(*states[k])
        elif settle:
            s.step(settle)
    for s in sims:  # one untimed step
        s.step(1)
    steps = 0
    t0 = time.perf_counter()
    while True:
        for s in sims:
            s.step(1)
        steps += 1
        el = time.perf_counter() - t0
        if el >= seconds or steps >= 100000:
            break
    for s in sims:
        s.close()
    return {"value": nv * steps / el, "unit": "vertex-steps/s", "cores": threads, "kind": "port",
            "sample": f"the first {len(items)} garments ({nv} vertices) from the draped state, {steps} steps "
                      f"({el:.1f} s), {threads} OpenMP threads; the rate per vertex-step of this sample stands "
                      f"for the whole batch (extrapolated: the sample's mix of garment sizes is not the batch's)"}


def config0_plain(vs, scenes, torch, params, stream, substeps: int, cpu: bool):
    """The smallest plain workload: a 64 x 64 sheet (1 m, two corners pinned) over an
    icosphere of subdivision 4 (radius 0.3 m) centred 0.5 m below, its stated 200
    frames (`substeps` steps each) from the initial state.  The simulator is
    autotuned first (visg_autotune, state unchanged).  The GPU runs the frames as one
    simulate call (graph replay; CUDA events on the launching stream), then again
    from the same initial state for a second timing; with `cpu`, the oracle (float,
    OpenMP) runs the same steps on the host cores for the CPU row beside it."""
    cloth, body = scenes.sheet_over_sphere(64, 4)
    n, steps = len(cloth.xyz), 200 * substeps
    sim = vs.Simulator(cloth.xyz, cloth.lists, body.xyz, body.tris, body.normals, params=params,
                       pinned=cloth.pinned)
    sim.set_stream(stream.cuda_stream)
    sim.autotune()
    zero = np.zeros_like(cloth.xyz)
    sim.simulate(steps)  # warm: graph capture, first launches
    times = []
    for _ in range(2):
        sim.set_state(cloth.xyz, cloth.xyz, zero)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        sim.simulate(steps)
        e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    ms = min(times)
    out = {"vertices": n, "spring_entries": int(sum(sl.n_entries for sl in cloth.lists)),
           "triangles": int(len(body.tris)), "frames": 200, "steps": steps,
           "gpu": {"value": n * steps / (ms / 1e3), "unit": "vertex-steps/s", "ms_per_step": ms / steps,
                   "how": "one simulate call of all steps (graph replay), best of 2 from the initial state"},
           "contacts_at_end": sim.count_contacts(), "launch": sim.launch_info()}
    sim.close()
    if cpu:
        from oracle.ffi import OracleSim, num_threads
        o = OracleSim(params, cloth.xyz, cloth.lists, body.xyz, body.tris, body.normals, prec=4,
                      pinned=cloth.pinned)
        t0 = time.perf_counter()
        o.step(steps)
        el = time.perf_counter() - t0
        o.close()
        out["cpu"] = {"value": n * steps / el, "unit": "vertex-steps/s", "cores": num_threads(0), "kind": "port",
                      "seconds": el, "sample": "the same steps from the same initial state"}
    return out


def moving_body_configs(vs, scenes, torch, params, stream, steps: int, warmup: int, substeps: int = 4):
    """The plain single-garment workloads whose body moves (LBVH rebuilt every step),
    each over its stated duration (1,000 frames for the capsules, 500 for the sphere,
    `substeps` steps per frame), from the initial state: the sheet falls, meets the
    moving body and drapes over it.  Per step the body's positions (precomputed on the
    device) go in through update_body_device, then one step runs.  Then `steps` more
    steps with the body held still show the rebuild's share.  Each simulator is
    autotuned when created (visg_autotune, state unchanged)."""
    out = {}
    for name, make, frames in (("garment_over_capsules", scenes.garment_over_capsules, 1000),
                               ("sheet_over_noisy_sphere", scenes.sheet_over_noisy_sphere, 500)):
        cloth, body, motion = make(0)
        n = len(cloth.xyz)
        sim = vs.Simulator(cloth.xyz, cloth.lists, body.xyz, body.tris, body.normals, params=params,
                           pinned=cloth.pinned)
        sim.set_stream(stream.cuda_stream)
        sim.autotune()
        timed = frames * substeps
        total = warmup + timed
        offs = np.stack([motion(k * params.dt) for k in range(total)]).astype(np.float32)
        d_base = torch.from_numpy(np.ascontiguousarray(body.xyz, np.float32)).cuda()
        d_frames = (d_base[None] + torch.from_numpy(offs).cuda()[:, None, :]).contiguous()
        d_nrm = torch.from_numpy(np.ascontiguousarray(body.normals, np.float32)).cuda()
        fb = d_frames.element_size() * d_base.numel()

        def run(k0, k, move):
            for j in range(k0, k0 + k):
                if move:
                    sim.update_body_device(d_frames.data_ptr() + j * fb, d_nrm.data_ptr())
                sim.simulate(1)

        run(0, warmup, True)
        torch.cuda.synchronize()
        e = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        e[0].record(stream)
        run(warmup, timed, True)
        e[1].record(stream)
        torch.cuda.synchronize()
        contacts = sim.count_contacts()
        e[2].record(stream)
        run(0, steps, False)
        e[3].record(stream)
        torch.cuda.synchronize()
        ms_move = e[0].elapsed_time(e[1]) / timed
        ms_still = e[2].elapsed_time(e[3]) / steps
        out[name] = {"vertices": n, "spring_entries": int(sum(sl.n_entries for sl in cloth.lists)),
                     "triangles": int(len(body.tris)), "frames": frames, "steps": timed,
                     "value": n / (ms_move / 1e3), "unit": "vertex-steps/s", "ms_per_step": ms_move,
                     "ms_per_step_body_still": ms_still, "lbvh_rebuild_ms": ms_move - ms_still,
                     "contacts_at_end": contacts, "launch": sim.launch_info()}
        del d_frames
        sim.close()
    return out


def rebuilds_only(vs, scenes, torch, params, n: int):
    """The LBVH rebuild alone: the 327,680-triangle noisy sphere moved along its
    1 Hz oscillation and rebuilt `n` times (update_body_device with positions already
    on the device), after 3 untimed rebuilds; CUDA events around the n calls.  The
    launches are the creation's build, 3 warm-up builds, then the n timed ones."""
    cloth, body, motion = scenes.sheet_over_noisy_sphere(0)
    sim = vs.Simulator(cloth.xyz, cloth.lists, body.xyz, body.tris, body.normals, params=params,
                       pinned=cloth.pinned)
    stream = torch.cuda.current_stream()
    sim.set_stream(stream.cuda_stream)
    total = 3 + n
    offs = np.stack([motion((k + 1) * params.dt) for k in range(total)]).astype(np.float32)
    d_base = torch.from_numpy(np.ascontiguousarray(body.xyz, np.float32)).cuda()
    d_frames = (d_base[None] + torch.from_numpy(offs).cuda()[:, None, :]).contiguous()
    d_nrm = torch.from_numpy(np.ascontiguousarray(body.normals, np.float32)).cuda()
    fb = d_frames.element_size() * d_base.numel()
    for j in range(3):
        sim.update_body_device(d_frames.data_ptr() + j * fb, d_nrm.data_ptr())
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for j in range(3, total):
        sim.update_body_device(d_frames.data_ptr() + j * fb, d_nrm.data_ptr())
    e1.record(stream)
    torch.cuda.synchronize()
    out = {"triangles": int(len(body.tris)), "rebuilds": n, "ms_per_rebuild": e0.elapsed_time(e1) / n,
           "leaves": sim.info()["n_leaves"]}
    sim.close()
    return out


def adjoint_config(vs, scenes, torch):
    """The differentiable configuration: a 128 x 128 sheet (16,384 vertices) with a
    stiffness per spring (the three lists' k as per-entry arrays) over the 64 x 64
    workload's sphere (radius 0.3 m, subdivision 4, centre 0.5 m below), its stated
    0.5 s as 2,000 FP64 forward steps of 2.5e-4 s (4 per 1e-3 s frame, as the other
    workloads) with a checkpoint every 50, then the backward sweep (the gradient of a
    mean squared final-position error for every spring's stiffness and the three
    damping scalars).  Host wall-clock around each call (both synchronise).  The
    forward pass's frozen active set is reported: vertices projected in every 200th
    step, and the steps that had any."""
    cloth = scenes.grid_cloth(128, 1.0, 0.0)
    body = scenes.icosphere(4, 0.3, center=(0.0, -0.5, 0.0))
    p = scenes.physics_params(4)
    lists = [scenes.SpringList(sl.row, sl.ent, np.full(sl.n_entries, k, np.float32))
             for sl, k in zip(cloth.lists, (2000.0, 1000.0, 500.0))]
    sim = vs.Simulator(cloth.xyz, lists, body.xyz, body.tris, body.normals, params=p, pinned=cloth.pinned)
    steps, ckpt = 2000, 50
    sim.forward(steps, ckpt)  # warm: allocations, first launches
    sim.backward(np.zeros_like(cloth.xyz))
    sim.set_state(cloth.xyz, cloth.xyz, np.zeros_like(cloth.xyz))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sim.forward(steps, ckpt)
    t1 = time.perf_counter()
    active = sim.forward_contacts()
    x = sim.positions()
    target = cloth.xyz + np.float32(0.005)
    dk, ds = sim.backward((2.0 * (x - target) / len(x)).astype(np.float32))
    t2 = time.perf_counter()
    n = len(cloth.xyz)
    out = {"vertices": n, "spring_entries": int(sum(sl.n_entries for sl in lists)), "steps": steps,
           "seconds_simulated": steps * p.dt, "checkpoint_every": ckpt, "forward_ms": (t1 - t0) * 1e3,
           "backward_ms": (t2 - t1) * 1e3, "value": n * steps / (t2 - t0),
           "unit": "vertex-steps/s (forward + backward)", "grad_max_abs": float(np.abs(dk).max()),
           "grad_finite": bool(np.isfinite(dk).all()), "contacts_at_end": sim.count_contacts(),
           "active_set_every_200_steps": [int(c) for c in active[199::200]],
           "steps_with_contacts": int((active > 0).sum()), "max_contacts_in_a_step": int(active.max())}
    sim.close()
    return out


# ---------------------------------------------------------------------------------------
def run_reference(args, rank):
    if rank != 0:
        return 0
    from simulator_gb300 import scenes
    items, nv, ne, nt = build_workload(args.garments, args.seed)
    params = scenes.physics_params(args.substeps)
    base = cpu_baseline(items[:args.cpu_garments], params, args.cpu_seconds, settle=args.settle)
    line = {
        "impl": "reference", "metric": METRIC, "value": base["value"], "unit": "vertex-steps/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": workload_name(args), "garments": args.garments, "substeps": args.substeps,
                   "vertices": nv, "spring_entries": ne, "triangles": nt,
                   "timed_sample": f"the first {args.cpu_garments} garments; the rate is extrapolated to the batch"},
        "cpu_baseline": base,
        "e2e": {"value": base["value"], "unit": "vertex-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, rank)

    import torch
    import simulator_gb300 as vs
    from simulator_gb300 import scenes

    from simulator_gb300.shards import RankGroup, my_shard

    torch.cuda.set_device(local)
    group = RankGroup("nccl", device=torch.device("cuda", local))
    barrier, max_over_ranks = group.barrier, group.max

    vis = os.environ.get("CUDA_VISIBLE_DEVICES")
    phys = int(vis.split(",")[local]) if vis and vis.split(",")[local].strip().isdigit() else local
    sampler = ClockSampler(phys)

    params = scenes.physics_params(args.substeps)
    if args.rebuilds:
        print(json.dumps({"lbvh_rebuilds": rebuilds_only(vs, scenes, torch, params, args.rebuilds)}), flush=True)
        return 0
    if args.moving_only:
        out = moving_body_configs(vs, scenes, torch, params, torch.cuda.current_stream(), args.steps, args.warmup,
                                  args.substeps)
        print(json.dumps({"moving_body_configs": out}), flush=True)
        return 0
    if args.stage is not None:
        params.stage_neighbours = args.stage
    params.overlap_groups = 0 if args.chains == 2 else 1
    if args.scaling == "strong":  # one batch, sharded by vertex count
        items, _, _, _ = build_workload(args.garments, args.seed)
        lo, hi = my_shard([len(c.xyz) for c, _ in items], rank, world)
        items = items[lo:hi]
        nv = sum(len(c.xyz) for c, _ in items)
        ne = sum(sum(sl.n_entries for sl in c.lists) for c, _ in items)
        nt = sum(len(b.tris) for _, b in items)
    else:  # every rank its own batch
        items, nv, ne, nt = build_workload(args.garments, args.seed + rank)
    nv_all = group.sum(nv)  # vertices stepped by all ranks
    stream = torch.cuda.current_stream()
    sh = stream.cuda_stream

    b = vs.BatchSimulator(params)
    pins = []
    off = 0
    for cloth, body in items:
        b.add(cloth.xyz, cloth.lists, body.xyz, body.tris, body.normals, pinned=cloth.pinned)
        pins.append(cloth.pinned.astype(np.int64) + off)
        off += len(cloth.xyz)
    b.finalize()
    b.set_stream(sh)
    pins = np.concatenate(pins).astype(np.uint32)
    pin_xyz0 = np.concatenate([c.xyz[c.pinned] for c, _ in items]).astype(np.float32)
    b.step(args.settle)  # drape the sheets over their spheres (untimed)
    if args.launch:
        b.set_launch(*(int(v) for v in args.launch.split(",")))
    elif not args.no_autotune:
        b.autotune()
    launch = b.launch_info()

    sampler.start()
    # ---- device-resident value: K steps replayed from CUDA graphs --------------------
    b.step(args.warmup)
    torch.cuda.synchronize()
    barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    b.step(args.steps)
    e1.record(stream)
    torch.cuda.synchronize()
    barrier()
    ms = max_over_ranks(e0.elapsed_time(e1))
    value = nv_all * args.steps / (ms / 1e3)
    contacts = b.count_contacts()
    # the roofline kernel's own launch time: 10 more steps as one chain (each launch
    # over the whole batch), CUDA events right around each launch on its stream
    k_step_ms, k_collide_ms = b.time_kernels(10)

    # ---- end to end through the C ABI with host buffers --------------------------------
    # three page-locked result buffers: step k's positions are copied to host memory
    # while steps k + 1 and k + 2 are issued and run (read_positions_async /
    # wait_positions, up to three reads in flight)
    outs = [torch.empty((nv, 3), dtype=torch.float32, pin_memory=True).numpy() for _ in range(3)]
    pin_host = torch.empty((len(pins), 3), dtype=torch.float32, pin_memory=True).numpy()
    k_e2e = max(1, min(args.steps, 50))
    for k in range(3):  # warm the staging buffers
        b.update_vertices(pins, pin_xyz0)
        b.step(1)
        b.read_positions_async(outs[k])
        b.wait_positions()
    torch.cuda.synchronize()
    barrier()
    t0 = time.perf_counter()
    for k in range(k_e2e):
        pin_host[:] = pin_xyz0  # the step's host input: pinned-vertex targets
        b.update_vertices(pins, pin_host)
        b.step(1)
        b.read_positions_async(outs[k % 3])  # the step's result, copied behind the next steps
        if k > 1:
            b.wait_positions()  # step k - 2's positions are in host memory
    for _ in range(min(2, k_e2e)):
        b.wait_positions()
    e2e_s = max_over_ranks(time.perf_counter() - t0)
    e2e_value = nv_all * k_e2e / e2e_s
    h2d = len(pins) * (4 + 12)
    d2h = nv * 12
    # the host link's own device-to-host rate for the same bytes (plain copies into
    # the same page-locked buffer): the end-to-end loop's ceiling
    src = torch.empty(nv * 3, dtype=torch.float32, device="cuda")
    dst = torch.from_numpy(outs[0].reshape(-1))
    for _ in range(2):
        dst.copy_(src, non_blocking=True)
    torch.cuda.synchronize()
    l0, l1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    l0.record()
    for _ in range(10):
        dst.copy_(src, non_blocking=True)
    l1.record()
    torch.cuda.synchronize()
    link_gbs = 10 * d2h / (l0.elapsed_time(l1) / 1e3) / 1e9
    del src
    d2h_gbs = d2h * k_e2e / e2e_s / 1e9

    # ---- the plain per-garment loop on the same GPU ------------------------------------
    plain = None
    if not args.no_plain:
        sims = []
        for g, (cloth, body) in enumerate(items):
            s = vs.Simulator(cloth.xyz, cloth.lists, body.xyz, body.tris, body.normals, params=params,
                             pinned=cloth.pinned)
            s.set_state(*b.state(g))  # the batch's draped state
            s.set_stream(sh)
            s.autotune()  # each plain simulator at its own best launch shape and variant
            sims.append(s)
        for s in sims:
            s.simulate(args.warmup)
        torch.cuda.synchronize()
        p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        p0.record(stream)
        for s in sims:
            s.simulate(args.steps)
        p1.record(stream)
        torch.cuda.synchronize()
        pms = max_over_ranks(p0.elapsed_time(p1))
        split_n = sum(s.launch_info()["split_collision"] for s in sims)
        plain = {"value": nv_all * args.steps / (pms / 1e3), "ms_per_step": pms / args.steps,
                 "how": "each garment its own Simulator, autotuned on its draped state, stepped K steps "
                        "(graph replay) one garment after another",
                 "autotuned_split_collision": f"{split_n} of {len(sims)}"}
        for s in sims:
            s.close()
    moving = config0 = None
    if rank == 0 and not args.no_moving:
        moving = moving_body_configs(vs, scenes, torch, params, stream, 100, 10, args.substeps)
        config0 = config0_plain(vs, scenes, torch, params, stream, args.substeps, cpu=world == 1 and not args.no_cpu)
    adjoint = None
    if rank == 0 and not args.no_adjoint:
        adjoint = adjoint_config(vs, scenes, torch)
    clocks = sampler.stop()

    # ---- roofline of the fused step kernel ---------------------------------------------
    # the per-unit figure B_int = 72 N + 4 (N+1) L + s E with one merged row
    # list (L = 1) and 8-byte entries (s = 8): x, x_old, normal read and written as
    # 12-byte vectors, the row offset, and one entry per directed spring
    alg_bytes = 72 * nv + 4 * (nv + 1) + 8 * ne
    t_launch = k_step_ms / 1e3
    achieved = alg_bytes / t_launch / 1e9
    achieved_step = alg_bytes / (ms / 1e3 / args.steps) / 1e9  # over the whole step (both kernels)
    peak, peak_kind = peak_hbm()
    traffic, traffic_source = committed_traffic()

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        ncpu = min(args.cpu_garments, len(items))
        cpu = cpu_baseline(items[:ncpu], params, args.cpu_seconds, states=[b.state(g) for g in range(ncpu)])

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "vertex-steps/s", "n_gpus": world, "steps": args.steps,
            "value_per_frame": {"value": value / args.substeps, "unit": "vertex-frames/s",
                                "frame": f"1e-3 s (the configurations' time step) = {args.substeps} steps"},
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": args.scaling,
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": workload_name(args), "garments": args.garments, "substeps": args.substeps,
                       "vertices_per_gpu": nv,
                       "vertices_all_gpus": int(nv_all),
                       "spring_entries": ne, "triangles": nt, "contacts": contacts,
                       "launch": launch,
                       "l2": f"inputs larger than L2: {alg_bytes / 1e6:.0f} MB moved per step vs 129 MB L2",
                       "parallelism": (f"{world} independent batches (one per GPU)" if args.scaling == "weak"
                                       else f"one batch in {world} shards by vertex count (one per GPU)")},
            "e2e": {"value": e2e_value, "unit": "vertex-steps/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "steps": k_e2e, "d2h_gbs": d2h_gbs,
                    "link_d2h_gbs_measured": link_gbs, "frac_of_link": d2h_gbs / link_gbs},
            "plain_loop": plain,
            "batched_vs_plain": (value / plain["value"]) if plain else None,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "traffic_source": traffic_source,
                         "peak_source": peak_kind,
                         "kernel": "k_step (fused integrate + springs + collision)",
                         "launch_note": ("launch_ms is the step kernel's own launch over the whole batch on "
                                         "every SM (one chain); inside the timed two-chain step each launch "
                                         "covers one garment group on the SMs not left to the other group's "
                                         "collision pass (config.launch.sms_left_to_collision)"),
                         "algorithmic_bytes_per_launch": alg_bytes,
                         "launch_ms": k_step_ms, "achieved_over_whole_step": achieved_step},
            "kernel_ms": {"k_step": k_step_ms, "k_collide": k_collide_ms,
                          "how": "one chain, CUDA events around each launch, mean of 10"},
            "cpu_baseline": cpu,
            "moving_body_configs": moving,
            "config0_plain": config0,
            "adjoint_config": adjoint,
            "clocks": clocks,
            "gpu_launches": args.steps * launch["kernels_per_step"],
        }
        print(json.dumps(line), flush=True)
    group.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
