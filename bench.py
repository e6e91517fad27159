#!/usr/bin/env python
"""Throughput of the GB300 soft-body solver, one JSON line.

Workload (N=1): one body, a seeded 64^3 value-noise blob (~130k occupied
cells, 0.016 m cells, E log-uniform 1e4-1e6, nu 0.45, rho 1000) above a
ground plane with self contact through the grid broadphase, carrying 1M
Gaussian splats. One step is one rendered frame: 10 substeps of 1/600 s
(predict, 8 colour passes, contact, finalize) then the deformation of every
splat and the depth sort of their keys. Metric: cell-updates/s = occupied
cells x substeps x Gauss-Seidel sweeps / time. Inputs are synthetic and
seeded (the reference has no dataset for this path).

Timing: W untimed frames, then K frames each bracketed by CUDA events on the
solver's stream; between timed frames a 512 MiB buffer is written to flush
the 129 MB L2. `e2e` repeats the frames through the public API with host
buffers: each step uploads the node state from pinned host memory, runs the
frame and reads the positions back.

--impl reference times the oracle (the CPU restatement of the reference step,
all host threads) on the same workload; the reference itself is WGSL for
WebGPU and has no CPU step that could run.

N>1 (torchrun): the workload does not shard (one body), so every rank runs
an independent replica; value counts the cells of all replicas over the
slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

# One hardware queue per stream for the server's request loop (the vsim
# package sets the same default; here it is set before anything can create
# the CUDA context).
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

import numpy as np

ROOT = Path(__file__).resolve().parent
for p in (ROOT / "visionary-sim_gb300", ROOT / "oracle"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))

METRIC = "cell-updates/s"
BYTES_PER_ELASTIC_CELL = 8 * 48  # 8 corner nodes: pos 16 B read, prev 16 B read, pos 16 B written
VIEW = (0.3, -0.25, -0.92)


def peaks():
    path = ROOT / "MEASURED_PEAKS.json"
    if path.exists():
        d = json.loads(path.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_traffic():
    """dram bytes per elastic launch from the committed ncu summary, or None."""
    path = ROOT / "profiles" / "elastic_pass_blob64.md"
    if not path.exists():
        return None
    m = re.search(r"traffic_bytes_per_launch:\s*([0-9.eE+]+)", path.read_text())
    return float(m.group(1)) if m else None


class ClockSampler:
    """nvidia-smi samples every 200 ms while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.device = device_index
        self.proc = None
        self.path = Path(tempfile.gettempdir()) / f"vsim_clocks_{os.getpid()}.csv"

    def __enter__(self):
        try:
            self.path.parent.mkdir(exist_ok=True)
            self.out = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-i", str(self.device), "-lms", "200"], stdout=self.out,
                                         stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            self.proc.wait(timeout=5)
            self.out.close()

    def summary(self):
        if not self.proc or not self.path.exists():
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm, mx, reasons = [], [], set()
        for line in self.path.read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for name, value in zip(("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"),
                                   parts[5:9]):
                if value.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def headline_scene(quick: bool):
    import vsim.scenes as sc

    if quick:
        return sc.noise_blob(n=24, seed=1, splats=50_000)
    return sc.noise_blob(n=64, seed=1, splats=1_000_000)


def units_per_frame(scene) -> int:
    return scene.cells * scene.substeps * scene.iterations


def run_frame(sim, scene):
    sim.dispatch(scene.substeps)
    if sim.splat_count:
        sim.deform_splats(VIEW)
        sim.sort_splats()


def time_frames(sim, scene, stream, frames: int, flush) -> list:
    import torch

    times = []
    for _ in range(frames):
        with torch.cuda.stream(stream):
            flush.zero_()
        start = torch.cuda.Event(enable_timing=True)
        end = torch.cuda.Event(enable_timing=True)
        start.record(stream)
        run_frame(sim, scene)
        end.record(stream)
        end.synchronize()
        times.append(start.elapsed_time(end) / 1e3)
    return times


def replica_throughput(local_seconds: float, units_per_rank: int, device):
    """Whole-job throughput of replicas: every rank processed
    `units_per_rank` units, and the job took the slowest rank's time (a MAX
    all-reduce of the timed interval, then a barrier). Returns (seconds,
    units/s over all ranks)."""
    import torch
    import torch.distributed as dist

    world = dist.get_world_size() if dist.is_available() and dist.is_initialized() else 1
    total = local_seconds
    if world > 1:
        t = torch.tensor([local_seconds], device=device, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total = float(t.item())
        dist.barrier()
    return total, units_per_rank * world / total


def colour_pass_rate(sim, sweeps: int = 10):
    """The elastic colour pass timed as the frame runs it: `sweeps` x 8
    passes back to back in one graph (programmatic dependent launch), events
    at the two ends only (vsim_time_colour_passes; state restored). Returns
    (algorithmic bytes per launch, average launch seconds)."""
    counts = sim.color_counts()
    passes = sweeps * int(np.count_nonzero(counts))
    ms = sim.time_colour_passes(sweeps)
    return int(counts.sum()) * sweeps * BYTES_PER_ELASTIC_CELL / passes, ms / 1e3 / passes


def roofline(sim, scene, hbm):
    """The dominant kernel's roofline: the elastic colour pass. `achieved` is
    algorithmic bytes per launch over the average launch time with the passes
    back to back as in the frame; `isolated_launch_us` is one launch
    bracketed by events on its own (no overlap with its neighbours)."""
    prof = sim.profile_frame(scene.substeps, splats=True, view_dir=VIEW)
    ms, launches = prof["elastic"]
    per_launch_bytes, per_launch_s = colour_pass_rate(sim)
    achieved = per_launch_bytes / per_launch_s / 1e9
    # The same passes with each cell split over four lanes (vsim_set_cell_lanes).
    sim.set_cell_lanes(4)
    _, quad_s = colour_pass_rate(sim)
    sim.set_cell_lanes(1)
    traffic = profiled_traffic()
    share = {k: round(v[0] / sum(x[0] for x in prof.values()), 4) for k, v in prof.items()}
    return {
        "bound": "hbm",
        "kernel": "elasticKernel (one colour pass)",
        "achieved": round(achieved, 1),
        "peak": hbm,
        "unit": "GB/s",
        "frac": round(achieved / hbm, 4),
        "traffic": traffic,
        "bytes_per_launch": round(per_launch_bytes),
        "avg_launch_us": round(per_launch_s * 1e6, 3),
        "isolated_launch_us": round(1e3 * ms / (scene.substeps * scene.iterations *
                                                 int(np.count_nonzero(sim.color_counts()))), 3),
        "method": "10 sweeps x 8 colour passes back to back in one graph, CUDA events at its ends",
        "four_lanes_a_cell_launch_us": round(quad_s * 1e6, 3),
    }, {k: {"ms": round(v[0], 4), "launches": v[1]} for k, v in prof.items()}, share


# Algorithmic bytes of the contact kernels: what each must move once.
# bin: record 16 + position 16 read, key 4 + rank 4 written, bucket count 8 (r/w)
# segment: rank 4 + key 4 per record; count 4 + start 4 per occupied bucket
# scatter: key 4 + rank 4 + start 4 read, entry 4 written
# order: key, count, start 12 + record 16 + position 16 + substep start 16 + friction 4
#        read; record 16 + position 16 + motion 16 + index 4 + bucket 4 written
# gather: own entry 56, 27 neighbour buckets' count + start 8 each, every
#         visible candidate's record 16 + position 16 + motion 16, correction 16 out
CONTACT_BYTES = {"bin": (48, 0, 0), "segment": (8, 8, 0), "scatter": (16, 0, 0), "order": (120, 0, 0),
                 "gather": (56 + 27 * 8 + 16, 0, 48)}  # (per record, per occupied bucket, per candidate)


def contact_roofline(sim, hbm):
    """The contact chain on the current positions (vsim_contact_census, one
    launch of each kernel bracketed by events): its work counted from the
    live grid -- records, occupied buckets, visible candidates -- and each
    kernel's achieved bandwidth over its algorithmic bytes. Also the total by
    the per-surface-node formula (key 8 B, an 8 B read+write per sort pass --
    here 4 passes: bin, segment, scatter, order -- the 27 buckets' 8 B, 36 B
    per candidate, 32 B to apply)."""
    c = sim.contact_census()
    r, b, k = c["records"], c["occupied_buckets"], c["candidates"]
    per = {}
    for name, (pr, pb, pc) in CONTACT_BYTES.items():
        nbytes = pr * r + pb * b + pc * k
        ms = c["ms"][name]
        gbs = nbytes / (ms / 1e3) / 1e9 if ms > 0 else None
        per[name] = {"bytes": nbytes, "us": round(ms * 1e3, 2), "achieved_gbs": round(gbs, 1) if gbs else None,
                     "frac_of_measured_hbm": round(gbs / hbm, 4) if gbs else None}
    formula = r * (8 + 4 * 16 + 27 * 8 + 32) + 36 * k
    total_ms = sum(c["ms"].values())
    return {"records": r, "occupied_buckets": b, "candidates": k,
            "candidates_per_record": round(k / r, 2) if r else 0,
            "kernels": per, "chain_us": round(total_ms * 1e3, 2),
            "formula_bytes": formula,
            "formula_gbs": round(formula / (total_ms / 1e3) / 1e9, 1) if total_ms else None,
            "formula_frac_of_measured_hbm": round(formula / (total_ms / 1e3) / 1e9 / hbm, 4) if total_ms else None,
            "method": "one contact chain on the bench body's current positions, each kernel bracketed by CUDA "
                      "events (no overlap between kernels), then the grid emptied without moving a node"}


def e2e(sim, scene, frames: int):
    """The same frames through the public API with host buffers: upload the
    node state from pinned memory, run the frame, read the positions back."""
    import torch

    n = sim.node_count
    pinned = [torch.empty((n, 4), dtype=torch.float32, pin_memory=True) for _ in range(4)]
    pos, prev, vel = sim.read_state()
    for buf, src in zip(pinned[:3], (pos, prev, vel)):
        buf.numpy()[:] = src
    out = pinned[3].numpy()
    h = [b.numpy() for b in pinned[:3]]
    from vsim._ffi import check, fptr, lib

    times = []
    for _ in range(frames):
        t0 = time.perf_counter()
        check(lib().vsim_write_state(sim.handle, fptr(h[0]), fptr(h[1]), fptr(h[2]), n))
        run_frame(sim, scene)
        check(lib().vsim_read_positions(sim.handle, fptr(out), n))
        times.append(time.perf_counter() - t0)
    return times, 3 * n * 16, n * 16


def cpu_baseline(scene, budget_s: float = 12.0, single_budget_s: float = 8.0):
    """The float oracle on the bench workload, whole frames (substeps, splat
    deformation, sort) for a bounded time: on every host thread (OpenMP over
    a colour's cells and over nodes), then on one thread."""
    import pyoracle

    def sample(threads, budget):
        pyoracle.set_threads(threads)
        orc = pyoracle.Oracle(scene, 32)
        splats = scene.splats.get(0)
        frames, t0 = 0, time.perf_counter()
        while True:
            orc.dispatch(scene.substeps)
            if splats is not None:
                m, q, s, *_ = splats
                _means, _cov, keys = orc.splat_deform(0, m, q, s, VIEW)
                pyoracle.stable_sort(keys)
            frames += 1
            elapsed = time.perf_counter() - t0
            if elapsed >= budget or frames >= 50:
                break
        desc = (f"{frames} full frames ({scene.substeps} substeps + {len(splats[0]) if splats else 0} "
                f"splat deformations and sort) of the bench workload, float oracle, {elapsed:.1f} s")
        return units_per_frame(scene) * frames / elapsed, desc

    threads = os.cpu_count() or 1
    value, desc = sample(threads, budget_s)
    one, one_desc = sample(1, single_budget_s)
    pyoracle.set_threads(threads)
    return {"value": value, "unit": METRIC, "cores": threads, "kind": "port", "sample": desc,
            "single_thread": {"value": one, "unit": METRIC, "cores": 1, "kind": "port", "sample": one_desc}}


def reference_arm(scene, steps: int, warmup: int):
    """The oracle, all host threads, W untimed then K timed frames of the
    bench workload (each a full frame: substeps, splat deformation, sort)."""
    import pyoracle

    threads = os.cpu_count() or 1
    pyoracle.set_threads(threads)
    orc = pyoracle.Oracle(scene, 32)
    m, q, s, *_ = scene.splats[0]

    def frame():
        orc.dispatch(scene.substeps)
        _means, _cov, keys = orc.splat_deform(0, m, q, s, VIEW)
        pyoracle.stable_sort(keys)

    for _ in range(warmup):
        frame()
    t0 = time.perf_counter()
    for _ in range(steps):
        frame()
    elapsed = time.perf_counter() - t0
    return {"value": units_per_frame(scene) * steps / elapsed, "unit": METRIC, "cores": threads, "kind": "port",
            "sample": f"{steps} timed frames after {warmup} warm-up frames of the bench workload, float oracle, "
                      f"{elapsed:.1f} s"}


def batched_vs_plain(frames: int, quick: bool, cpu: bool = True):
    """The batching workload: 256 uneven boxes with 20k splats each. One
    frame = 10 substeps, every splat deformed, the depth keys sorted.

    - batched: one simulator stepping every body in the same launches, its
      frame a captured graph (programmatic dependent launch), one deformation
      and one sort over all 5.12M splats;
    - plain: one simulator per body, each body its own launch sequence, its
      own 20k splats deformed and sorted, in three forms: on one stream
      launched kernel by kernel; on one stream with each body's frame a
      captured graph; and each body on a stream of its own with its graph
      (bodies overlap on the device).

    Every arm is timed with CUDA events over `frames` frames after two
    untimed ones: events on a common stream, with per-body streams joined to
    it by events. `cpu_baseline`: the float oracle on all host cores, a
    bounded sample of the same frames."""
    import torch

    import vsim.scenes as sc
    from vsim import Simulator

    count = 32 if quick else 256
    splats = 2_000 if quick else 20_000
    t0 = time.perf_counter()
    scene = sc.box_batch(count, seed=2, splats_per_body=splats)
    gen_s = time.perf_counter() - t0
    units = units_per_frame(scene)
    main = torch.cuda.Stream()

    def one_body(b):
        one = sc.Scene([scene.bodies[b]], scene.tank, step_duration=scene.step_duration, substeps=scene.substeps,
                       contact=False)
        one.splats[0] = scene.splats[b]
        return one

    def timed(run, streams=None):
        for _ in range(2):
            run()
        torch.cuda.synchronize()
        start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        start.record(main)
        for st in streams or []:
            st.wait_event(start)
        for _ in range(frames):
            run()
        for st in streams or []:
            done = torch.cuda.Event()
            done.record(st)
            main.wait_event(done)
        end.record(main)
        end.synchronize()
        return start.elapsed_time(end) / 1e3 / frames

    out = {"workload": f"{len(scene.bodies)} boxes, sides log-uniform 4-48 cells, {scene.cells} cells, "
                       f"{splats} splats per body ({splats * len(scene.bodies)} in all), ground contact; one frame = "
                       f"{scene.substeps} substeps + splat deformation + depth sort",
           "unit": METRIC, "frames_timed": frames, "timing": "CUDA events on a common stream"}
    batch = Simulator(scene, stream=main.cuda_stream)
    t_batch = timed(lambda: run_frame(batch, scene))
    out["batched"] = round(units / t_batch)
    out["batched_frame_ms"] = round(t_batch * 1e3, 3)
    batch.destroy()

    arms = {}
    bodies = [one_body(b) for b in range(len(scene.bodies))]
    singles = [Simulator(one, stream=main.cuda_stream) for one in bodies]

    def plain():
        for sim, one in zip(singles, bodies):
            run_frame(sim, one)

    for s in singles:
        s.set_graph(False)
        s.set_pdl(False)
    arms["plain_one_stream_no_graph"] = timed(plain)
    for s in singles:
        s.set_graph(True)
        s.set_pdl(True)
    arms["plain_one_stream_graph"] = timed(plain)
    for s in singles:
        s.destroy()
    streams = [torch.cuda.Stream() for _ in bodies]
    singles = [Simulator(one, stream=st.cuda_stream) for one, st in zip(bodies, streams)]
    arms["plain_stream_per_body_graph"] = timed(plain, streams)
    for s in singles:
        s.destroy()
    for name, t in arms.items():
        out[name] = round(units / t)
        out[name + "_frame_ms"] = round(t * 1e3, 3)
    best = min(arms, key=arms.get)
    out["ratio_vs_plain_no_graph"] = round(arms["plain_one_stream_no_graph"] / t_batch, 2)
    out["ratio_vs_plain_graph"] = round(arms["plain_one_stream_graph"] / t_batch, 2)
    out["ratio_vs_plain_stream_per_body"] = round(arms["plain_stream_per_body_graph"] / t_batch, 2)
    out["ratio_vs_fastest_plain"] = round(arms[best] / t_batch, 2)
    out["fastest_plain"] = best
    out["scene_generation_s"] = round(gen_s, 1)
    if cpu:
        out["cpu_baseline"] = batch_cpu_baseline(scene, budget_s=6.0 if quick else 20.0)
    return out


def batch_cpu_baseline(scene, budget_s: float):
    """The float oracle, all host threads, on the batching workload: whole
    frames (every body's substeps, every body's splats deformed, the depth
    keys of all of them sorted together) until `budget_s` has passed."""
    import pyoracle

    threads = os.cpu_count() or 1
    pyoracle.set_threads(threads)
    orc = pyoracle.Oracle(scene, 32)
    frames, t0 = 0, time.perf_counter()
    while True:
        orc.dispatch(scene.substeps)
        keys = [orc.splat_deform(b, m, q, s, VIEW)[2] for b, (m, q, s, *_r) in scene.splats.items()]
        if keys:
            pyoracle.stable_sort(np.concatenate(keys))
        frames += 1
        elapsed = time.perf_counter() - t0
        if elapsed >= budget_s or frames >= 20:
            break
    return {"value": round(units_per_frame(scene) * frames / elapsed), "unit": METRIC, "cores": threads,
            "kind": "port", "sample": f"{frames} full frames of the batching workload, float oracle, "
                                      f"{elapsed:.1f} s"}


def single_body_pass(quick: bool, hbm: float):
    """The colour pass of one large body alone: the stress workload's 192^3
    noise blob without the sheet (48^3 with --quick), timed as
    colour_pass_rate times it."""
    import vsim.scenes as sc
    from vsim import Simulator

    scene = sc.noise_blob(n=48 if quick else 192, seed=4, splats=0)
    sim = Simulator(scene)
    per_launch, per_launch_s = colour_pass_rate(sim)
    achieved = per_launch / per_launch_s / 1e9
    out = {"workload": f"noise blob {scene.bodies[0].cell_dims[0]}^3 alone, {scene.cells} cells",
           "achieved_gbs": round(achieved, 1), "frac_of_measured_hbm": round(achieved / hbm, 4),
           "bytes_per_launch": round(per_launch), "avg_launch_us": round(per_launch_s * 1e6, 2)}
    # The same passes in the TMA brick form (vsim_set_tma_pass), measured
    # against the streaming form it would replace.
    sim.set_tma_pass(True)
    per_launch, per_launch_s = colour_pass_rate(sim)
    sim.synchronize()
    achieved = per_launch / per_launch_s / 1e9
    out["tma_bricks"] = {"achieved_gbs": round(achieved, 1), "frac_of_measured_hbm": round(achieved / hbm, 4),
                         "avg_launch_us": round(per_launch_s * 1e6, 2)}
    sim.destroy()
    return out


def stress(quick: bool, hbm: float, frames: int = 3):
    """The stress workload: a 192^3 noise blob with a 192 x 192 x 2 sheet above it
    (E 5e5, nu 0.48), ground, self and body contact, 20 substeps of 2
    Gauss-Seidel sweeps per frame, 20M splats deformed and depth-sorted."""
    import torch

    import vsim.scenes as sc
    from vsim import Simulator

    t0 = time.perf_counter()
    scene = sc.blob_and_sheet(n=48 if quick else 192, seed=4, splats=200_000 if quick else 20_000_000)
    gen_s = time.perf_counter() - t0
    stream = torch.cuda.Stream()
    sim = Simulator(scene, stream=stream.cuda_stream)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")
    run_frame(sim, scene)
    sim.synchronize()
    times = time_frames(sim, scene, stream, frames, flush)
    prof = sim.profile_frame(scene.substeps, splats=True, view_dir=VIEW)
    ms, launches = prof["elastic"]
    per_launch, per_launch_s = colour_pass_rate(sim)
    achieved = per_launch / per_launch_s / 1e9
    n_splats = sim.splat_count
    sort_ms, sort_launches = prof.get("sort", (0.0, 0))
    splat_ms, _ = prof.get("splat", (0.0, 0))
    out = {"workload": f"blob {scene.bodies[0].cell_dims[0]}^3 + sheet, {scene.cells} cells, "
                       f"{sim.node_count} node slots, {scene.substeps} substeps x {scene.iterations} sweeps, "
                       f"{n_splats} splats",
           "value": round(units_per_frame(scene) * frames / sum(times)), "unit": METRIC,
           "frame_ms": round(1e3 * statistics.median(times), 3),
           "elastic_pass": {"achieved_gbs": round(achieved, 1), "frac_of_measured_hbm": round(achieved / hbm, 4),
                            "bytes_per_launch": round(per_launch), "avg_launch_us": round(per_launch_s * 1e6, 2),
                            "isolated_launch_us": round(1e3 * ms / launches, 2),
                            "method": "10 sweeps x 8 colour passes back to back in one graph"},
           "single_body_elastic_pass": single_body_pass(quick, hbm),
           "splat_deform_gbs": round(92 * n_splats / (splat_ms / 1e3) / 1e9, 1) if splat_ms else None,
           "sort_keys_per_s": round(n_splats / (sort_ms / 1e3)) if sort_ms else None,
           "kernel_groups_one_frame": {k: {"ms": round(v[0], 3), "launches": v[1]} for k, v in prof.items()},
           "scene_generation_s": round(gen_s, 1)}
    sim.destroy()
    del flush
    return out


def cloud_voxelize(quick: bool, reps: int = 5):
    """The Gaussian-cloud voxeliser (cloudVolume.js's voxelizeCloud) on a
    synthetic capture: 2M Gaussians on a 0.3 m sphere (vsim.scenes.
    capture_cloud, seed 7), 2 mm cells (a 311^3 grid), sigma 2, seal 2, fill
    on. `gaussians_per_s`: the cloud resident on the device, the grid left
    there (vsim_voxelize_cloud_device returns with it built); `e2e`: from
    pinned host arrays to the occupancy in pinned host memory
    (vsim_voxelize_cloud + vsim_cloud_volume_read); `cpu`: the host
    restatement of the reference's voxeliser (numpy, one core) on the same
    cloud, with its grid compared to the device's."""
    import ctypes as C

    import torch

    import vsim.scenes as sc
    from vsim import _ffi
    from vsim import voxelize as vz

    n = 200_000 if quick else 2_000_000
    element = 0.004 if quick else 0.002
    cloud = sc.capture_cloud(n, 0.3, seed=7)
    lib = _ffi.lib()
    opts = _ffi.CloudOptions(element, 2.0, 2, 2, 1)
    dev = [torch.from_numpy(a).cuda() for a in cloud]
    pinned = [torch.from_numpy(a).pin_memory() for a in cloud]
    fp = [C.cast(t.data_ptr(), C.POINTER(C.c_float)) for t in pinned]

    def on_device():
        vol = C.c_void_p()
        _ffi.check(lib.vsim_voxelize_cloud_device(dev[0].data_ptr(), dev[1].data_ptr(), dev[2].data_ptr(), n,
                                                  C.byref(opts), None, C.byref(vol)))
        return vol

    grid = _ffi.CloudGrid()
    lib.vsim_cloud_volume_destroy(on_device())
    torch.cuda.synchronize()
    device_s = []
    for _ in range(reps):
        t = time.perf_counter()
        vol = on_device()
        device_s.append(time.perf_counter() - t)
        _ffi.check(lib.vsim_cloud_volume_grid(vol, C.byref(grid)))
        lib.vsim_cloud_volume_destroy(vol)
    dims = [int(v) for v in grid.dims]
    cells = dims[0] * dims[1] * dims[2]
    occupancy = torch.empty(cells, dtype=torch.uint8).pin_memory()
    out_ptr = C.cast(occupancy.data_ptr(), C.POINTER(C.c_uint8))
    e2e_s = []
    for _ in range(reps):
        t = time.perf_counter()
        vol = C.c_void_p()
        _ffi.check(lib.vsim_voxelize_cloud(fp[0], fp[1], fp[2], n, C.byref(opts), C.byref(vol)))
        _ffi.check(lib.vsim_cloud_volume_read(vol, out_ptr, cells))
        e2e_s.append(time.perf_counter() - t)
        lib.vsim_cloud_volume_destroy(vol)
    t = time.perf_counter()
    host = vz.voxelize_cloud(*cloud, element)
    cpu_s = time.perf_counter() - t
    med, e2e_med = statistics.median(device_s), statistics.median(e2e_s)
    return {"workload": f"synthetic capture, {n} Gaussians on a 0.3 m sphere, {element * 1e3:g} mm cells "
                        f"({dims[0]}x{dims[1]}x{dims[2]} grid), sigma 2, seal 2, fill",
            "gaussians_per_s": round(n / med), "ms": round(med * 1e3, 3),
            "occupied": int(grid.occupied), "filled": int(grid.filled),
            "e2e": {"gaussians_per_s": round(n / e2e_med), "ms": round(e2e_med * 1e3, 3),
                    "h2d_bytes": 40 * n, "d2h_bytes": cells},
            "cpu": {"gaussians_per_s": round(n / cpu_s), "s": round(cpu_s, 2), "cores": 1,
                    "kind": "host restatement (numpy)"},
            "grid_equal_to_host": host.dims == dims and bool(np.array_equal(host.occupancy, occupancy.numpy()))}


def capture_sessions(settle_frames: int = 30):
    """Profiler capture of one session-kernel launch: the 64-session pool
    (every session settled for `settle_frames` frames), then one request of
    one frame for each session small enough for a block, run through the
    request loop with only that launch between cudaProfilerStart/Stop, for
    `ncu --profile-from-start off -k regex:sessionKernel`."""
    import torch

    import vsim.scenes as sc
    from vsim.server import Server

    bodies, tank = sc.session_pool(64, seed=3)
    server = Server(bodies, tank, budget_bytes=150e9)
    n = server.admitted
    for q in range(n):
        server.submit(q, settle_frames)
    while server.stats()["pending"]:
        server.tick()
        server.poll()
    small = [q for q in range(n) if bodies[q].cell_count <= 1500]
    ones = np.ones(len(small), np.int64)
    server.run(np.zeros(len(small)), np.array(small), ones, np.zeros(len(small), np.int64))  # warm
    torch.cuda.synchronize()
    torch.cuda.profiler.start()
    done, _ = server.run(np.zeros(len(small)), np.array(small), ones, np.zeros(len(small), np.int64))
    torch.cuda.synchronize()
    torch.cuda.profiler.stop()
    server.destroy()
    return {"captured_session_requests": len(small), "cells": int(sum(bodies[q].cell_count for q in small))}


def tick_sweep(quick: bool, capture: int | None = None, reps: int = 25, settle_frames: int = 30):
    """Tick time of the session server against the number of sessions a tick
    runs: the 1000-session pool of the serving workload (64 with --quick),
    settled for `settle_frames` frames, then ticks of k = 1, 3, 10, 40, 200,
    1000 sessions (random, one frame each), median host-timed tick over
    `reps` ticks after 5 unrecorded. With `capture` = k, one tick of k
    sessions is bracketed by cudaProfilerStart/Stop for
    `ncu --profile-from-start off` instead."""
    import torch

    import vsim.scenes as sc
    from vsim.server import Server

    count = 64 if quick else 1000
    bodies, tank = sc.session_pool(count, seed=3)
    server = Server(bodies, tank, budget_bytes=150e9)
    n = server.admitted
    for s in range(n):
        server.submit(s, settle_frames)
    while server.stats()["pending"]:
        server.tick()
        server.poll()
    rng = np.random.default_rng(1)
    if capture is not None:
        for _ in range(3):
            for s in rng.choice(n, capture, replace=False):
                server.submit(int(s), 1)
            server.tick()
            server.poll()
        for s in rng.choice(n, capture, replace=False):
            server.submit(int(s), 1)
        torch.cuda.profiler.start()
        server.tick()
        torch.cuda.profiler.stop()
        server.poll()
        return {"captured_tick_sessions": capture}
    out = {}
    for k in (1, 3, 10, 40, 200, 1000):
        k = min(k, n)
        ts = []
        for rep in range(reps + 5):
            for s in rng.choice(n, k, replace=False):
                server.submit(int(s), 1)
            t = time.perf_counter()
            server.tick()
            ts.append(time.perf_counter() - t)
            server.poll()
        out[str(k)] = round(statistics.median(ts[5:]) * 1e3, 3)
    server.destroy()
    return {"workload": f"{n} sessions resident, settled {settle_frames} frames; ticks of k sessions, one frame each",
            "tick_ms_by_sessions": out}


def drift(frames: int = 300):
    """The 16 x 4 x 4 bar for `frames` frames on the GPU against the oracle
    in double precision from the same start: the float trajectory's
    departure from the exact arithmetic (reported, not gated; the configs'
    CFL numbers are above 1, so trajectories are sensitive)."""
    import pyoracle
    import vsim.scenes as sc
    from vsim import Simulator

    scene = sc.single_box()
    sim = Simulator(scene)
    ref = pyoracle.Oracle(scene, 64)
    diag = float(np.linalg.norm(np.asarray(scene.bodies[0].cell_dims) * scene.bodies[0].h))
    worst, at = 0.0, 0
    for f in range(frames):
        sim.dispatch(scene.substeps)
        ref.dispatch(scene.substeps)
        if f % 10 == 9 or f == frames - 1:
            g = sim.read_positions()[:, :3].astype(np.float64)
            r = ref.state_f64()[0][:, :3]
            err = float(np.max(np.abs(g - r))) / max(float(np.max(np.abs(r))), diag)
            if err > worst:
                worst, at = err, f + 1
    g = sim.read_positions()[:, :3].astype(np.float64)
    r = ref.state_f64()[0][:, :3]
    sim.destroy()
    return {"workload": "16x4x4 bar, pinned end, 10 substeps/frame", "frames": frames,
            "max_relative_error": worst, "at_frame": at,
            "final_max_abs_m": float(np.max(np.abs(g - r)))}


def serving_sweep(quick: bool, budgets=(0,), seconds_per_point: float = 5.0, settle_frames: int = 30,
                  repeats_at_70: int = 3, engines=("sessions", "frames"), block_cells=(32,), cluster_cells=(512,)):
    """Continuous batching under load: a pool of sessions resident on the
    GPU; requests advance a session k ~ U{1..4} frames, half of them dragging
    a random surface node along a seeded Bezier curve at 0.5 m/s. Every
    session first runs `settle_frames` frames (all at once), so that the
    bodies have landed and flattened -- the state they spend their life in,
    with far more self contact than at rest -- before anything is measured.

    For each engine of the library's request loop (vsim_server_set_engine:
    "sessions", small sessions' requests run whole by the session kernel,
    launches overlapping, the larger ones in ticks alongside; "frames",
    ticks of one shared frame for all, under each tick budget -- occupied
    cells one tick may step, 0 = no cap): saturation measured closed-loop
    (as many requests outstanding as sessions, each completion replaced by
    one to a uniformly drawn session: the capacity for the open loop's
    session mix), then Poisson arrivals
    at 25/50/70/90 % of that saturation, the 70 % point `repeats_at_70`
    times, each run by vsim_server_run against a pre-drawn schedule, so no
    client code sits between launches, after half a second of the same
    load that is not measured. Each of these starts from the same
    settled state (every session checkpointed after the settling frames and
    written back before the measurement). Frame latency of a request =
    (completion - scheduled arrival) / k."""
    import vsim.scenes as sc
    from vsim.server import Server

    count = 64 if quick else 1000
    t0 = time.perf_counter()
    bodies, tank = sc.session_pool(count, seed=3)
    gen_s = time.perf_counter() - t0
    server = Server(bodies, tank, budget_bytes=150e9)
    admitted = server.admitted
    rng = np.random.default_rng(7)
    # every session's drag: a random surface node along a seeded Bezier curve
    drags = [sc.drag_request(bodies[s], rng) for s in range(admitted)]

    def drain():
        while server.stats()["pending"]:
            server.tick()
            server.poll()

    t0 = time.perf_counter()
    server.set_tick_budget(0)
    for s in range(admitted):
        server.submit(s, settle_frames)
    drain()
    settle_s = time.perf_counter() - t0
    # Every measurement starts from this settled state: the bodies keep
    # deforming under the drags, and a saturation measured on one state and
    # loads applied to a later, costlier one would not be fractions of the
    # same capacity.
    checkpoint = [server.read_state(s) for s in range(admitted)]

    def restore():
        for s in range(admitted):
            server.write_state(s, *checkpoint[s])

    def specs(count):
        return rng.integers(1, 5, count), rng.random(count) < 0.5

    def widest_colour(b):
        occ = np.asarray(b.occupancy).reshape(b.cell_dims[2], b.cell_dims[1], b.cell_dims[0])
        k, j, i = np.nonzero(occ)
        return int(np.bincount((i & 1) | ((j & 1) << 1) | ((k & 1) << 2), minlength=8).max())

    widest = np.array([widest_colour(b) for b in bodies])
    engine_shape = {"block": 0, "cluster": 0}

    def saturation():
        restore()
        frames, flags = specs(200_000)
        sessions = rng.integers(0, admitted, frames.size)
        c0 = server.stats()["cell_updates"]
        _, rep = server.run(None, sessions, frames, flags, drags, closed_loop_seconds=seconds_per_point)
        cells = server.stats()["cell_updates"] - c0
        return {"requests_per_s": round(rep["requests"] / rep["seconds"], 1),
                "session_frames_per_s": round(rep["frames"] / rep["seconds"], 1), "ticks": rep["ticks"],
                "cell_updates_per_s_incl_drain": round(cells / rep["seconds"]),
                "method": "closed loop in the library's request loop (vsim_server_run): as many requests "
                          "outstanding as sessions, each completion replaced by one to a uniformly drawn session"}

    def schedule(lam, seconds):
        arrivals = np.cumsum(rng.exponential(1 / lam, int(lam * seconds * 1.5) + 16))
        arrivals = arrivals[arrivals < seconds]
        sessions = rng.integers(0, admitted, arrivals.size)
        frames, flags = specs(arrivals.size)
        return arrivals, sessions, frames, flags

    def point(frac, sat_rate):
        lam = frac * sat_rate
        # warm-up: half a second at the same rate, not measured, then the
        # settled state again
        restore()
        server.run(*schedule(lam, 0.5), drags)
        restore()
        arrivals, sessions, frames, flags = schedule(lam, seconds_per_point)
        st_before = server.stats()
        done, rep = server.run(arrivals, sessions, frames, flags, drags)
        st_after = server.stats()
        lat = np.array([(c["completed"] - c["submitted"]) / c["frames"] for c in done])
        req_lat = np.array([c["completed"] - c["submitted"] for c in done])
        # p99 by where the session runs under the session engine's thresholds
        kernel_limit = max(engine_shape["block"], engine_shape["cluster"])
        in_kernel = np.array([widest[c["session"]] <= kernel_limit for c in done])
        by_class = {}
        for name, sel in (("kernel", in_kernel), ("ticks", ~in_kernel)):
            if sel.any():
                by_class[name] = {"requests": int(sel.sum()),
                                  "p99": round(1e3 * float(np.percentile(lat[sel], 99)), 3)}
        ticks_run = max(1, st_after["ticks"] - st_before["ticks"])
        tick_ms = {k: round(1e3 * (st_after[f"{k}_seconds"] - st_before[f"{k}_seconds"]) / ticks_run, 3)
                   for k in ("tick", "prepare", "frame")}
        return {"load": frac, "offered_req_per_s": round(lam, 1),
                "frame_latency_ms": {"p50": round(1e3 * float(np.percentile(lat, 50)), 3),
                                     "p99": round(1e3 * float(np.percentile(lat, 99)), 3)},
                "request_latency_ms": {"p50": round(1e3 * float(np.percentile(req_lat, 50)), 3),
                                       "p99": round(1e3 * float(np.percentile(req_lat, 99)), 3)},
                "requests": len(lat),
                "frame_latency_p99_by_class_ms": by_class,
                "sessions_per_tick": round((st_after["session_frames"] - st_before["session_frames"]) / ticks_run, 1),
                "mean_tick_ms": tick_ms,
                "cell_updates_per_s": round((st_after["cell_updates"] - st_before["cell_updates"]) / rep["seconds"])}

    def sweep():
        sat = saturation()
        points = []
        for frac in (0.25, 0.5, 0.7, 0.9):
            for _ in range(repeats_at_70 if frac == 0.7 else 1):
                points.append(point(frac, sat["requests_per_s"]))
        p99_70 = [p["frame_latency_ms"]["p99"] for p in points if p["load"] == 0.7]
        return {"saturation": sat, "sweep": points,
                "p99_frame_latency_ms_at_70pct": {"max": max(p99_70), "all": p99_70}}

    def floors(engine):
        """One 1-frame request alone on the idle server, for the smallest,
        median and largest resident session and the sessions at the 10th to
        40th percentiles of size: median of 15 (completion - arrival), the
        latency with no queueing at all."""
        order = sorted(range(admitted), key=lambda q: bodies[q].cell_count)
        out = {}
        picks = [("smallest", order[0])] + [(f"p{k}", order[len(order) * k // 100]) for k in (10, 20, 30, 40)]
        for label, q in picks + [("median", order[len(order) // 2]), ("largest", order[-1])]:
            lat = []
            for _ in range(15):
                done, _ = server.run(np.zeros(1), np.array([q]), np.ones(1, np.int64), np.zeros(1, np.int64))
                lat.append(done[0]["completed"] - done[0]["submitted"])
            out[label] = {"session_cells": bodies[q].cell_count, "ms": round(1e3 * float(np.median(lat)), 3)}
        return out

    by_engine = {}
    for engine in engines:
        if engine == "sessions":
            shapes = [(b, c, t) for b in block_cells for c in cluster_cells for t in budgets]
            for cells, wide, budget in shapes:
                server.set_engine(server.SESSIONS, cells, wide)
                server.set_tick_budget(budget)
                engine_shape.update(block=cells, cluster=wide)
                restore()
                key = engine if len(shapes) == 1 else f"{engine}_block{cells}_cluster{wide}_budget{budget}"
                by_engine[key] = {"block_cells": cells, "cluster_cells": wide, "tick_cell_budget": budget,
                                  "one_request_floor": floors(engine), **sweep()}
            server.set_tick_budget(0)
        else:
            server.set_engine(server.FRAMES)
            engine_shape.update(block=0, cluster=0)
            restore()
            by_engine[engine] = {"one_request_floor": floors(engine)}
            runs = {}
            for budget in budgets:
                server.set_tick_budget(budget)
                runs[str(budget)] = {"tick_cell_budget": budget, **sweep()}
            server.set_tick_budget(0)
            by_engine[engine]["by_tick_budget"] = runs
    st = server.stats()
    server.destroy()
    return {"workload": f"{admitted} sessions ({count} offered), noise blobs on 8^3-64^3 grids, "
                        f"{sum(b.cell_count for b in bodies[:admitted])} cells resident, "
                        f"{st['resident_bytes'] / 1e9:.2f} GB of the 150 GB budget; k ~ U{{1..4}} frames, "
                        f"50% with a Bezier drag at 0.5 m/s",
            "by_engine": by_engine, "settle": {"frames": settle_frames, "seconds": round(settle_s, 1)},
            "hardware_queues": os.environ.get("CUDA_DEVICE_MAX_CONNECTIONS", "8 (driver default)"),
            "pool_generation_s": round(gen_s, 1)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="vsim", choices=["vsim", "reference"])
    ap.add_argument("--quick", action="store_true", help="small workload, for checking the harness")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--no-stress", action="store_true")
    ap.add_argument("--no-cloud", action="store_true")
    ap.add_argument("--stress-only", action="store_true", help="only the stress workload's frames (for captures)")
    ap.add_argument("--cloud-only", action="store_true", help="only the cloud voxeliser section (for captures)")
    ap.add_argument("--pass-only", action="store_true", help="only the single large body's colour pass, both forms")
    ap.add_argument("--tick-sweep", action="store_true", help="only the server's tick time against sessions per tick")
    ap.add_argument("--serve-only", action="store_true", help="only the serving sweep")
    ap.add_argument("--batch-only", action="store_true", help="only the batching comparison")
    ap.add_argument("--tick-budgets", default=None,
                    help="comma-separated tick cell budgets for the serving sweep (0 = no cap)")
    ap.add_argument("--serve-block-cells", default="32",
                    help="comma-separated block thresholds of the session engine (cells of a session's largest colour)")
    ap.add_argument("--serve-cluster-cells", default="512",
                    help="comma-separated cluster thresholds of the session engine (0: no cluster jobs)")
    ap.add_argument("--serve-engines", default="sessions,frames",
                    help="comma-separated request-loop engines for the serving sweep (sessions, frames)")
    ap.add_argument("--capture-sessions", action="store_true",
                    help="profiler capture mode: one session-kernel launch over the 64-session pool's small sessions")
    ap.add_argument("--capture-tick", type=int, default=None, metavar="K",
                    help="profiler capture mode: one server tick of K sessions, for `ncu --profile-from-start off`")
    ap.add_argument("--capture-after", type=int, default=None, metavar="N",
                    help="profiler capture mode: run N frames of the bench workload, then bracket one more frame "
                         "(or --capture-substeps substeps) with cudaProfilerStart/Stop for "
                         "`ncu --profile-from-start off`, and exit")
    ap.add_argument("--capture-substeps", type=int, default=None)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    scene = headline_scene(args.quick)
    config = {"workload": ("noise blob %d^3 (%d cells), self contact + ground, %d splats; one frame = %d "
                           "substeps + splat deformation + depth sort" %
                           (scene.bodies[0].cell_dims[0], scene.cells, len(scene.splats[0][0]), scene.substeps)),
              "cells": scene.cells, "substeps": scene.substeps, "iterations": scene.iterations,
              "splats": len(scene.splats[0][0]), "l2": "flushed between timed frames (512 MiB write)",
              "parallelism": f"replicas x{args.gpus}" if args.gpus > 1 else "single GPU"}

    if args.impl == "reference":
        if rank != 0:
            return
        base = reference_arm(scene, args.steps, args.warmup)
        line = {"impl": "reference", "metric": METRIC, "value": base["value"], "unit": METRIC,
                "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": 1e3 * units_per_frame(scene) / base["value"], "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
                "config": config, "cpu_baseline": base,
                "e2e": {"value": base["value"], "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    import torch

    import __graft_entry__

    __graft_entry__.build()
    from vsim import Simulator

    torch.cuda.set_device(local)
    if args.stress_only:
        print(json.dumps({"stress": stress(args.quick, peaks()[0], frames=args.steps)}))
        return
    if args.cloud_only:
        print(json.dumps({"cloud_voxelize": cloud_voxelize(args.quick)}))
        return
    if args.pass_only:
        print(json.dumps({"single_body_elastic_pass": single_body_pass(args.quick, peaks()[0])}))
        return
    budgets = [int(float(v)) for v in args.tick_budgets.split(",")] if args.tick_budgets else [0]
    if args.serve_only:
        print(json.dumps({"serving": serving_sweep(args.quick, budgets, engines=args.serve_engines.split(","),
                                   block_cells=[int(v) for v in args.serve_block_cells.split(",")],
                                   cluster_cells=[int(v) for v in args.serve_cluster_cells.split(",")])}))
        return
    if args.batch_only:
        print(json.dumps({"batching": batched_vs_plain(10, args.quick, cpu=not args.no_cpu)}))
        return
    if args.capture_sessions:
        print(json.dumps({"capture_sessions": capture_sessions()}))
        return
    if args.tick_sweep or args.capture_tick is not None:
        print(json.dumps({"tick_sweep": tick_sweep(args.quick, args.capture_tick)}))
        return
    if args.capture_after is not None:
        sim = Simulator(scene)
        for _ in range(args.capture_after):
            run_frame(sim, scene)
        sim.synchronize()
        torch.cuda.profiler.start()
        if args.capture_substeps:
            sim.dispatch(args.capture_substeps)
        else:
            run_frame(sim, scene)
        sim.synchronize()
        torch.cuda.profiler.stop()
        print(json.dumps({"captured_after_frames": args.capture_after, "substeps": args.capture_substeps}))
        return
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    stream = torch.cuda.Stream()
    sim = Simulator(scene, stream=stream.cuda_stream)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")
    for _ in range(args.warmup):
        run_frame(sim, scene)
    sim.synchronize()
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    with ClockSampler(local) as clocks:
        times = time_frames(sim, scene, stream, args.steps, flush)
    torch.cuda.synchronize()
    total, value = replica_throughput(float(sum(times)), units_per_frame(scene) * args.steps, "cuda")
    launches = args.steps * (sim.frame_launches(scene.substeps) + sim.splat_launches())

    hbm, peak_kind = peaks()
    roof, groups, share = roofline(sim, scene, hbm)
    roof["peak_source"] = f"{peak_kind} hbm_gbs"
    e2e_times, h2d, d2h = e2e(sim, scene, max(3, args.steps // 2))
    e2e_value = units_per_frame(scene) / statistics.mean(e2e_times) * world

    detail = {"kernel_groups_one_frame": groups, "time_share": share,
              "contact_roofline": contact_roofline(sim, hbm),
              "frame_ms": {"min": round(min(times) * 1e3, 4), "median": round(statistics.median(times) * 1e3, 4)}}
    if rank == 0 and not args.no_batch:
        detail["batching"] = batched_vs_plain(10, args.quick, cpu=not args.no_cpu)
    if rank == 0 and not args.no_serve:
        detail["serving"] = serving_sweep(args.quick, budgets, engines=args.serve_engines.split(","),
                                   block_cells=[int(v) for v in args.serve_block_cells.split(",")],
                                   cluster_cells=[int(v) for v in args.serve_cluster_cells.split(",")])
    if rank == 0 and not args.no_stress:
        detail["stress"] = stress(args.quick, hbm)
    if rank == 0 and not args.no_cloud:
        detail["cloud_voxelize"] = cloud_voxelize(args.quick)
    if rank == 0:
        detail["drift_vs_fp64"] = drift(30 if args.quick else 300)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_baseline(scene)
    if rank == 0:
        line = {"metric": METRIC, "value": round(value), "unit": METRIC, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": round(1e3 * total / args.steps, 4), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
                "config": config, "gpu_launches": launches, "clocks": clocks.summary(), "roofline": roof,
                "cpu_baseline": cpu,
                "e2e": {"value": round(e2e_value), "unit": METRIC, "h2d_bytes_per_step": h2d,
                        "d2h_bytes_per_step": d2h},
                "detail": detail}
        print(json.dumps(line))
    sim.destroy()
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
