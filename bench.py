#!/usr/bin/env python
"""Benchmark: particle-steps/s of the voxel SPH step on the 4M-particle box.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

One step = hash, voxel sort, voxel table, density, forces, integrate and wall
response for all 4,194,304 particles (128x256x128 dam break in a [0,2]^3 box,
h = 0.0112, 5,735,339 voxels).  The state (~0.4 GB with both sort buffers) is
larger than the 129 MB L2, so no flush is needed between steps.

--impl gb300 (default): W untimed steps, then K steps timed with CUDA events
(one CUDA-graph replay per step), barrier + synchronize on both sides, max over
ranks.  Every step is a complete compute_next_state of the same resident
input (the dam-break start state), written to separate output buffers: under
the reference's formulas this scene is not stable (the pressure term has no
MASS factor, voxel_kernels.py:171, so forces scale like h^-4; the FP64 oracle
reaches |v| = 571 m/s at step 2 and non-finite velocities at step 3), so a
free-running benchmark would time the collapse instead of the step.  The
free-running rate over the first steps is reported beside it.  Under torchrun each rank advances its own replica of the scene (the
single scene does not shard; replicas only).  Also reported:
  e2e      the same metric through the C ABI host-buffer entry point
           (sphgb_compute_next_state_host): FP64 AoS state copied from pinned
           host memory and the next state copied back, every step;
  roofline the dominant kernel's algorithmic bytes / its mean CUDA-event time;
  cpu_baseline  the oracle's C/OpenMP FP64 step on the host cores (rank 0);
  oracle_err    the step's error against that FP64 step of the same input;
  batched, served, pipe_flow  the batched-scene, served-request and pipe-flow
           workloads (skipped with --no-batched).
--impl reference: the reference's algorithm on the host cores (the oracle's
C/OpenMP restatement; the reference itself is numba-CUDA Python and cannot run
here), same metric; rank 0 only.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (os.path.join(ROOT, "cuda-sph_gb300"), ROOT):
    if _p not in sys.path:
        sys.path.insert(0, _p)

# algorithmic bytes per particle of each stage (FP32 SoA, each array touched
# once per pass): hash 16 + histogram 4; scan 8 per voxel (+4 clear);
# scatter 8; rank-gather (reorder) 48; density 16; forces 40 + integrate/wall 60
STAGE_BYTES_PER_PARTICLE = {"hash": 20, "scan": 0, "scatter": 8, "rank_gather": 48,
                            "density": 16, "force_integrate": 100, "step_counter": 0}
STAGE_BYTES_PER_VOXEL = {"hash": 4, "scan": 8}
# kernels per step: hash, scan (2; 3 for voxel tables over 8192 x 4096 entries),
# scatter, big-voxel sort, rank-gather, density, force+integrate, step counter
def kernels_per_step(n_voxels):
    """Our kernels per fused step of a box context: hash, tile reduce, tile
    scan (plus the one-block scan of the tile sums above 8192 tiles), scatter,
    big-voxel sort, rank-gather, density, the force pass's two launches (the
    list path, then the deferred particles) and the step counter."""
    return 10 if (n_voxels + 4095) // 4096 <= 8192 else 11


_T0 = time.perf_counter()


def log(msg):
    """Progress on stderr (the JSON line alone goes to stdout)."""
    print(f"[bench {time.perf_counter() - _T0:8.2f}s] {msg}", file=sys.stderr, flush=True)


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--workload", choices=["config2", "box2m", "config0", "config1"],
                    default="config2")
    ap.add_argument("--e2e-steps", type=int, default=None)
    ap.add_argument("--cpu-steps", type=int, default=10, help="oracle steps of the CPU baseline")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched/served sections")
    ap.add_argument("--batched-scenes", type=int, default=256)
    ap.add_argument("--batched-steps", type=int, default=50)
    ap.add_argument("--tuning", choices=["auto", "default", "warp", "thread"],
                    default="auto", help="launch tuning: autotuned on the scene, the library "
                    "defaults, or the defaults with the named density kernel")
    ap.add_argument("--served-requests", type=int, default=48)
    ap.add_argument("--served-rate", type=float, default=64.0,
                    help="Poisson arrivals per second of the headline served entry")
    ap.add_argument("--served-rates", default="16,64,256",
                    help="comma-separated arrival rates of the served sweep")
    return ap.parse_args()


METRIC = {"config2": "particle-steps/s (4M box, 1 GB300)",
          "box2m": "particle-steps/s (2M box, 1 GB300)",
          "config0": "particle-steps/s (8k box, 1 GB300)",
          "config1": "particle-steps/s (262k pipe start state, 1 GB300)"}


def workload(name):
    from sphgb import scenes
    if name == "config2":
        spec, st = scenes.config2()
        desc = ("4M-particle dam-break box: 128x256x128 jittered lattice, spacing 0.005, "
                "box [0,2]^3, h 0.0112, mass 1.25e-4, rho0 1000, K 3, visc 3.5, g -9.81, "
                "restitution 0.5, dt 5e-4, 32-neighbour cap")
    elif name == "box2m":
        # profiling case: same spacing, h and box as the 4M scene, 2M particles
        # (kernel inputs still above the 129 MB L2)
        spec, st = scenes.box_dam_break(nx=100, ny=200, nz=100, spacing=0.005, jitter=0.0005,
                                        box=(2.0, 2.0, 2.0), h=0.0112, mass=1.25e-4, seed=2)
        desc = "2M-particle dam-break box (100x200x100 lattice, spacing 0.005, h 0.0112, [0,2]^3)"
    elif name == "config1":
        # the pipe flow's start state: ~133 particles per voxel, so the density
        # pass takes its dense-walk path (a profiling and parity case)
        spec, st = scenes.config1()
        desc = ("262k-particle pipe flow start state (3-segment pipe, radii 0.10/0.06/0.10, "
                "h 0.02, ~133 particles per voxel)")
    else:
        spec, st = scenes.config0()
        desc = "8k-particle dam-break box (16x32x16 lattice, h 0.045), 32-neighbour cap"
    return spec, st, desc


def dist_setup(args, backend):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group(backend=backend)
    return rank, world, local


def max_over_ranks(x, world, device=None):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons every 200 ms during a region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm, smax, reasons, samples = [], [], set(), 0
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            samples += 1
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                pass
            for name, val in zip(names, f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": samples}


def measured_peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def committed_inst_per_particle(stage, workload="config2"):
    """Warp instructions per particle of a stage's kernel from the committed ncu
    summary of this workload (its '... N warp instructions per particle.'
    line), or None when there is none."""
    import re
    names = {"force_integrate": "k_integrate", "density": "k_density_wc",
             "rank_gather": "k_rank_gather"}
    p = os.path.join(ROOT, "profiles", f"{names.get(stage, stage)}_{workload}.md")
    try:
        m = re.search(r"(\d+) warp instructions per particle", open(p).read())
        return int(m.group(1)) if m else None
    except OSError:
        return None


def committed_traffic(stage, workload="config2"):
    """DRAM bytes per launch of a stage's kernel from the committed ncu summary
    of this workload (profiles/<kernel>_<workload>.md, line
    'traffic_bytes_per_launch: X'), or None when there is none."""
    names = {"force_integrate": "k_integrate", "density": "k_density_wc",
             "rank_gather": "k_rank_gather"}
    p = os.path.join(ROOT, "profiles", f"{names.get(stage, stage)}_{workload}.md")
    try:
        for line in open(p):
            if line.startswith("traffic_bytes_per_launch:"):
                return float(line.split(":")[1])
    except OSError:
        pass
    return None


def profile_source(stage, workload="config2"):
    """Where the committed per-kernel figures (DRAM traffic, warp
    instructions) come from: the ncu summary file and the case it captured,
    read from its 'case:' line.  These figures are not measured in this run."""
    names = {"force_integrate": "k_integrate", "density": "k_density_wc",
             "rank_gather": "k_rank_gather"}
    rel = os.path.join("profiles", f"{names.get(stage, stage)}_{workload}.md")
    case = None
    try:
        for line in open(os.path.join(ROOT, rel)):
            if line.startswith("case:"):
                case = line.split(":", 1)[1].strip()
                break
    except OSError:
        return None
    return {"file": rel, "case": case, "measured_in_this_run": False}


def scene_facts(batch):
    """Facts of a batch's current state: non-finite particles, mean capped
    and uncapped neighbour counts (self included, the reference's
    get_neighbours counts) and the FP64 conservation sums per scene."""
    import numpy as np
    pos, vel, _ = batch.export_aos_f64()
    bad_pos = int((~pos.isfinite().all(dim=1)).sum())
    bad_vel = int((~vel.isfinite().all(dim=1)).sum())
    cons = batch.conservation()
    cap, unc = batch.neighbour_counts()
    return {"nonfinite_positions": bad_pos, "nonfinite_velocities": bad_vel,
            "neighbours_capped_mean": round(float(np.mean(cap)), 3) if len(cap) else 0.0,
            "neighbours_uncapped_mean": round(float(np.mean(unc)), 3) if len(unc) else 0.0}, cons


def drift(cons0, cons1):
    """Conservation drift between two FP64 conservation records (S, 8):
    total mass change (relative), total momentum change (relative to the
    summed |momentum| scale) and total energy change (relative to |E0|)."""
    import numpy as np
    c0, c1 = np.asarray(cons0).sum(0), np.asarray(cons1).sum(0)
    with np.errstate(invalid="ignore", divide="ignore"):
        p0, p1 = c0[1:4], c1[1:4]
        return {"mass_rel": float(abs(c1[0] - c0[0]) / c0[0]) if c0[0] else 0.0,
                "momentum_change": [float(x) for x in (p1 - p0)],
                "kinetic_start": float(c0[4]), "kinetic_end": float(c1[4]),
                "energy_start": float(c0[6]), "energy_end": float(c1[6]),
                "energy_rel": float(abs(c1[6] - c0[6]) / abs(c0[6])) if c0[6] else None}


def cpu_baseline(spec, state, steps, step_index=0):
    from oracle import ref
    import numpy as np
    sp = ref.params_from_spec(spec)
    pos = np.ascontiguousarray(state.position, dtype=np.float64)
    vel = np.ascontiguousarray(state.velocity, dtype=np.float64)
    pipe = spec.params.pipe.to_numpy() if spec.mode == 'PIPE' else None
    # like the timed GPU steps: every step is a full step of the step-0 state
    t0 = time.perf_counter()
    for _ in range(steps):
        out = ref.step(sp, pos, vel, pipe=pipe, step_index=step_index)
    dt = time.perf_counter() - t0
    return {"value": spec.n * steps / dt, "unit": "particle-steps/s", "cores": ref.num_threads(),
            "kind": "port", "sample": f"{steps} full steps of the {spec.n}-particle scene's step-0 "
                                     f"state ({dt:.1f} s wall, FP64 C/OpenMP restatement)"}, out


def oracle_error(got, want, pos_in=None, dt=None):
    """The GPU step against the FP64 oracle's step of the same input: density
    relative error, position absolute error, and velocity error over the
    largest velocity (cancellation in the force sum makes a per-particle
    relative velocity error meaningless).  For a pipe scene (pos_in and dt
    given), particles whose wall response or respawn fired on either side are
    counted apart: at the wall, an FP32 and an FP64 velocity can land on
    different sides of a decision, so those particles are reported on their own."""
    import numpy as np
    (gp, gv, gr), (wp, wv, wr) = got, want
    ok = np.isfinite(wr) & (wr > 0)
    out = {"density_max_rel": float(np.max(np.abs(gr[ok] - wr[ok]) / wr[ok])),
           "particles_compared": int(ok.sum())}
    free = np.ones(len(gp), dtype=bool)
    if pos_in is not None:
        with np.errstate(invalid="ignore"):
            def fired(v, x):
                return ~np.all(np.abs(pos_in + v * dt - x) <= 1e-9 * np.maximum(np.abs(x), 1.0), axis=1)
            wall = fired(wv, wp) | fired(gv, gp)
        free = ~wall
        out["wall_response_particles"] = int(wall.sum())
        if wall.any():
            dw = np.abs(gp[wall] - wp[wall])
            out["wall_position_max_abs"] = float(np.max(dw))
            # the parity tests' bound for these particles: 1e-3 of |x|
            out["wall_within_1e-3"] = int(np.all(dw <= 1e-3 * np.maximum(np.abs(wp[wall]), 1.0),
                                                 axis=1).sum())
    out["position_max_abs"] = float(np.max(np.abs(gp[free] - wp[free])))
    out["velocity_max_abs_over_max"] = float(np.max(np.abs(gv[free] - wv[free])) / np.max(np.abs(wv)))
    return out


def run_gb300(args):
    import numpy as np
    import torch
    rank, world, local = dist_setup(args, "nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    from sphgb.device import SceneBatch
    spec, state, desc = workload(args.workload)
    n = spec.n
    log(f"workload {args.workload}: {n} particles")
    # launch tuning picked by the autotuner on this scene (results unchanged)
    from sphgb.autotune import Tuning, autotune, summary
    if args.tuning == "auto":
        best, tried = autotune([(spec, state)], steps=3, device=str(dev))
    else:
        best, tried = Tuning(), []
        if args.tuning != "default":
            best.density_variant = {"warp": 0, "thread": 1}[args.tuning]
    log(f"tuning: {best}")
    batch = SceneBatch([spec], device=str(dev))
    best.apply(batch)
    batch.load_states([state])
    # every timed step is a full compute_next_state of the same resident
    # input: the step writes to separate output buffers (see module docstring)
    batch.bind_output(True)
    torch.cuda.synchronize()
    log("state loaded")
    stream = torch.cuda.current_stream(dev)
    for _ in range(max(args.warmup, 0)):
        batch.step(1, use_graph=True)      # first call captures the one-step graph
    torch.cuda.synchronize()
    log(f"{args.warmup} warm-up steps done")
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    barrier(world)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            batch.step(1, use_graph=True)
        e1.record(stream)
        torch.cuda.synchronize()
    barrier(world)
    ms = e0.elapsed_time(e1)
    ms = max_over_ranks(ms, world, dev)
    value = n * args.steps * world / (ms / 1e3)
    clocks = clk.summary()
    log(f"timed {args.steps} steps: {ms:.3f} ms")

    # per-stage CUDA-event times (same kernels, no graph) -> dominant kernel roofline
    stages = batch.step_profiled(min(args.steps, 10))
    log(f"stage ms: {stages}")
    dom = max(("density", "force_integrate", "rank_gather", "hash", "scatter"),
              key=lambda k: stages[k])
    peak, peak_kind = measured_peak_hbm()
    b_alg = STAGE_BYTES_PER_PARTICLE[dom] * n + STAGE_BYTES_PER_VOXEL.get(dom, 0) * batch.n_voxels
    achieved = b_alg / (stages[dom] / 1e3) / 1e9
    step_bytes = (192 * n + 12 * batch.n_voxels)
    roofline = {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak,
                "peak_kind": peak_kind, "unit": "GB/s", "frac": round(achieved / peak, 4),
                "traffic": committed_traffic(dom, args.workload),
                "traffic_source": profile_source(dom, args.workload),
                "algorithmic_bytes": b_alg, "kernel_ms": round(stages[dom], 4),
                "kernel_ms_source": "CUDA events around the kernel in this run"}
    step_roofline = {"algorithmic_bytes_per_step": step_bytes,
                     "achieved": round(step_bytes / (ms / args.steps / 1e3) / 1e9, 1),
                     "frac": round(step_bytes / (ms / args.steps / 1e3) / 1e9 / peak, 4),
                     "stage_ms": {k: round(v, 4) for k, v in stages.items()}}

    # The dominant kernel is bound by instruction issue, not DRAM: its warp
    # instructions (per particle, from the committed ncu summary) over its
    # live time, against one warp instruction per cycle on each of the SMs' 4
    # sub-partitions at the SM clock sampled during the timed region.
    ipp = committed_inst_per_particle(dom, args.workload)
    issue_roofline = None
    if ipp and clocks.get("sm_mhz"):
        got = ipp * n / (stages[dom] / 1e3)
        top = sms * 4 * clocks["sm_mhz"] * 1e6
        issue_roofline = {"kernel": dom, "warp_instructions_per_particle": ipp,
                          "warp_instructions_source": profile_source(dom, args.workload),
                          "achieved": round(got / 1e12, 4), "peak": round(top / 1e12, 4),
                          "unit": "1e12 warp instructions/s", "frac": round(got / top, 4)}

    # per-step working set: state and sort buffers (~100 B), neighbour list
    # (128 B) and force inputs (32 B) per particle, 12 B per voxel
    ws = 260 * n + 12 * batch.n_voxels
    l2_note = (f"inputs larger than L2 (~{ws / 1e9:.2f} GB per step > 129 MB)" if ws > 129e6 else
               f"working set ~{ws / 1e6:.0f} MB fits in the 129 MB L2")

    # free-running simulation from the same start (informational): the
    # reference's formulas make this scene blow up within a few steps
    batch.bind_output(False)
    k_free = min(args.steps, 10)
    cons0 = batch.conservation()
    f0 = torch.cuda.Event(enable_timing=True)
    f1 = torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    batch.step(k_free, use_graph=False)
    f1.record(stream)
    torch.cuda.synchronize()
    facts, cons1 = scene_facts(batch)
    free = {"steps": k_free, "ms_per_step": f0.elapsed_time(f1) / k_free, **facts,
            "conservation_drift": drift(cons0, cons1)}
    log(f"free running: {free}")

    # end to end through the C ABI host-buffer entry point: each step copies
    # the same FP64 AoS input from pinned host memory and the result back
    k_e2e = args.e2e_steps if args.e2e_steps is not None else min(args.steps, 10)
    pin = lambda shape: torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()  # noqa
    h_pos, h_vel = pin((n, 3)), pin((n, 3))
    o_pos, o_vel, o_rho = pin((n, 3)), pin((n, 3)), pin((n,))
    h_pos[:] = state.position
    h_vel[:] = state.velocity
    # warm-up: the first six calls run the entry point's three force-pass orders
    # (slot order, particle-order ranges, buckets pipelined behind the density
    # pass) once each, then time them; later calls use the fastest
    for _ in range(6):
        batch.compute_next_state_host(h_pos, h_vel, o_pos, o_vel, o_rho)
    barrier(world)
    t0 = time.perf_counter()
    for i in range(k_e2e):
        batch.compute_next_state_host(h_pos, h_vel, o_pos, o_vel, o_rho)
    e2e_s = time.perf_counter() - t0
    e2e_s = max_over_ranks(e2e_s, world, dev)
    # the scene's step counter of the last call (keys a pipe's respawn draws)
    e2e_step = int(batch.steps[0].item()) - 1
    log(f"e2e {k_e2e} steps: {e2e_s:.3f} s")
    e2e = {"value": n * k_e2e * world / e2e_s, "unit": "particle-steps/s",
           "h2d_bytes_per_step": 48 * n, "d2h_bytes_per_step": 56 * n, "steps": k_e2e,
           "warmup_calls": 6, "api": "sphgb_compute_next_state_host"}
    assert np.isfinite(o_rho).all()

    out = {"metric": METRIC[args.workload],
           "value": value, "unit": "particle-steps/s", "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
           "config": {"workload": desc, "particles": n, "voxels": batch.n_voxels,
                      "l2": l2_note, "sms": sms,
                      "parallelism": f"replicas x{world}", "graph": "one CUDA graph per step",
                      "input": "every step is a full step of the same resident step-0 state"},
           "e2e": e2e, "roofline": roofline, "issue_roofline": issue_roofline,
           "step_roofline": step_roofline,
           "free_running": free,
           "autotune": {"chosen": {"density": {0: "warp", 1: "thread"}[best.density_variant],
                                   "sort_block": best.sort_block, "big_voxel": best.big_voxel},
                        "ms_per_step": summary(tried)},
           "clocks": clocks, "gpu_launches": kernels_per_step(batch.n_voxels) * args.steps}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"], want = cpu_baseline(spec, state, max(args.cpu_steps, 1),
                                                 step_index=e2e_step)
        log(f"cpu baseline: {out['cpu_baseline']}")
        # the end-to-end outputs are one step of the same step-0 state, at the
        # step index of the last call
        pipe_scene = spec.mode == 'PIPE'
        out["oracle_err"] = oracle_error(
            (o_pos, o_vel, o_rho), want,
            pos_in=np.asarray(state.position, dtype=np.float64) if pipe_scene else None,
            dt=float(np.float32(1.0 / spec.params.fps)) if pipe_scene else None)
        log(f"error against the FP64 oracle: {out['oracle_err']}")
    batch.close()
    if not args.no_batched and args.workload == "config2":
        out["batched"] = batched_section(args)
        out["served"] = served_section(args)
        out["pipe_flow"] = pipe_section(args)
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def batched_section(args):
    """Batched scenes (256 boxes, N log-uniform in [1024, 65536], 50 steps):
    one graph launch for all scenes against one scene per launch."""
    import numpy as np
    from oracle import ref
    from sphgb import scenes
    from sphgb.batch import particle_steps, run_batched, run_plain
    pairs = scenes.config3_specs(n_scenes=args.batched_scenes, seed=3)
    steps = args.batched_steps
    work = particle_steps([p[0] for p in pairs], steps)
    tb, sb = run_batched(pairs, steps, repeats=2)
    log(f"batched: {len(pairs)} scenes, {work} particle-steps in {tb:.4f} s")
    tp, sp_ = run_plain(pairs, steps)
    log(f"plain (one scene per launch): {tp:.4f} s")
    tg, _ = run_plain(pairs, steps, use_graph=True)
    log(f"plain with one graph per scene: {tg:.4f} s")
    same = all(np.array_equal(a.position, b.position) and np.array_equal(a.density, b.density)
               for a, b in zip(sb, sp_))
    # density error of the first step against the FP64 oracle, 8 scenes
    _, one = run_batched(pairs[:8], 1, repeats=0)
    err = 0.0
    for (spec, st), got in zip(pairs[:8], one):
        _, _, rho = ref.step(ref.params_from_spec(spec), st.position, st.velocity)
        err = max(err, float(np.max(np.abs(got.density - rho) / rho)))
    # what the workload's state is at its end: the same run again, untimed
    from sphgb.device import SceneBatch
    b = SceneBatch([p[0] for p in pairs])
    b.load_states([p[1] for p in pairs])
    cons0 = b.conservation()
    b.step(steps, use_graph=True)
    facts, cons1 = scene_facts(b)
    b.close()
    return {"scenes": len(pairs), "particles": sum(p[0].n for p in pairs), "steps": steps,
            "value": work / tb, "unit": "particle-steps/s",
            "plain_value": work / tp, "plain_graph_value": work / tg,
            "vs_plain": tb and tp / tb, "vs_plain_graph": tg / tb,
            "identical_to_plain": bool(same), "density_rel_err_vs_fp64": err,
            "at_end": facts, "conservation_drift": drift(cons0, cons1),
            "graph": "all scenes and steps in one CUDA graph launch"}


def pipe_section(args):
    """Pipe flow (262,144 particles in the 3-segment pipe, FP64 position
    accumulator and pipe wall response with respawns): the 1,000 steps of the
    workload, free-running from the generated start state, 10 steps per
    graph launch, CUDA events around all of them."""
    import torch
    from sphgb import scenes
    from sphgb.device import SceneBatch
    spec, st = scenes.config1()
    b = SceneBatch([spec])
    b.load_states([st])
    b.step(10, use_graph=True)      # captures the 10-step graph
    b.load_states([st])             # back to the start state and step 0
    start_facts, cons0 = scene_facts(b)
    torch.cuda.synchronize()
    steps = 1000
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps // 10):
        b.step(10, use_graph=True)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    facts, cons1 = scene_facts(b)
    b.close()
    log(f"pipe flow: {spec.n} particles x {steps} steps in {ms:.1f} ms")
    return {"particles": spec.n, "steps": steps, "value": spec.n * steps / (ms / 1e3),
            "unit": "particle-steps/s", "ms_per_step": ms / steps,
            "at_start": start_facts, "at_end": facts,
            "mass_fp64": float(cons1[0][0]), "conservation_drift": drift(cons0, cons1),
            "note": (f"under the reference's formulas this flow blows up: after {steps} steps "
                     f"{facts['nonfinite_velocities']} of {spec.n} particles have a non-finite "
                     f"velocity; the pipe wall response sends their non-finite positions back "
                     f"to the inlet each step (a finite respawn), so they crowd the inlet in "
                     f"dense clusters ({facts['neighbours_uncapped_mean']:.0f} neighbours within "
                     f"h on average); the rate is that of this trajectory, not of the start state"),
            "graph": "10 steps per CUDA graph launch"}


def served_section(args):
    """Served workload: Poisson arrivals, 70 % box / 30 % pipe, N log-uniform
    in [2048, 524288], steps uniform in [100, 2000], 150 GB HBM budget;
    continuous batching against serving the same requests one at a time.
    The arrival rate is swept: the same requests (sizes, steps, start states)
    arrive at each rate, their arrival times scaled."""
    import dataclasses
    from sphgb.device import SceneBatch
    from sphgb.serve import SceneServer, poisson_requests
    import torch
    base = poisson_requests(1.0, args.served_requests, seed=4)     # arrivals at rate 1
    work = sum(r.spec.n * r.steps for r in base)
    plain_s = 0.0
    plain_each = []                 # (particle-steps, seconds) per request served alone
    for r in base:
        b = SceneBatch([r.spec])
        b.load_states([r.state])
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        b.step(r.steps)
        e1.record()
        torch.cuda.synchronize()
        t = e0.elapsed_time(e1) / 1e3
        plain_s += t
        plain_each.append((r.spec.n * r.steps, t))
        b.close()
    log(f"served one at a time: {plain_s:.3f} s of GPU time for {work} particle-steps")
    rates = sorted({float(x) for x in args.served_rates.split(",")} | {args.served_rate})
    rates.append(float("inf"))     # every request at time 0: the server saturated
    sweep = []
    head_reqs = []
    for rate in rates:
        reqs = [dataclasses.replace(r, arrival=r.arrival / rate if rate != float("inf") else 0.0)
                for r in base]
        if rate == args.served_rate:
            head_reqs = reqs
        server = SceneServer(hbm_budget_bytes=150e9, max_tick_steps=64)
        st = server.run(reqs)
        server.close()
        log(f"served at {rate:g}/s: {st.requests} requests in {st.wall_s:.3f} s, "
            f"GPU busy {st.gpu_busy:.2f}, re-packs {st.repack_s:.3f} s, "
            f"p50 {st.pct(50):.3f} s p99 {st.pct(99):.3f} s, max active {st.max_active}")
        sweep.append({"rate_per_s": rate if math.isfinite(rate) else "all at t=0",
                      "value": st.throughput, "wall_s": st.wall_s,
                      "p50_latency_s": st.pct(50), "p99_latency_s": st.pct(99),
                      "max_active": st.max_active, "ticks": st.ticks, "repacks": st.repacks,
                      "gpu_busy": round(st.gpu_busy, 4), "gpu_s": st.gpu_s,
                      "repack_s": st.repack_s,
                      "vs_plain": st.throughput / (work / plain_s)})
    head = next(s for s in sweep if s["rate_per_s"] == args.served_rate)
    sat = sweep[-1]                          # every request at time 0
    # density error of the mix's first step against the FP64 oracle, the first
    # 8 requests (box and pipe scenes as they come), through one batch
    import numpy as np
    from oracle import ref
    b = SceneBatch([r.spec for r in base[:8]])
    b.load_states([r.state for r in base[:8]])
    b.step(1)
    got = b.states()
    b.close()
    err = 0.0
    for r, g in zip(base[:8], got):
        pipe = r.spec.params.pipe.to_numpy() if r.spec.mode == 'PIPE' else None
        _, _, rho = ref.step(ref.params_from_spec(r.spec), r.state.position, r.state.velocity,
                             pipe=pipe)
        ok = rho > 0
        err = max(err, float(np.max(np.abs(g.density[ok] - rho[ok]) / rho[ok])))
    bad_pos = sum(int((~np.isfinite(r.result.position).all(1)).sum())
                  for r in head_reqs if r.result is not None)
    bad_vel = sum(int((~np.isfinite(r.result.velocity).all(1)).sum())
                  for r in head_reqs if r.result is not None)
    # work share of the requests that run alone at no less than half the
    # saturated served rate: batching cannot speed those up by more than 2x
    fast = sum(w for w, t in plain_each if w / t >= 0.5 * sat["value"])
    return {"requests": len(base), "particle_steps": work, "unit": "particle-steps/s",
            "plain_value": work / plain_s, "hbm_budget_gb": 150, **head, "sweep": sweep,
            "saturated": {"value": sat["value"], "vs_plain": sat["vs_plain"],
                          "gpu_busy": sat["gpu_busy"],
                          "how": "the same requests all arriving at time 0"},
            "work_share_fast_alone": fast / work,
            "density_rel_err_vs_fp64": err,
            "box_requests": sum(r.spec.mode == 'BOX' for r in base),
            "pipe_requests": sum(r.spec.mode == 'PIPE' for r in base),
            "results_nonfinite_positions": bad_pos, "results_nonfinite_velocities": bad_vel,
            "nonfinite_note": ("the reference's formulas blow the pipe flows up: their velocities "
                               "go non-finite and the wall response respawns the particles at the "
                               "inlet every step")}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import numpy as np
    from oracle import ref
    spec, state, desc = workload(args.workload)
    sp = ref.params_from_spec(spec)
    pipe = spec.params.pipe.to_numpy() if spec.mode == 'PIPE' else None
    pos = np.ascontiguousarray(state.position, dtype=np.float64)
    vel = np.ascontiguousarray(state.velocity, dtype=np.float64)
    # like the GPU arm, every step is a full step of the same step-0 state
    for _ in range(max(args.warmup, 0)):
        ref.step(sp, pos, vel, pipe=pipe, step_index=0)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ref.step(sp, pos, vel, pipe=pipe, step_index=0)
    dt = time.perf_counter() - t0
    value = spec.n * args.steps / dt
    cores = ref.num_threads()
    out = {"impl": "reference",
           "metric": METRIC[args.workload],
           "value": value, "unit": "particle-steps/s", "n_gpus": int(os.environ.get("WORLD_SIZE", 1)),
           "steps": args.steps, "warmup": max(args.warmup, 0), "ms_per_step": dt / args.steps * 1e3,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic",
           "config": {"workload": desc, "particles": spec.n, "parallelism": "host cores"},
           "cpu_baseline": {"value": value, "unit": "particle-steps/s", "cores": cores,
                            "kind": "port",
                            "sample": f"{args.steps} full steps of the {spec.n}-particle "
                                      "scene's step-0 state"},
           "e2e": {"value": value, "unit": "particle-steps/s", "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def main():
    args = parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
