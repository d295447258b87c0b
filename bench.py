"""Benchmark of the Physarum step on GB300 (one JSON line on rank 0).

Workload (default): the plain method at scale -- a toroidal 4096x4096 binary32
trail and 16,777,216 agents (x, y ~ U[0,4096), heading ~ U[0,2pi),
speed ~ U[1,2] px/step, seed 0), sensor angle 0.4 rad, distance 9 px, turn
0.3 rad/step, jitter 0.05 rad, deposition 1.0, multiplicative decay 0.97,
diffusion 0.5 through a 3-tap sigma=1 Gaussian.  A "step" is one simulation
step (agents sense/turn/move/deposit, then fused deposit-fold + decay +
diffuse).  Data are synthetic (seeded), there is no dataset.

  value   agent-steps/s with the state resident in HBM, the step loop
          replayed from CUDA graphs, timed with CUDA events on the
          simulation's stream;
  e2e     the same metric through the C ABI with host buffers: every step
          uploads the parameter block (the reference's per-frame uniform
          write) and downloads the new trail into pinned host memory;
  roofline  the dominant kernel's algorithmic bytes per launch over its
          CUDA-event launch time, against the measured HBM copy bandwidth;
  cpu_baseline  the CPU oracle (a binary32 restatement of the reference
          shader) on a bounded sample of the same workload, threaded over the
          host's cores.

`--impl reference` times that CPU implementation alone on the same workload
and metric (the reference's own GPU path needs wgpu and a graphics stack,
neither of which exists on the box).  Under torchrun every rank runs an
independent replica (a single colony does not shard), value = the sum.
"""
import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "slime-mold_gb300"))

CONFIGS = {
    # name: (W, H, n_agents, speed_lo, speed_hi, sensor_distance)
    "plain-4096": (4096, 4096, 16_777_216, 1.0, 2.0, 9.0),
    "plain-512": (512, 512, 65_536, 1.0, 2.0, 9.0),
    "plain-8192": (8192, 8192, 67_108_864, 1.5, 3.0, 18.0),
    "adjoint-1024": (1024, 1024, 1_048_576, 1.0, 2.0, 9.0),
}
EXTRA_CONFIGS = ["ensemble-64", "adjoint-1024"]


def metric_name(cfg_name):
    W, H, n = CONFIGS[cfg_name][:3]
    return f"agent-steps/s (plain step, {n:,} agents on {W}x{H})"


def agents_kernel_name(shape):
    """Kernel of agent-shape table entry `shape` (agents.cu): 9-11 and 13-15
    are the persistent kernel (13-15 sample through the trail texture)."""
    return "agents_persistent_kernel" if shape in (9, 10, 11, 13, 14, 15) else "agents_kernel"


def trail_kernel_name(tile, blur_mode):
    """Kernel of trail-tile table entry `tile` (trail.cu): 10 is the
    tensor-copy tile, 7-9 stream rows, 0-6 are shared-memory tiles of the box
    or Gaussian kernel."""
    if tile == 10:
        return "trail_tma_kernel"
    if tile >= 7:
        return "trail_stream_kernel"
    return "trail_gauss_kernel" if blur_mode == 1 else "trail_box3_kernel"


# ncu summaries (profiles/) that hold the DRAM traffic of one launch of a
# kernel on a workload: the "traffic (read + write) per launch" row.
TRAFFIC_PROFILES = {
    ("plain-4096", "agents_persistent_kernel"): "agents_kernel_plain-4096.md",
    ("plain-4096", "trail_stream_kernel"): "trail_stream_kernel_plain-4096.md",
    ("plain-8192", "agents_persistent_kernel"): "agents_kernel_plain-8192.md",
    ("plain-8192", "trail_stream_kernel"): "trail_stream_kernel_plain-8192.md",
    ("plain-8192", "trail_tma_kernel"): "trail_tma_kernel_plain-8192.md",
}


def profiled_traffic(workload, kernel):
    """dram__bytes_read.sum + dram__bytes_write.sum of one launch, in bytes,
    from the committed ncu summary of that kernel on that workload, if the
    summary's capture is of the same kernel; else None."""
    import re
    name = TRAFFIC_PROFILES.get((workload, kernel))
    if not name:
        return None, None
    path = os.path.join(ROOT, "profiles", name)
    try:
        with open(path) as f:
            text = f.read()
    except OSError:
        return None, None
    if not text.startswith("# " + kernel):
        return None, None
    m = re.search(r"traffic \(read \+ write\) per launch \| ([0-9.]+) MB", text)
    if not m:
        return None, None
    return float(m.group(1)) * 1e6, "profiles/" + name


def reference_dispatch_visited(n):
    """Agents the reference's dispatch updates: min(ceil(n / 64), 65535) x wy
    workgroups of 64, invocation (gx, gy) updating agent gx + 65535 gy, reach
    every index below (wy - 1) 65535 + 64 wx."""
    groups = -(-n // 64)
    wx = min(groups, 65535)
    wy = -(-groups // wx)
    return min(n, (wy - 1) * 65535 + 64 * wx)


def make_params(W, H, speed_lo, speed_hi, dist):
    import slime_gb300 as sg
    p = sg.SlimeParams()
    p.width, p.height = W, H
    p.decay_factor = 0.97
    p.agent_jitter = 0.05
    p.agent_speed_min, p.agent_speed_max = speed_lo, speed_hi
    p.agent_turn_speed = 0.3
    p.agent_sensor_angle = 0.4
    p.agent_sensor_distance = dist
    p.diffusion_rate = 0.5
    p.pheromone_deposition_amount = 1.0
    p.blur_radius = 1.0
    p.blur_sigma = 1.0
    p.time_step = 0.016
    p.decay_mode = sg.DECAY_MULTIPLY
    p.blur_mode = sg.BLUR_GAUSS
    return p


def make_agents(n, W, H, lo, hi, seed=0):
    rng = np.random.default_rng(seed)
    a = np.empty((n, 4), np.float32)
    a[:, 0] = rng.uniform(0, W, n)
    a[:, 1] = rng.uniform(0, H, n)
    a[:, 2] = rng.uniform(0, 2 * np.pi, n)
    a[:, 3] = rng.uniform(lo, hi, n)
    np.minimum(a[:, 0], np.nextafter(np.float32(W), np.float32(0)), out=a[:, 0])
    np.minimum(a[:, 1], np.nextafter(np.float32(H), np.float32(0)), out=a[:, 1])
    return a


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    @staticmethod
    def smi_id(index):
        """nvidia-smi's name for CUDA device `index` of this process: the
        index-th entry of CUDA_VISIBLE_DEVICES (an index or a UUID) when that
        is set, since nvidia-smi sees every GPU of the machine."""
        vis = [v.strip() for v in os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",") if v.strip()]
        return vis[index] if 0 <= index < len(vis) else str(index)

    def __enter__(self):
        try:
            ident = self.smi_id(self.index)
            if ident != str(self.index):  # keep the plain index if nvidia-smi does not know that name
                probe = subprocess.run(["nvidia-smi", f"--id={ident}", "--query-gpu=index", "--format=csv,noheader"],
                                       capture_output=True, timeout=20)
                ident = ident if probe.returncode == 0 else str(self.index)
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={ident}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            time.sleep(0.2)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baseline(params, W, H, n, agents, budget_s=12.0, max_steps=20):
    """Time the CPU oracle on the full workload for a bounded number of steps."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    threads = oracle.num_threads()
    a = agents.copy()
    t = np.zeros((H, W), np.float32)
    steps = 0
    t0 = time.perf_counter()
    while steps < max_steps:
        oracle.run(params, W, H, a, t, 1, threads=threads)
        steps += 1
        if time.perf_counter() - t0 > budget_s:
            break
    dt = time.perf_counter() - t0
    return {"value": n * steps / dt, "unit": "agent-steps/s", "cores": threads, "kind": "port",
            "sample": f"{steps} full steps of the {W}x{H}/{n}-agent workload from the seeded initial state "
                      f"({dt:.1f} s), CPU oracle (binary32 restatement of compute.wgsl), OpenMP {threads} threads",
            "cells_per_s": W * H * steps / dt}


def ensemble_colonies(seed=1, k=64):
    """64 independent colonies: side ~ U{256, 512, 1024, 2048}, density ~ U[0.25, 4]
    agents/cell, per-colony sensor angle [0.2,0.8], distance [4,20], turn
    [0.1,0.6], jitter [0,0.1], decay [0.90,0.995], diffusion [0.1,0.9],
    deposition [0.5,2.0]; fp32, seed 1."""
    import slime_gb300 as sg
    rng = np.random.default_rng(seed)
    cols = []
    for j in range(k):
        side = int(rng.choice([256, 512, 1024, 2048]))
        n = int(side * side * rng.uniform(0.25, 4.0))
        p = make_params(side, side, 1.0, 2.0, float(rng.uniform(4, 20)))
        p.agent_sensor_angle = float(rng.uniform(0.2, 0.8))
        p.agent_turn_speed = float(rng.uniform(0.1, 0.6))
        p.agent_jitter = float(rng.uniform(0.0, 0.1))
        p.decay_factor = float(rng.uniform(0.90, 0.995))
        p.diffusion_rate = float(rng.uniform(0.1, 0.9))
        p.pheromone_deposition_amount = float(rng.uniform(0.5, 2.0))
        cols.append((side, side, n, p, j))
    return cols


def ensemble_comparisons(args, cols, cells, agents_total, R):
    """The ensemble's colonies one plain Simulation after the other, the
    plain 4096^2 per-cell throughput, and the plain path's per-agent and
    per-cell costs (for the ensemble at equal work)."""
    import torch
    import slime_gb300 as sg
    # the same colonies, one plain Simulation after the other
    seq_steps = max(3, min(args.steps, 50))
    seq_ms = 0.0
    seq_reorder_ms = 0.0
    for W, H, n, p, seed in cols:
        sim = sg.Simulation(W, H, n, p)
        sim.seed_agents(1000 + seed)
        sim.set_options(reorder_every=args.reorder_every)
        sim.autotune(2)
        sim.step(3)
        sim.prepare_steps(seq_steps)
        sim.sync()
        st = torch.cuda.ExternalStream(sim.stream_ptr())
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(st)
        sim.step(seq_steps)
        b.record(st)
        sim.sync()
        # charged as the ensemble's window: reorders inside it out, each
        # step's share in
        r_ms = sim.profile_reorder(1) if R else 0.0
        r_in = sum(1 for s in range(3, 3 + seq_steps) if R and s % R == 0)
        seq_reorder_ms += seq_steps * r_ms / R if R else 0.0
        seq_ms += a.elapsed_time(b) - r_in * r_ms + (seq_steps * r_ms / R if R else 0.0)
        sim.close()
    seq_cells = cells * seq_steps / (seq_ms / 1e3)
    # plain single-colony per-cell throughput at 4096^2 (short run)
    W, H, n, lo, hi, dist = CONFIGS["plain-4096"]
    sim = sg.Simulation(W, H, n, make_params(W, H, lo, hi, dist))
    sim.seed_agents(0)
    sim.set_options(reorder_every=200)
    sim.autotune(3)
    sim.step(5)
    sim.prepare_steps(50)
    sim.sync()
    st = torch.cuda.ExternalStream(sim.stream_ptr())
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(st)
    sim.step(50)
    b.record(st)
    sim.sync()
    plain_cells = W * H * 50 / (a.elapsed_time(b) / 1e3)
    # per-agent and per-cell cost of the plain path (direct launches), to
    # compare the ensemble at equal work: its colonies average ~2 agents per
    # cell against 1 in the plain workload, so per-cell rates alone favour
    # the plain path
    pa_ms, pt_ms, _ = sim.profile_steps(50)
    t_agent = pa_ms / 50 / n
    t_cell = pt_ms / 50 / (W * H)
    plain_model_ms = agents_total * t_agent + cells * t_cell
    sim.close()
    return {"seq_cells": seq_cells, "seq_reorder_ms_per_step": seq_reorder_ms / seq_steps,
            "plain_cells": plain_cells, "plain_model_ms": plain_model_ms}


def run_ensemble(args):
    """Batched ensemble over 64 colonies (the autotuned engine: lanes of
    single-colony kernel chains in one CUDA graph, or one cooperative launch
    per step), against the same colonies run one after the other with the
    plain path, and against the plain 4096^2 per-cell throughput."""
    import torch
    import slime_gb300 as sg
    torch.cuda.set_device(0)
    cols = ensemble_colonies(k=args.colonies)
    cells = sum(c[0] * c[1] for c in cols)
    agents_total = sum(c[2] for c in cols)
    ens = sg.Ensemble([c[0] for c in cols], [c[1] for c in cols], [c[2] for c in cols], [c[3] for c in cols])
    for j, (W, H, n, p, seed) in enumerate(cols):
        ens.seed_agents(j, 1000 + seed)
    ens.set_reorder(args.reorder_every, 2)
    if args.ensemble_engine == "auto":
        ens.autotune(2)
    elif args.ensemble_engine == "lanes":  # the autotuner's usual pick, fixed (short profiler runs)
        ens.set_engine(sg.ENSEMBLE_LANES, 13, 9, 0)
    else:
        ens.set_engine(sg.ENSEMBLE_COOPERATIVE)
        ens.set_shape(16, 4, 4)
    info = ens.info()
    if info.engine == sg.ENSEMBLE_LANES:
        tuned = {"engine": "lanes", "what": "each colony a chain of the single-colony kernels on its own "
                 "capture lane, one CUDA graph per chunk of steps",
                 "agent_shape": info.lane_agent_shape, "trail_tile": info.lane_trail_tile}
    else:
        tuned = {"engine": "cooperative", "what": "one cooperative persistent launch per step",
                 "strip_rows": info.strip_rows, "grid_blocks": info.grid_blocks,
                 "agents_per_thread": info.agents_per_thread}
    stream = torch.cuda.ExternalStream(ens.stream_ptr())
    ens.step(args.warmup)
    ens.prepare_steps(args.steps)
    ens.sync()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    l0 = ens.launch_count()
    s0 = ens.info().steps_done
    with ClockSampler(0) as clocks:
        e0.record(stream)
        ens.step(args.steps)
        e1.record(stream)
        ens.sync()
    window_ms = e0.elapsed_time(e1)
    launches = ens.launch_count() - l0
    info = ens.info()
    tuned["lanes"] = info.lanes
    tuned["marks_colonies"] = info.marks_colonies
    # every step pays its share of the Morton reorders (one per reorder_every
    # steps), whether or not one fell inside the window
    R = args.reorder_every
    reorders_in = sum(1 for s in range(s0, s0 + args.steps) if R and s % R == 0)
    reorder_ms = ens.profile_reorder(3) / 3 if R else 0.0
    ms = window_ms - reorders_in * reorder_ms + (args.steps * reorder_ms / R if R else 0.0)
    ens_cells = cells * args.steps / (ms / 1e3)
    ens_agents = agents_total * args.steps / (ms / 1e3)
    del ens
    cmp = {} if args.no_compare else ensemble_comparisons(args, cols, cells, agents_total, R)
    line = {
        "metric": "trail cells/s (batched ensemble, 64 colonies)",
        "value": ens_cells, "unit": "cells/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": f"ensemble-{len(cols)}", "colonies": len(cols), "cells": cells, "agents": agents_total,
                   "sides": sorted(set(c[0] for c in cols)), "reorder_every": args.reorder_every},
        "agent_steps_per_s": ens_agents, "window_ms_per_step": window_ms / args.steps,
        "reorder": {"ms": reorder_ms, "every": R, "ms_per_step": reorder_ms / R if R else 0.0,
                    "in_timed_window": reorders_in,
                    "sequential_ms_per_step": cmp.get("seq_reorder_ms_per_step"),
                    "what": "ms_per_step = timed window - reorders inside it + K x (one reorder's time / "
                            "reorder_every), the sequential runs charged the same way"},
        "tuned": tuned, "gpu_launches": launches, "clocks": clocks.summary(),
    }
    if cmp:
        line.update({
            "sequential_plain_cells_per_s": cmp["seq_cells"], "ensemble_over_sequential": ens_cells / cmp["seq_cells"],
            "plain_4096_cells_per_s": cmp["plain_cells"],
            "ensemble_over_plain_per_cell": ens_cells / cmp["plain_cells"],
            "plain_path_ms_for_this_work": cmp["plain_model_ms"],
            "ensemble_over_plain_equal_work": cmp["plain_model_ms"] / (ms / args.steps)})
    print(json.dumps(line), flush=True)


def run_adjoint(args):
    """Adjoint of the trail chain at 1024^2 / 1,048,576 agents: the forward
    with checkpoints every 50 steps against the backward (segment replay +
    adjoint stencil), 2000 steps; loss 0.5*||T_2000 - T_target||^2 with the
    target from a run at decay 0.975, diffusion 0.55, deposition 1.1."""
    import torch
    import slime_gb300 as sg
    torch.cuda.set_device(0)
    W, H, n, lo, hi, dist = CONFIGS["adjoint-1024"]
    steps = args.adjoint_steps
    p = make_params(W, H, lo, hi, dist)
    agents = make_agents(n, W, H, lo, hi, seed=0)
    sim = sg.Simulation(W, H, n, p)
    # target
    pt = p.copy()
    pt.decay_factor, pt.diffusion_rate, pt.pheromone_deposition_amount = 0.975, 0.55, 1.1
    sim.set_params(pt)
    sim.upload_agents(agents)
    sim.step(steps)
    target = sim.download_trail()
    sim.set_params(p)
    sim.upload_agents(agents)
    sim.clear_trail()
    sim.set_options(reorder_every=0)
    sim.autotune(2)
    sim.upload_agents(agents)
    sim.clear_trail()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sim.forward_record(steps, 50)
    t_fwd = time.perf_counter() - t0
    tn = sim.download_trail()
    g = tn - target
    loss = 0.5 * float((g.astype(np.float64) ** 2).sum())
    t0 = time.perf_counter()
    grads, d0 = sim.backward(g)
    t_bwd = time.perf_counter() - t0
    # plain forward (graphs, no checkpoints) for reference
    sim.upload_agents(agents)
    sim.clear_trail()
    sim.prepare_steps(steps)
    sim.sync()
    t0 = time.perf_counter()
    sim.step(steps)
    sim.sync()
    t_plain = time.perf_counter() - t0
    line = {
        "metric": f"adjoint cost / forward cost (1024x1024, 1,048,576 agents, {steps} steps, checkpoints every 50)",
        "value": t_bwd / t_fwd, "unit": "ratio", "n_gpus": 1, "steps": steps, "warmup": 0,
        "ms_per_step": 1000 * t_bwd / steps, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": "adjoint-1024", "width": W, "height": H, "n_agents": n, "ckpt_every": 50},
        "forward_record_s": t_fwd, "backward_s": t_bwd, "plain_forward_s": t_plain,
        "backward_over_plain_forward": t_bwd / t_plain, "loss": loss,
        "grads": {"d_decay_factor": grads.d_decay_factor, "d_diffusion_rate": grads.d_diffusion_rate,
                  "d_deposition_amount": grads.d_deposition_amount, "d_trail0_abs_max": float(np.abs(d0).max())},
    }
    print(json.dumps(line), flush=True)


def workload_config(args, ws=1, cfg_name=None):
    """The `config` object of a plain-workload line, the same for both arms."""
    cfg_name = cfg_name or args.config
    W, H, n = CONFIGS[cfg_name][:3]
    n_visited = reference_dispatch_visited(n) if args.dispatch == "reference" else n
    return {"workload": cfg_name, "width": W, "height": H, "n_agents": n,
            "sensor_angle": 0.4, "sensor_distance": CONFIGS[cfg_name][5], "turn": 0.3, "jitter": 0.05,
            "speed": list(CONFIGS[cfg_name][3:5]), "deposition": 1.0,
            "decay": "multiply 0.97", "blur": "gauss r=1 sigma=1 rate 0.5",
            "sensor_mode": "shader: cos/sin(angle -/+ a) as compute.wgsl:75-86",
            "reorder_every": args.reorder_every, "graph_chunk": 50,
            "l2_persist": not args.no_l2_persist,
            "l2": f"agent state {16 * n / 1e6:.0f} MB streamed per step (> 129 MB L2, inputs larger "
                  f"than L2 between timed steps); trail {4 * W * H / 1e6:.0f} MB"
                  + (" (fits the 129 MB L2; a persisting window over it is the autotuner's choice, "
                     "see tuned.l2_window_passes)" if 4 * W * H < 129e6 else " (exceeds L2)"),
            "parallelism": f"replicas x{ws}",
            "dispatch": "every agent once per step" if args.dispatch == "each" else
                        f"the reference's dispatch: {n_visited} of {n} agents updated per step"}


def measure_plain(sim, stream, params, agents, args, barrier, local, torch):
    """One parameter set on the plain workload: the seeded initial state,
    autotuning, W untimed warm-up steps, then K steps replayed from CUDA
    graphs, timed with CUDA events on the simulation's stream while the
    clocks are sampled.  The Morton reorders inside the window are counted
    and the reorder's own time is measured, so that the returned `ms` charges
    every step its share (one reorder per reorder_every steps) whatever the
    window's length.  Then per-kernel times over direct launches."""
    sim.upload_agents(agents)
    sim.clear_trail()
    sim.set_params(params)
    # step 0 of the seeded run for every mode: the Morton reorder falls due
    # at once (the upload left the agents unsorted), with or without tuning
    sim.set_steps_done(0)
    if not (args.trail_tile and args.agent_shape):
        sim.autotune(5)
    tuned = sim.info()
    sim.step(args.warmup)
    # the graphs the timed steps replay are captured here, once, as a
    # long-running user's first chunks capture them
    sim.prepare_steps(args.steps)
    sim.sync()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    info0 = sim.info()
    barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        e0.record(stream)
        sim.step(args.steps)
        e1.record(stream)
        sim.sync()
        torch.cuda.synchronize()
    barrier()
    window_ms = e0.elapsed_time(e1)
    info1 = sim.info()
    reorders_in = int(info1.reorders_done - info0.reorders_done)
    reorder_ms = sim.profile_reorder(5) / 5 if args.reorder_every else 0.0
    ms = window_ms
    if args.reorder_every:
        ms = window_ms - reorders_in * reorder_ms + args.steps * reorder_ms / args.reorder_every
    kern_steps = min(args.steps, 100)
    agents_ms, trail_ms, other_ms = sim.profile_steps(kern_steps)
    return {"tuned": tuned, "clocks": clocks.summary(), "launches": int(info1.kernel_launches -
                                                                      info0.kernel_launches),
            "window_ms": window_ms, "ms": ms, "reorders_in": reorders_in, "reorder_ms": reorder_ms,
            "kern_steps": kern_steps, "t_agents": agents_ms / kern_steps, "t_trail": trail_ms / kern_steps,
            "other_ms": other_ms}


def aggregate_ranks(ms, units_per_rank, seconds=None):
    """Whole-job figures over replicas: the slowest rank's time and the sum of
    the units every rank processed (a single colony does not shard, so each
    rank runs an independent replica; no collective touches the data path).
    Works with any initialised torch.distributed backend (NCCL on GPUs, gloo
    in the CPU tests); without one it is the identity."""
    import torch
    import torch.distributed as dist
    ws = dist.get_world_size() if dist.is_available() and dist.is_initialized() else 1
    if ws > 1:
        dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
        t = torch.tensor([float(ms), float(units_per_rank)], dtype=torch.float64, device=dev)
        mx = t.clone()
        dist.all_reduce(mx, op=dist.ReduceOp.MAX)
        sm = t.clone()
        dist.all_reduce(sm, op=dist.ReduceOp.SUM)
        ms, units = float(mx[0].item()), float(sm[1].item())
    else:
        units = float(units_per_rank)
    return ms, units, units / (ms / 1e3)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def run_reference(args, cfg_name):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    W, H, n, lo, hi, dist = CONFIGS[cfg_name]
    params = make_params(W, H, lo, hi, dist)
    agents = make_agents(n, W, H, lo, hi)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    threads = oracle.num_threads()
    a = agents.copy()
    t = np.zeros((H, W), np.float32)
    # warm-up steps (bounded to ~20 s), then timed steps bounded to ~90 s of CPU work
    warm, t0 = 0, time.perf_counter()
    while warm < args.warmup and time.perf_counter() - t0 < 20.0:
        oracle.run(params, W, H, a, t, 1, threads=threads)
        warm += 1
    steps, t0 = 0, time.perf_counter()
    while steps < args.steps:
        oracle.run(params, W, H, a, t, 1, threads=threads)
        steps += 1
        if time.perf_counter() - t0 > 90.0:
            break
    dt = time.perf_counter() - t0
    value = n * steps / dt
    line = {
        "impl": "reference", "metric": metric_name(cfg_name), "value": value, "unit": "agent-steps/s",
        "n_gpus": args.gpus, "steps": steps, "warmup": warm, "ms_per_step": 1000 * dt / steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(args, 1, cfg_name),
        "cells_per_s": W * H * steps / dt,
        "cpu_baseline": {"value": value, "unit": "agent-steps/s", "cores": threads, "kind": "port",
                         "sample": f"{steps} of {args.steps} requested full steps (time-bounded at 90 s) after "
                                   f"{warm} warm-up steps; the reference's wgpu path cannot run here "
                                   "(no Rust toolchain, no graphics stack), so the CPU restatement of its shader "
                                   "(OpenMP, pinned against a mechanical C++ translation of compute.wgsl) is the "
                                   "reference implementation"},
        "e2e": {"value": value, "unit": "agent-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="plain-4096", choices=sorted(set(CONFIGS) | set(EXTRA_CONFIGS)))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--reorder-every", type=int, default=200)
    ap.add_argument("--no-l2-persist", action="store_true")
    ap.add_argument("--trail-tile", type=int, default=0,
                    help="1 + tile-table index of the trail kernel (0: autotuned)")
    ap.add_argument("--agent-shape", type=int, default=0,
                    help="1 + shape-table index of the agent kernel (0: autotuned)")
    ap.add_argument("--dispatch", default="each", choices=["each", "reference"],
                    help="agents updated per step: every agent once, or the reference's own dispatch")
    ap.add_argument("--colonies", type=int, default=64,
                    help="ensemble-64: the first K of the 64 seeded colonies (smaller captures)")
    ap.add_argument("--ensemble-engine", default="auto", choices=["auto", "lanes", "cooperative"],
                    help="ensemble-64: autotuned engine, or one fixed without tuning (profiler runs)")
    ap.add_argument("--no-compare", action="store_true",
                    help="ensemble-64: skip the sequential and plain comparison runs (profiler runs)")
    ap.add_argument("--adjoint-steps", type=int, default=2000,
                    help="adjoint-1024: steps recorded and back-propagated (2000 in the configuration)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    if args.impl == "reference":
        run_reference(args, args.config if args.config in CONFIGS and args.config != "adjoint-1024"
                      else "plain-4096")
        return
    if args.config == "ensemble-64":
        run_ensemble(args)
        return
    if args.config == "adjoint-1024":
        run_adjoint(args)
        return

    import torch
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    torch.cuda.init()
    import slime_gb300 as sg

    W, H, n, lo, hi, sdist = CONFIGS[args.config]
    params = make_params(W, H, lo, hi, sdist)
    n_visited = n
    if args.dispatch == "reference":
        params.dispatch_mode = sg.DISPATCH_REFERENCE
        n_visited = reference_dispatch_visited(n)
    agents = make_agents(n, W, H, lo, hi, seed=rank)
    sim = sg.Simulation(W, H, n, params)
    sim.set_options(reorder_every=args.reorder_every, reorder_cell_log2=2, graph_chunk=50,
                    l2_persist=0 if args.no_l2_persist else 1,
                    trail_tile=args.trail_tile, agent_shape=args.agent_shape)
    stream = torch.cuda.ExternalStream(sim.stream_ptr())

    def barrier():
        if ws > 1:
            torch.distributed.barrier()

    # headline: the shader's sensor evaluation (the reference's result); the
    # opt-in rotated form is timed after the end-to-end loops, on the same
    # workload from the same start
    head = measure_plain(sim, stream, params, agents, args, barrier, local, torch)
    tuned, clocks, launches = head["tuned"], head["clocks"], head["launches"]
    ms, _, value = aggregate_ranks(head["ms"], n * args.steps)
    ms_per_step = ms / args.steps
    cells = ws * W * H * args.steps / (ms / 1e3)
    t_agents, t_trail, kern_steps = head["t_agents"], head["t_trail"], head["kern_steps"]
    other_ms = head["other_ms"]
    peak, peak_kind = load_peaks()
    bytes_agents = 32.0 * n_visited  # agent state read + write (agents the dispatch never updates sit in
                                     # the last slots, untouched)
    bytes_trail = 8.0 * W * H        # trail read + write
    k_agents = {"name": agents_kernel_name(tuned.agent_shape), "ms": t_agents,
                "bytes": bytes_agents, "gbs": bytes_agents / (t_agents * 1e-3) / 1e9}
    k_trail = {"name": trail_kernel_name(tuned.trail_tile, int(params.blur_mode)), "ms": t_trail,
               "bytes": bytes_trail, "gbs": bytes_trail / (t_trail * 1e-3) / 1e9}
    dom = k_agents if t_agents >= t_trail else k_trail
    traffic, traffic_src = profiled_traffic(args.config, dom["name"])
    roofline = {"bound": "hbm", "kernel": dom["name"], "achieved": dom["gbs"], "peak": peak, "unit": "GB/s",
                "frac": dom["gbs"] / peak, "traffic": traffic, "traffic_unit": "bytes per launch",
                "traffic_source": traffic_src, "peak_kind": peak_kind,
                "algorithmic_bytes_per_launch": dom["bytes"], "launch_ms": dom["ms"]}
    step_bytes = bytes_agents + bytes_trail
    pct_roofline = step_bytes / (ms_per_step * 1e-3) / 1e9 / peak

    # -- end to end through the C ABI with host buffers: every step uploads the
    # parameter block and the new trail reaches pinned host memory; the copy of
    # step s overlaps step s+1 (double-buffered host trails)
    host = [torch.empty((H, W), dtype=torch.float32, pin_memory=True).numpy() for _ in range(2)]
    e2e_steps = max(3, min(args.steps, 50))
    param_bytes = ctypes.sizeof(sg.SlimeParams)
    for _ in range(2):  # both parities' one-step graphs captured before the clock starts
        sim.set_params(params)
        sim.step(1)
    sim.download_trail_async(host[0])
    sim.wait_download()
    barrier()
    t0 = time.perf_counter()
    for i in range(e2e_steps):
        sim.set_params(params)
        sim.step(1)
        sim.download_trail_async(host[i % 2])
    sim.wait_download()
    dt = time.perf_counter() - t0
    _, _, e2e_value = aggregate_ranks(dt * 1e3, n * e2e_steps)
    e2e = {"value": e2e_value, "unit": "agent-steps/s",
           "h2d_bytes_per_step": param_bytes, "d2h_bytes_per_step": 4 * W * H,
           "steps": e2e_steps, "what": f"per step: slime_set_params ({param_bytes}-byte parameter block), "
                                       "slime_step(1), slime_download_trail_async of the new trail into pinned "
                                       "host memory (copy overlapped with the next step; all copies waited for); "
                                       "Morton reorders fall where the step schedule puts them"}

    # -- the reference's own frame loop end to end (src/main.rs:1163-1235):
    # per step the parameter block, slime_step(1) and the display pass
    # (display.wgsl) at the reference's default 1600x900 window, the frame
    # read back into pinned host memory for a host-side presenter
    tw, th = 1600, 900
    lut = np.random.default_rng(0).integers(0, 256, 768).astype(np.uint8)  # a LUT's shape; values do not matter
    frames = [torch.empty((th, tw, 4), dtype=torch.uint8, pin_memory=True).numpy() for _ in range(2)]
    for _ in range(2):
        sim.set_params(params)
        sim.step(1)
    sim.colorize_async(lut, frames[0])
    sim.wait_download()
    barrier()
    t0 = time.perf_counter()
    for i in range(e2e_steps):
        sim.set_params(params)
        sim.step(1)
        sim.colorize_async(lut, frames[i % 2])
    sim.wait_download()
    dt = time.perf_counter() - t0
    _, _, e2e_display_value = aggregate_ranks(dt * 1e3, n * e2e_steps)
    e2e_display = {"value": e2e_display_value, "unit": "agent-steps/s",
                   "h2d_bytes_per_step": param_bytes, "d2h_bytes_per_step": tw * th * 4, "steps": e2e_steps,
                   "what": f"per step: slime_set_params ({param_bytes}-byte parameter block), slime_step(1), "
                           "slime_colorize_async of the display pass into a 1600x900 RGBA8 frame in pinned "
                           "host memory (copy overlapped with the next step; all copies waited for)"}

    rotated_params = params.copy()
    rotated_params.sensor_mode = sg.SENSOR_ROTATED
    rot = measure_plain(sim, stream, rotated_params, agents, args, barrier, local, torch)
    rot_ms, _, rot_value = aggregate_ranks(rot["ms"], n * args.steps)

    def mode_summary(m, total_ms, val):
        return {"value": val, "ms_per_step": total_ms / args.steps,
                "window_ms_per_step": m["window_ms"] / args.steps, "agents_ms": m["t_agents"],
                "trail_ms": m["t_trail"], "agent_shape": m["tuned"].agent_shape,
                "trail_tile": m["tuned"].trail_tile, "clocks": m["clocks"]}

    if rank == 0:
        cpu = None
        if not args.no_cpu_baseline:
            cpu = cpu_baseline(params, W, H, n, agents)
        line = {
            "metric": metric_name(args.config),
            "value": value, "unit": "agent-steps/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (seeded)",
            "config": workload_config(args, ws),
            "cells_per_s": cells, "pct_roofline_step": pct_roofline,
            "sensor_modes": {"shader": mode_summary(head, ms, value),
                             "rotated": mode_summary(rot, rot_ms, rot_value)},
            "tuned": {"trail_tile": tuned.trail_tile, "agent_shape": tuned.agent_shape,
                      "trail_texture": tuned.trail_texture, "l2_persist_bytes": tuned.l2_persist_bytes,
                      "l2_window_passes": {0: "none", 1: "agents", 2: "trail", 3: "both"}[tuned.l2_window_passes]},
            "kernels": {"agents": k_agents, "trail": k_trail, "other_ms_per_step": other_ms / kern_steps,
                        "reorder": {"ms": head["reorder_ms"], "every": args.reorder_every,
                                    "ms_per_step": head["reorder_ms"] / args.reorder_every if args.reorder_every
                                    else 0.0, "in_timed_window": head["reorders_in"],
                                    "what": "ms_per_step = timed window - reorders inside it + K x (one "
                                            "reorder's time / reorder_every): every step pays its share"}},
            "roofline": roofline, "e2e": e2e, "e2e_display": e2e_display, "gpu_launches": launches,
            "clocks": clocks,
            "cpu_baseline": cpu,
        }
        print(json.dumps(line), flush=True)
    sim.close()
    if ws > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
