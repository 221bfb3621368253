#!/usr/bin/env python3
"""Barnes-Hut step throughput of the GB300 library.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (one "step" = bbox -> build -> summarize -> sort -> force+Euler on
the whole system): N = 4,194,304 bodies, positions normal with
sigma = (1, 1, 0.2), lognormal(0, 0.5) masses normalised to 1, zero
velocities, G = 1, theta = 0.5, eps = 0.005, dt = 1e-3, compensated force
accumulation, seeded synthetic data.  Metric: body-updates/s.

`value` is device time (CUDA events on the library's stream) with the bodies
resident in HBM; `e2e` goes through the public C ABI every step:
nb_set_state from pinned host arrays, nb_step, nb_get_state into pinned host
arrays (page-locked: the library's kernels read and write them across the host
link in place, with no staging copy); `e2e.host_link` measures the link's
width for the same bytes and the transfer floor it sets.  The accuracy gate (RMS relative force error vs an FP64 direct sum
on 8192 sample bodies <= 1e-3) is evaluated after the timed region.

The same line carries more measurements, each with its own timed region
(the last three also available alone through --mode):
  bh_configs  the plain Barnes-Hut configuration (N = 262,144 unit ball,
           monopole, FP32) and the 4M workload at theta 0.3 and 0.8, with
           their FP64-probe accuracy;
  direct   the TMA-tiled direct sum on N = 262,144 (interactions/s against
           the FP32-pipe roofline) and the naive kernel on N = 4096;
  collision  the collision update on the 262,144-body unit ball (pairs/s);
  batched  512 systems, N log-uniform in [1024, 262144], one CUDA graph per
           step, against a loop of plain solves (one handle per system);
  serving  a seeded Poisson job stream (200 jobs/s; N log-uniform in
           [1024, 2^20], 10-500 steps) through the job server, p50/p99 job
           latency and served body-updates/s, against plain solves one job
           at a time.

Under torchrun (--gpus N > 1) every rank advances its own independent
system on its own GPU (replicas; no exchange); rank 0 prints the aggregate.
--impl reference times the CPU restatement of the reference's kernels
(oracle/, OpenMP on every host thread): whole steps of all N bodies of the
same workload, without loading the GPU library.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = dict(name="bh_plummer_n4m_theta0.5", n=4194304, sigma=(1.0, 1.0, 0.2), mass_sigma=0.5, theta=0.5,
                eps=0.005, dt=1e-3, G=1.0, precision="compensated", multipole="quadrupole")
PROBE_SAMPLES = 8192
FP32_LANES_PER_SM = 128
MUFU_LANES_PER_SM = 16  # rsqrt results per SM per clock
# FP32-pipe operations of the force walk's arithmetic, counted in its source:
# a body (or monopole cell) interaction is d = x_j - x_i (3 FADD), d^2 + eps^2
# (3 FFMA), F = m r^3 (3 FMUL), a += d F (3 FFMA) = 12, plus one MUFU rsqrt;
# a quadrupole cell interaction is d (3), d^2 (3), r^2 (1), Q.d (9), d.Q.d (3),
# r^5 (2), t = 2.5 (d.Q.d) r^2 + m d^2 (3), a += (d t - Q d) r^5 (6) = 30, plus
# one MUFU rsqrt.  Votes, loads and the compensated TwoSum are overhead.
OPS_PER_BODY_INTERACTION = 12
OPS_PER_QUADRUPOLE_CELL = 30
# DRAM bytes (read + write) of one force launch per body, measured by ncu on
# the same workload at N = 1,048,576 (390.4 MB read + 75.0 MB written); the
# tree, and the cells each body opens, grow in proportion to N at fixed
# theta and distribution, so the per-body figure scales to 4M
FORCE_DRAM_BYTES_PER_BODY = (390.426624e6 + 75.037696e6) / 1048576


# ---------------------------------------------------------------------------
# distributed plumbing (host-side only: barriers and a max over ranks)
# ---------------------------------------------------------------------------
class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local_rank = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group("gloo")
            self.dist = dist

    def barrier(self):
        if self.world > 1:
            self.dist.barrier()

    def max(self, x: float) -> float:
        if self.world == 1:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def sum(self, x: float) -> float:
        if self.world == 1:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.world > 1:
            self.dist.destroy_process_group()


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for name, val in zip(names, f[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def device_sm_count(dev: int) -> int:
    """Multiprocessor count from the CUDA driver API."""
    drv = ctypes.CDLL("libcuda.so.1")
    drv.cuInit(0)
    h = ctypes.c_int(0)
    drv.cuDeviceGet(ctypes.byref(h), dev)
    v = ctypes.c_int(0)
    drv.cuDeviceGetAttribute(ctypes.byref(v), 16, h)  # CU_DEVICE_ATTRIBUTE_MULTIPROCESSOR_COUNT
    return v.value


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return d, "measured"
    except (OSError, ValueError):
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "sm_max_mhz": 2070.0}, "fallback"


def workload_ic(nb, n, seed):
    cfg = nb.default_config(num_of_bodies=n, pos_config=nb.NORMAL_SIGMA_POS, pos_sigma=WORKLOAD["sigma"],
                            mass_config=nb.MASS_LOGNORMAL, mass_lognormal_sigma=WORKLOAD["mass_sigma"],
                            vel_config=nb.FUNC_ZERO_VEL, seed=seed)
    pos, _, mass = nb.generate_ic(cfg)
    vel = np.zeros_like(pos)
    return pos, vel, mass


def workload_ic_cpu(n, seed):
    """The same bytes as workload_ic, from the oracle's restatement of the
    library's generator (the CPU arm never loads the library)."""
    from oracle import oracle as O
    O.build()
    pos, mass = O.generate_ic(n, seed, O.POS_NORMAL_SIGMA, WORKLOAD["sigma"], mass_mode=O.MASS_LOGNORMAL,
                              mass_sigma=WORKLOAD["mass_sigma"])
    return pos, np.zeros_like(pos), mass


def step_config(n, world):
    """The config of the Barnes-Hut step line; both arms print this dict."""
    return {"workload": WORKLOAD["name"] if n == WORKLOAD["n"] else f"bh_plummer_n{n}_theta0.5", "n_bodies": n,
            "theta": WORKLOAD["theta"], "eps": WORKLOAD["eps"], "dt": WORKLOAD["dt"], "G": WORKLOAD["G"],
            "integrator": "euler", "precision": WORKLOAD["precision"], "multipole": WORKLOAD["multipole"],
            "tree": "geometric octree, standard opening criterion, 32-lane warp vote",
            "l2": "inputs larger than L2 (bodies + tree about 2.3 GB per system)",
            "parallelism": f"replicas x{world}"}


def make_sim(nb, n, precision, device):
    return nb.Simulation(num_of_bodies=n, algo_config=nb.BARNES_HUT, theta=WORKLOAD["theta"],
                         epsilon=WORKLOAD["eps"], gravitational_constant=WORKLOAD["G"], numerical_method=nb.EULER,
                         precision=precision, device=device, multipole=nb.MULTIPOLE_QUADRUPOLE)


# ---------------------------------------------------------------------------
# CPU baseline: the oracle's restatement of the reference kernels, whole
# steps on every host core (oracle/nbpipeline.c)
# ---------------------------------------------------------------------------
def cpu_steps(pos, vel, mass, steps, warmup):
    """`warmup` untimed then `steps` timed whole steps of the workload on the
    CPU: bbox, build, summarise (+ quadrupoles), sort, the force walk of every
    body (compensated, vote width 32) and the Euler update, each stage on all
    host threads (OpenMP).  Advances pos/vel in place."""
    from oracle import oracle as O
    O.build()
    n = len(mass)
    acc = np.zeros_like(pos)
    pipe = O.Pipeline(n)
    args = (WORKLOAD["theta"], WORKLOAD["eps"], WORKLOAD["G"], WORKLOAD["dt"])
    for _ in range(warmup):
        pipe.step(pos, vel, acc, mass, *args, quadrupole=True, compensated=True)
    stage = dict.fromkeys(O.PIPE_STAGES, 0.0)
    inter = 0
    t0 = time.perf_counter()
    for _ in range(steps):
        for k, v in pipe.step(pos, vel, acc, mass, *args, quadrupole=True, compensated=True).items():
            stage[k] += v
        inter += int(pipe.stats.sum())
    seconds = time.perf_counter() - t0
    pipe.close()
    cores = int(O.lib().orc_max_threads())
    return {"value": n * steps / seconds, "unit": "body-updates/s", "cores": cores, "kind": "port",
            "sample": (f"{steps} whole step(s) of all N={n} bodies after {warmup} warm-up step(s): bbox, build, "
                       f"summarise + quadrupoles, sort, force walk of every body and Euler update, every stage "
                       f"on {cores} OpenMP threads (oracle/nbpipeline.c; the region counts and the few top "
                       f"cells of the build are sequential)"),
            "seconds_per_step": seconds / steps,
            "stages_s_per_step": {k: round(v / steps, 4) for k, v in stage.items()},
            "interactions_per_body": inter / steps / n}


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------
def stage_roofline(stage_ms, n, cells, hbm_gbs, quad=True):
    """Algorithmic bytes of every Barnes-Hut stage (each datum moved once)
    over its CUDA-event time, against the measured HBM copy rate.  N bodies,
    C = cells the tree allocated; layout as in the library (float4 bodies,
    8-int child rows, packed child lines)."""
    model = {
        # body {x,y,z,m} read
        "bbox": 16 * n,
        # body read; per cell: child row 32 B, parent/arrive/start 12 B written
        "build": 16 * n + 44 * cells,
        # per cell: child row read; every body and cell {x,y,z,m} read once;
        # compacted row 32, packed line 128, centre/mass 16, count 4 written,
        # with quadrupoles cell moments 32 and packed moments 192 more
        "summarize": 32 * cells + 16 * (n + cells) + (180 + (224 if quad else 0)) * cells,
        # per cell: compacted row 32 + child counts 4 read, start 4 written;
        # sorted index 4 per body written
        "sort": 40 * cells + 4 * n,
        "force": 84 * n + (352 if quad else 160) * cells,
    }
    out = {}
    for k, b in model.items():
        ms = stage_ms.get(k) or 0.0
        gbs = b / (ms / 1e3) / 1e9 if ms > 0 else None
        out[k] = {"ms": ms, "algorithmic_bytes": b, "achieved_gbs": gbs,
                  "frac_of_hbm": (gbs / hbm_gbs) if gbs else None}
    return out


def host_link(dev, h2d_bytes, d2h_bytes, reps=5):
    """Width of the host link for one step's transfers: copy-engine copies
    between page-locked host buffers and device buffers of the e2e step's
    sizes, timed with CUDA events on the copying stream after 3 warm-up
    copies.  Kernels that read or write page-locked host arrays in place
    (nb_set_state / nb_get_state) run at the same width on this link, so
    bytes / width is the floor of the transfer part of an e2e step."""
    import torch
    out = {}
    with torch.cuda.device(dev):
        for name, nbytes, to_dev in (("h2d", h2d_bytes, True), ("d2h", d2h_bytes, False)):
            h = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
            d = torch.empty(nbytes, dtype=torch.uint8, device=f"cuda:{dev}")
            src, dst = (h, d) if to_dev else (d, h)
            for _ in range(3):
                dst.copy_(src, non_blocking=True)
            torch.cuda.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            for _ in range(reps):
                dst.copy_(src, non_blocking=True)
            b.record()
            b.synchronize()
            out[f"{name}_gbs"] = nbytes * reps / (a.elapsed_time(b) * 1e6)
            del h, d
    out["transfer_floor_ms_per_step"] = (h2d_bytes / out["h2d_gbs"] + d2h_bytes / out["d2h_gbs"]) / 1e6
    return out


def run_ours(args, dist: Dist):
    from nbodysimulation_gb300 import build as nbbuild
    if dist.local_rank == 0:
        nbbuild.build()
    dist.barrier()
    import nbodysimulation_gb300 as nb
    L = nb.load()
    n, dt = args.n, WORKLOAD["dt"]
    dev = dist.local_rank
    pos, vel, mass = workload_ic(nb, n, seed=dist.rank)
    sim = make_sim(nb, n, nb.PRECISION_COMPENSATED, dev)
    sim.set_state(pos, mass, vel)
    sim.set_profiling(True)
    sim.step(dt, args.warmup)

    # --- value: bodies resident in HBM, CUDA events on the library stream ---
    clocks = ClockSampler(dev)
    launches0 = sim.kernel_launches()
    dist.barrier()
    clocks.start()
    time.sleep(0.3)
    ms = sim.time_steps(dt, args.steps)
    clk = clocks.stop()
    dist.barrier()
    launches = sim.kernel_launches() - launches0
    stage = sim.timings()
    inter, opened, cell_inter = sim.work_counters()
    info = sim.stage_debug(nb.DEBUG_TREE_INFO)
    cells_used = int(info[0] + info[1] - info[2] + 1)
    ms_max = dist.max(ms)
    total_bodies = dist.sum(float(n))
    value = total_bodies * args.steps / (ms_max / 1e3)

    # --- e2e through the C ABI with pinned host buffers ---
    hp = [L.nb_host_alloc(12 * n), L.nb_host_alloc(12 * n), L.nb_host_alloc(4 * n), L.nb_host_alloc(12 * n),
          L.nb_host_alloc(12 * n)]
    if not all(hp):
        raise RuntimeError("nb_host_alloc failed")
    ctypes.memmove(hp[0], pos.ctypes.data, 12 * n)
    ctypes.memmove(hp[1], vel.ctypes.data, 12 * n)
    ctypes.memmove(hp[2], mass.ctypes.data, 4 * n)
    sim.set_profiling(False)
    dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        st = L.nb_set_state(sim.h, hp[0], hp[1], hp[2], n)
        st = st or L.nb_step(sim.h, dt, 1)
        st = st or L.nb_get_state(sim.h, hp[3], hp[4], None, None)
        if st:
            raise RuntimeError(f"e2e step failed: {L.nb_last_error_message(sim.h).decode()}")
    e2e_s = time.perf_counter() - t0
    dist.barrier()
    e2e_s = dist.max(e2e_s)
    for p in hp:
        L.nb_host_free(p)
    e2e_value = total_bodies * args.steps / e2e_s
    link = host_link(dev, 28 * n, 24 * n + 64)
    link["e2e_ms_per_step"] = e2e_s * 1e3 / args.steps
    link["device_ms_per_step"] = ms_max / args.steps

    # --- accuracy gate (after the timed regions) ---
    rng = np.random.default_rng(1234)
    sample = rng.choice(n, PROBE_SAMPLES, replace=False).astype(np.int32)
    err_max, err_rms, _ = sim.force_error(sample)

    # --- plain FP32 accumulation, same workload, for reference ---
    fp32_value = None
    if not args.skip_fp32:
        sim.close()
        sim2 = make_sim(nb, n, nb.PRECISION_FP32, dev)
        sim2.set_state(pos, mass, vel)
        sim2.step(dt, args.warmup)
        ms2 = sim2.time_steps(dt, args.steps)
        fp32_value = total_bodies * args.steps / (dist.max(ms2) / 1e3)
        sim2.close()
    else:
        sim.close()

    if dist.rank != 0:
        return None
    peaks, peak_kind = measured_peaks()
    force_ms = stage["force"]
    # algorithmic bytes of one force launch: per body sorted index 4 B, body
    # {x,y,z,m} 16 B, velocity 16 B read; body, velocity, acceleration 48 B
    # written; per cell in the tree its child list 32 B, packed child line
    # 128 B and packed child quadrupoles 192 B read once
    alg_bytes = 84 * n + 352 * cells_used
    achieved = alg_bytes / (force_ms / 1e3) / 1e9
    sm_mhz = (clk or {}).get("sm_max_mhz") or peaks.get("sm_max_mhz", 2070.0)
    sm_count = device_sm_count(dev)
    inter_per_step = inter / args.steps
    body_inter = inter - cell_inter
    ops_per_step = (OPS_PER_BODY_INTERACTION * body_inter + OPS_PER_QUADRUPOLE_CELL * cell_inter) / args.steps
    fp32_peak_ops = FP32_LANES_PER_SM * sm_count * sm_mhz * 1e6  # one FP32 op per lane per clock
    achieved_ops = ops_per_step / (force_ms / 1e3)
    traffic = FORCE_DRAM_BYTES_PER_BODY * n
    out = {
        "metric": "BH body-updates/s N=4M theta=0.5 (RMS force err <= 1e-3)",
        "value": value,
        "unit": "body-updates/s",
        "n_gpus": dist.world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_max / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded normal sigma=(1,1,0.2) positions, lognormal masses)",
        "config": step_config(n, dist.world),
        "e2e": {"value": e2e_value, "unit": "body-updates/s", "h2d_bytes_per_step": 28 * n,
                "d2h_bytes_per_step": 24 * n + 64, "host_link": link},
        "gpu_launches": int(launches),
        "stages_ms": {k: round(v, 4) for k, v in stage.items() if v > 0},
        "accuracy": {"rms_rel_err": err_rms, "max_rel_err": err_max, "samples": PROBE_SAMPLES,
                     "oracle": "FP64 direct sum on the GPU", "gate_rms_le_1e-3": bool(err_rms <= 1e-3)},
        "fp32_accumulation_value": fp32_value,
        "roofline": {"bound": "fp32", "kernel": "k_force", "achieved": achieved_ops / 1e12,
                     "peak": fp32_peak_ops / 1e12, "unit": "T FP32-pipe ops/s",
                     "frac": achieved_ops / fp32_peak_ops, "traffic": traffic, "algorithmic_bytes": alg_bytes,
                     "traffic_over_algorithmic": traffic / alg_bytes,
                     "ops_per_step": ops_per_step,
                     "ops_model": (f"{OPS_PER_BODY_INTERACTION} FP32-pipe ops per body interaction, "
                                   f"{OPS_PER_QUADRUPOLE_CELL} per quadrupole cell interaction"),
                     "peak_kind": (f"derived: {FP32_LANES_PER_SM} FP32 lanes x {sm_count} SMs x "
                                   f"{sm_mhz:.0f} MHz (no FP32 figure is measured; the walk is bound by "
                                   f"instruction issue on the FP32 pipe, not by memory)"),
                     "hbm": {"achieved_gbs": achieved, "peak_gbs": peaks["hbm_gbs"],
                             "frac": achieved / peaks["hbm_gbs"], "peak_kind": f"{peak_kind} hbm copy"}},
        "compute": {"kernel": "k_force", "interactions_per_step": inter_per_step,
                    "body_interactions_per_step": body_inter / args.steps,
                    "cell_interactions_per_step": cell_inter / args.steps,
                    "interactions_per_s": inter_per_step / (force_ms / 1e3),
                    "cells_opened_per_step": opened / args.steps},
        "tree": {"cells_used": cells_used, "max_depth": int(info[3])},
        "stages_roofline": stage_roofline(stage, n, cells_used, peaks["hbm_gbs"]),
        "clocks": clk,
    }
    if not args.skip_cpu:
        cpos, cvel, cmass = workload_ic_cpu(n, seed=0)
        out["cpu_baseline"] = cpu_steps(cpos, cvel, cmass, steps=1, warmup=1)
    return out


def run_reference(args, dist: Dist):
    """The reference's step on the CPU: the oracle's restatement of its
    kernels (oracle/, OpenMP on every host thread), whole steps of all N
    bodies, the same workload and config as our arm.  The GPU library is not
    loaded.  Rank 0 alone runs it."""
    if dist.rank != 0:
        return None
    n = args.n
    pos, vel, mass = workload_ic_cpu(n, seed=0)
    t0 = time.perf_counter()
    cb = cpu_steps(pos, vel, mass, steps=args.steps, warmup=args.warmup)
    wall = time.perf_counter() - t0
    value = cb["value"]
    cb["wall_s_with_warmup"] = wall
    return {
        "impl": "reference",
        "metric": "BH body-updates/s N=4M theta=0.5 (RMS force err <= 1e-3)",
        "value": value,
        "unit": "body-updates/s",
        "n_gpus": dist.world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": cb["seconds_per_step"] * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded normal sigma=(1,1,0.2) positions, lognormal masses)",
        "config": step_config(n, dist.world),
        "cpu_baseline": cb,
        "e2e": {"value": value, "unit": "body-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


# ---------------------------------------------------------------------------
# other Barnes-Hut configurations: the plain N = 262,144 unit ball (monopole,
# FP32: the reference's physics) and the 4M workload at theta 0.3 and 0.8
# ---------------------------------------------------------------------------
BALL = dict(n=262144, theta=0.5, eps=0.01, dt=1e-3, G=1.0, steps=50)


def bh_leg(nb, dev, cfg, pos, vel, mass, dt, steps, warmup):
    """CUDA-event time of `steps` Barnes-Hut steps, stage times, work
    counters and the FP64-probe accuracy after the timed region."""
    n = cfg.num_of_bodies
    with nb.Simulation(cfg) as s:
        s.set_state(pos, mass, vel)
        s.set_profiling(True)
        s.step(dt, warmup)
        ms = s.time_steps(dt, steps)
        stage = s.timings()
        inter, opened, cell_inter = s.work_counters()
        rng = np.random.default_rng(1234)
        sample = rng.choice(n, min(n, PROBE_SAMPLES), replace=False).astype(np.int32)
        err_max, err_rms, _ = s.force_error(sample)
    return {"n_bodies": n, "theta": cfg.theta, "eps": cfg.epsilon, "steps": steps, "ms_per_step": ms / steps,
            "body_updates_per_s": n * steps / (ms / 1e3),
            "stages_ms": {k: round(stage[k], 4) for k in ("bbox", "build", "summarize", "sort", "force")},
            "interactions_per_body": inter / steps / n, "interactions_per_s": inter / (ms / 1e3),
            "accuracy": {"rms_rel_err": err_rms, "max_rel_err": err_max, "samples": int(len(sample)),
                         "oracle": "FP64 direct sum on the GPU"}}


def run_bh_configs(args, dist: Dist):
    import nbodysimulation_gb300 as nb
    dev = dist.local_rank
    out = {}
    cfg = nb.default_config(num_of_bodies=BALL["n"], algo_config=nb.BARNES_HUT, theta=BALL["theta"],
                            epsilon=BALL["eps"], gravitational_constant=BALL["G"], numerical_method=nb.EULER,
                            device=dev, pos_config=nb.BALL_POS, starting_volume_radius=1.0,
                            vel_config=nb.CIRCULAR_Z_VEL, mass_config=nb.MASS_EQUAL, seed=0)
    pos, vel, mass = nb.generate_ic(cfg)
    leg = bh_leg(nb, dev, cfg, pos, vel, mass, BALL["dt"], BALL["steps"], args.warmup)
    leg["workload"] = "bh_ball_n262144_theta0.5 (monopole, FP32, circular z velocities, masses 1/N)"
    out["ball_262k"] = leg
    pos, vel, mass = workload_ic(nb, WORKLOAD["n"], seed=dist.rank)
    sweep = {}
    for theta in (0.3, 0.8):
        c = nb.default_config(num_of_bodies=WORKLOAD["n"], algo_config=nb.BARNES_HUT, theta=theta,
                              epsilon=WORKLOAD["eps"], gravitational_constant=WORKLOAD["G"],
                              numerical_method=nb.EULER, device=dev, precision=nb.PRECISION_COMPENSATED,
                              multipole=nb.MULTIPOLE_QUADRUPOLE)
        sweep[f"theta_{theta}"] = bh_leg(nb, dev, c, pos, vel, mass, WORKLOAD["dt"], 5, args.warmup)
    out["theta_sweep_4m"] = sweep
    return out if dist.rank == 0 else None


# ---------------------------------------------------------------------------
# direct sum: tiled all-pairs on N = 262,144 and the naive kernel on N = 4096
# ---------------------------------------------------------------------------
DIRECT = dict(n=262144, n_global=4096, eps=0.01, eps_global=0.05, dt=1e-3, G=1.0, steps=50)
DIRECT_FP32_OPS = 12  # per pair: 3 FADD, 3 FFMA (d^2), 3 FMUL (r^3 m), 3 FFMA (accumulate); +1 MUFU rsqrt


def direct_leg(nb, dev, n, tiled, eps, steps, warmup, sm_count, sm_mhz):
    """Device time of `steps` direct-sum steps (Euler) and the FP32-pipe
    roofline: interactions/s x 12 over 128 FP32 lanes x SMs x clock."""
    cfg = nb.default_config(num_of_bodies=n, algo_config=nb.BRUTE_FORCE_LOCAL if tiled else nb.BRUTE_FORCE_GLOBAL,
                            epsilon=eps, direct_epsilon=eps, gravitational_constant=DIRECT["G"],
                            numerical_method=nb.EULER, device=dev,
                            pos_config=nb.BALL_POS if tiled else nb.NORMAL_SIGMA_POS, pos_sigma=(1.0, 1.0, 1.0),
                            starting_volume_radius=1.0, vel_config=nb.CIRCULAR_Z_VEL if tiled else nb.FUNC_ZERO_VEL,
                            mass_config=nb.MASS_EQUAL, seed=0)
    pos, vel, mass = nb.generate_ic(cfg)
    with nb.Simulation(cfg) as s:
        s.set_state(pos, mass, vel)
        s.step(DIRECT["dt"], warmup)
        ms = s.time_steps(DIRECT["dt"], steps)
        rng = np.random.default_rng(99)
        sample = rng.choice(n, min(n, PROBE_SAMPLES), replace=False).astype(np.int32)
        err_max, err_rms, _ = s.force_error(sample)
    inter = float(n) * n * steps
    ips = inter / (ms / 1e3)
    peak_ips = FP32_LANES_PER_SM * sm_count * sm_mhz * 1e6 / DIRECT_FP32_OPS
    return {"kernel": "k_direct_tiled" if tiled else "k_direct_global", "n_bodies": n, "eps": eps,
            "steps": steps, "ms_per_step": ms / steps, "body_updates_per_s": n * steps / (ms / 1e3),
            "interactions_per_s": ips, "fp32_gops": ips * DIRECT_FP32_OPS / 1e9,
            "roofline": {"bound": "fp32", "achieved": ips * DIRECT_FP32_OPS / 1e12,
                         "peak": FP32_LANES_PER_SM * sm_count * sm_mhz * 1e6 / 1e12, "unit": "TFLOP/s (FP32 ops)",
                         "frac": ips / peak_ips,
                         "peak_kind": "derived: 128 FP32 lanes x SMs x maximum SM clock"},
            "gflops_20_per_pair": ips * 20 / 1e9,
            "mufu_frac": ips / (MUFU_LANES_PER_SM * sm_count * sm_mhz * 1e6),
            "accuracy": {"rms_rel_err": err_rms, "max_rel_err": err_max, "samples": int(len(sample)),
                         "oracle": "FP64 direct sum on the GPU"}}


def run_direct(args, dist: Dist):
    from nbodysimulation_gb300 import build as nbbuild
    if dist.local_rank == 0:
        nbbuild.build()
    dist.barrier()
    import nbodysimulation_gb300 as nb
    dev = dist.local_rank
    sm_count = device_sm_count(dev)
    peaks, _ = measured_peaks()
    steps = max(args.steps, DIRECT["steps"])
    max_mhz = peaks.get("sm_max_mhz", 2070.0)
    clocks = ClockSampler(dev)
    clocks.start()
    time.sleep(0.3)
    tiled = direct_leg(nb, dev, DIRECT["n"], True, DIRECT["eps"], steps, args.warmup, sm_count, max_mhz)
    clk = clocks.stop()
    glob = direct_leg(nb, dev, DIRECT["n_global"], False, DIRECT["eps_global"], 20, args.warmup, sm_count, max_mhz)
    ms = dist.max(tiled["ms_per_step"] * steps)
    if dist.rank != 0:
        return None
    return {
        "metric": "direct-sum interactions/s, tiled N=262144 (FP32 roofline fraction)",
        "value": dist.world * float(DIRECT["n"]) ** 2 * steps / (ms / 1e3),
        "unit": "interactions/s",
        "n_gpus": dist.world, "steps": steps, "warmup": args.warmup, "ms_per_step": ms / steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded unit ball with circular z velocities, masses 1/N)",
        "config": {"workload": "direct_tiled_n262144", "n_bodies": DIRECT["n"], "eps": DIRECT["eps"],
                   "dt": DIRECT["dt"], "G": DIRECT["G"], "integrator": "euler",
                   "l2": "inputs (4 MiB) fit in L2: the sum is compute-bound, no flush needed",
                   "parallelism": f"replicas x{dist.world}"},
        "tiled": tiled, "global_n4096": glob, "clocks": clk,
    }


# ---------------------------------------------------------------------------
# collision update (update_collision_local) on the 262,144-body unit ball
# ---------------------------------------------------------------------------
COLLIDE = dict(n=262144, steps=10)


def run_collision(args, dist: Dist):
    """CUDA-event time of the collision stage inside Barnes-Hut steps of the
    plain configuration's bodies (unit ball, circular velocities, masses
    1/N, theta 0.5, eps 0.01) with collision on.  Every ordered pair is
    tested, so pairs/s = N^2 / stage time.  Roofline: the exact test of a
    pair needs at least its x separation, one FP32-pipe operation, so pairs/s
    over 128 FP32 lanes x SMs x clock is an upper bound of the fraction."""
    import nbodysimulation_gb300 as nb
    dev = dist.local_rank
    n = COLLIDE["n"]
    cfg = nb.default_config(num_of_bodies=n, algo_config=nb.BARNES_HUT, theta=BALL["theta"], epsilon=BALL["eps"],
                            gravitational_constant=BALL["G"], numerical_method=nb.EULER, device=dev,
                            pos_config=nb.BALL_POS, starting_volume_radius=1.0, vel_config=nb.CIRCULAR_Z_VEL,
                            mass_config=nb.MASS_EQUAL, seed=0, collision=1)
    pos, vel, mass = nb.generate_ic(cfg)
    with nb.Simulation(cfg) as s:
        s.set_state(pos, mass, vel)
        s.set_profiling(True)
        s.step(BALL["dt"], args.warmup)
        ms = s.time_steps(BALL["dt"], COLLIDE["steps"])
        stage = s.timings()
    if dist.rank != 0:
        return None
    peaks, _ = measured_peaks()
    sm_count = device_sm_count(dev)
    mhz = peaks.get("sm_max_mhz", 2070.0)
    coll_ms = stage["collision"]
    pairs = float(n) * n
    pps = pairs / (coll_ms / 1e3)
    peak = FP32_LANES_PER_SM * sm_count * mhz * 1e6
    return {"workload": "collision_ball_n262144 (Barnes-Hut steps with collision on; unit ball, masses 1/N)",
            "kernel": "k_collision (block form, targets in sort order)", "n_bodies": n,
            "steps": COLLIDE["steps"], "ms_per_step": ms / COLLIDE["steps"], "collision_ms": coll_ms,
            "stages_ms": {k: round(v, 4) for k, v in stage.items() if v > 0},
            "pairs_per_s": pps,
            "roofline": {"bound": "fp32", "achieved": pps / 1e12, "peak": peak / 1e12,
                         "unit": "T pairs/s at one FP32-pipe op per pair", "frac": pps / peak,
                         "peak_kind": "derived: 128 FP32 lanes x SMs x maximum SM clock"}}


# ---------------------------------------------------------------------------
# batched systems vs a loop of plain solves
# ---------------------------------------------------------------------------
BATCH = dict(name="batch512_loguniform_1k_256k", systems=512, n_min=1024, n_max=262144, direct_below=8192,
             theta=0.5, eps=0.01, dt=1e-3, G=1.0, seed=0, steps=100, plain_steps=5)


def batch_configs(nb, systems=BATCH["systems"], seed=BATCH["seed"]):
    """Seeded systems: N log-uniform in [1024, 262144]; even systems normal(0,1)
    at rest, odd systems uniform in the unit ball with circular velocities
    about z; masses 1/N; N < 8192 direct sum, the rest Barnes-Hut."""
    rng = np.random.default_rng(seed)
    ns = np.exp(rng.uniform(np.log(BATCH["n_min"]), np.log(BATCH["n_max"]), size=systems)).astype(np.int64)
    cfgs = []
    for k, n in enumerate(ns):
        ball = k % 2 == 1
        cfgs.append(nb.default_config(
            num_of_bodies=int(n), algo_config=nb.BARNES_HUT if n >= BATCH["direct_below"] else nb.BRUTE_FORCE_LOCAL,
            theta=BATCH["theta"], epsilon=BATCH["eps"], direct_epsilon=BATCH["eps"],
            gravitational_constant=BATCH["G"], numerical_method=nb.EULER,
            pos_config=nb.BALL_POS if ball else nb.NORMAL_SIGMA_POS, pos_sigma=(1.0, 1.0, 1.0),
            starting_volume_radius=1.0, vel_config=nb.CIRCULAR_Z_VEL if ball else nb.FUNC_ZERO_VEL,
            mass_config=nb.MASS_EQUAL, seed=seed * 100003 + k))
    return cfgs


def run_batch(args, dist: Dist):
    from nbodysimulation_gb300 import build as nbbuild
    if dist.local_rank == 0:
        nbbuild.build()
    dist.barrier()
    import nbodysimulation_gb300 as nb
    dev = dist.local_rank
    dt = BATCH["dt"]
    cfgs = batch_configs(nb, args.systems, BATCH["seed"] + dist.rank)
    for c in cfgs:
        c.device = dev
    states = [nb.generate_ic(c) for c in cfgs]
    ns = np.array([c.num_of_bodies for c in cfgs], np.int64)
    bodies = int(ns.sum())
    n_bh = int(sum(1 for c in cfgs if c.algo_config == nb.BARNES_HUT))

    # --- batched: one graph per step over all systems ---
    b = nb.Batch(cfgs)
    for k, (p, v, m) in enumerate(states):
        b.set_state(k, p, m, v)
    cache = os.path.join(ROOT, "nbodysimulation_gb300", "_build", "autotune.json")
    variant = b.autotune(cache)
    shape = b.tree_shape()
    b.step(dt, args.warmup)
    steps = args.batch_steps
    clocks = ClockSampler(dev)
    dist.barrier()
    clocks.start()
    time.sleep(0.3)
    ms = b.time_steps(dt, steps)
    clk = clocks.stop()
    t0 = time.perf_counter()
    b.step(dt, steps)
    wall_b = time.perf_counter() - t0
    dist.barrier()
    info = b.info()
    # end to end: the states go up from the host, `steps` steps, the
    # positions come back
    t0 = time.perf_counter()
    for k, (p, v, m) in enumerate(states):
        b.set_state(k, p, m, v)
    b.step(dt, steps)
    for k in range(len(cfgs)):
        b.get_state(k)
    e2e_b = time.perf_counter() - t0
    b.close()
    ms = dist.max(ms)
    wall_b = dist.max(wall_b)
    e2e_b = dist.max(e2e_b)
    total = dist.sum(float(bodies))
    batched = total * steps / (ms / 1e3)
    batched_wall = total * steps / wall_b

    # --- plain: one standalone handle at a time, nb_step per system ---
    pk = args.plain_steps
    wall_p = 0.0
    dev_p = 0.0
    for c, (p, v, m) in zip(cfgs, states):
        with nb.Simulation(c) as s:
            s.set_state(p, m, v)
            s.step(dt, 1)
            t0 = time.perf_counter()
            s.step(dt, pk)
            wall_p += time.perf_counter() - t0
            dev_p += s.time_steps(dt, pk)
    wall_p = dist.max(wall_p)
    dev_p = dist.max(dev_p)
    plain_wall = total * pk / wall_p
    plain_dev = total * pk / (dev_p / 1e3)
    if dist.rank != 0:
        return None
    return {
        "metric": "batched body-updates/s, 512 systems N log-uniform 1k-256k (vs a loop of plain solves)",
        "value": batched,
        "unit": "body-updates/s",
        "n_gpus": dist.world,
        "steps": steps,
        "warmup": args.warmup,
        "ms_per_step": ms / steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded: normal(0,1) at rest / unit ball with circular z velocities, masses 1/N)",
        "config": {"workload": BATCH["name"], "systems": len(cfgs), "bodies": bodies, "tree_systems": n_bh,
                   "direct_systems": len(cfgs) - n_bh, "direct_below": BATCH["direct_below"],
                   "theta": BATCH["theta"], "eps": BATCH["eps"], "dt": dt, "G": BATCH["G"], "integrator": "euler",
                   "precision": "fp32", "multipole": "monopole", "direct_variant": variant, "tree_shape": shape,
                   "launches_per_step": info["launches_per_step"],
                   "l2": "inputs larger than L2 (all systems' bodies and trees, several GB)",
                   "parallelism": f"replicas x{dist.world}"},
        "batched_wall": batched_wall,
        "plain": {"value_wall": plain_wall, "value_device": plain_dev, "steps_per_system": pk,
                  "how": "one nb_create handle per system, nb_step(dt, k) per system in turn"},
        "batched_over_plain_wall": batched_wall / plain_wall,
        "e2e": {"value": total * steps / e2e_b, "unit": "body-updates/s",
                "h2d_bytes_per_step": 28 * bodies / steps, "d2h_bytes_per_step": 48 * bodies / steps,
                "how": "all states up once, steps steps, all states down once; bytes amortised per step"},
        "gpu_launches": info["launches_per_step"] * steps,
        "clocks": clk,
    }


# ---------------------------------------------------------------------------
# serving: a Poisson job stream through the job server vs plain solves
# ---------------------------------------------------------------------------
SERVE = dict(name="serve_poisson200_n1k_1m", rate=200.0, seconds=2.0, n_min=1024, n_max=1048576, steps_min=10,
             steps_max=500, thetas=(0.5, 0.7), eps=0.01, dt=1e-3, G=1.0, direct_below=8192, budget=120e9,
             snapshot_every=10, seed=0, seconds_in_step=1.0)


def serve_jobs(nb, rate, seconds, seed):
    """Seeded job stream: Poisson arrivals; N log-uniform in [1024, 2^20];
    steps uniform in [10, 500]; normal(0,1) or unit-ball initial conditions
    50/50 (the ball with circular velocities about z); masses 1/N; theta 0.5
    or 0.7; N < 8192 direct sum, the rest Barnes-Hut."""
    rng = np.random.default_rng(seed)
    jobs, t = [], 0.0
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= seconds:
            break
        n = int(np.exp(rng.uniform(np.log(SERVE["n_min"]), np.log(SERVE["n_max"]))))
        steps = int(rng.integers(SERVE["steps_min"], SERVE["steps_max"] + 1))
        ball = bool(rng.integers(0, 2))
        theta = float(rng.choice(SERVE["thetas"]))
        cfg = nb.default_config(
            num_of_bodies=n, algo_config=nb.BARNES_HUT if n >= SERVE["direct_below"] else nb.BRUTE_FORCE_LOCAL,
            theta=theta, epsilon=SERVE["eps"], direct_epsilon=SERVE["eps"], gravitational_constant=SERVE["G"],
            numerical_method=nb.EULER, pos_config=nb.BALL_POS if ball else nb.NORMAL_SIGMA_POS,
            pos_sigma=(1.0, 1.0, 1.0), starting_volume_radius=1.0,
            vel_config=nb.CIRCULAR_Z_VEL if ball else nb.FUNC_ZERO_VEL, mass_config=nb.MASS_EQUAL,
            seed=seed * 1000003 + len(jobs))
        jobs.append((t, cfg, steps))
    return jobs


def run_serve_arm(nb, jobs, dt, dev):
    """The job server: a client thread submits each job at its arrival time
    (initial conditions generated by the server); snapshots and results come
    back through the callback."""
    counts = {"snapshots": 0, "snapshot_bytes": 0, "done": 0}
    lock = threading.Lock()

    def on_event(job, event, value, pos, vel):
        with lock:
            if event == nb.JOB_EVENT_SNAPSHOT:
                counts["snapshots"] += 1
            elif event == nb.JOB_EVENT_DONE:
                counts["done"] += 1

    srv = nb.Server(on_event=on_event, copy_arrays=False, device=dev, hbm_budget_bytes=int(SERVE["budget"]),
                    snapshot_every=SERVE["snapshot_every"])
    sizes = {}
    t0 = time.perf_counter()
    for t, cfg, steps in jobs:
        delay = t - (time.perf_counter() - t0)
        if delay > 0:
            time.sleep(delay)
        cfg.device = dev
        j = srv.submit(cfg, steps, dt)
        sizes[j] = cfg.num_of_bodies
    st_wait = srv.wait(-1, 3600.0)
    wall = time.perf_counter() - t0
    st = srv.stats()
    srv.close()
    if st_wait != 0 or st["failed"]:
        raise RuntimeError(f"serving run failed: status {st_wait}, {st['failed']} failed jobs")
    span = st["last_done_s"] - st["first_submit_s"]
    return {"value": st["body_updates"] / span, "latency_p50_s": st["latency_p50_s"],
            "latency_p99_s": st["latency_p99_s"], "latency_max_s": st["latency_max_s"],
            "latency_mean_s": st["latency_mean_s"], "jobs": st["completed"], "rounds": st["rounds"],
            "peak_jobs_on_gpu": st["peak_jobs"], "peak_bytes": st["peak_bytes"], "span_s": span,
            "snapshots": counts["snapshots"], "wall_s": wall, "body_updates": st["body_updates"]}


def run_plain_arm(nb, jobs, dt, dev):
    """One job at a time in arrival order through a standalone handle:
    initial conditions, nb_set_state, nb_step in rounds of 10 with the
    positions read back after each round (the snapshots), final state."""
    lat = []
    total = 0.0
    t0 = time.perf_counter()
    for t, cfg, steps in jobs:
        now = time.perf_counter() - t0
        if now < t:
            time.sleep(t - now)
        cfg.device = dev
        pos, vel, mass = nb.generate_ic(cfg)
        with nb.Simulation(cfg) as s:
            s.set_state(pos, mass, vel)
            done = 0
            while done < steps:
                k = min(SERVE["snapshot_every"], steps - done)
                s.step(dt, k)
                done += k
                # the served path returns the same: positions at every
                # snapshot, positions and velocities at the end
                s.positions(with_velocities=done == steps)
        lat.append(time.perf_counter() - t0 - t)
        total += cfg.num_of_bodies * steps
    span = time.perf_counter() - t0 - jobs[0][0]
    lat = np.sort(np.array(lat))
    pick = lambda p: float(lat[min(len(lat) - 1, max(0, int(np.ceil(p / 100 * len(lat))) - 1))])
    return {"value": total / span, "latency_p50_s": pick(50), "latency_p99_s": pick(99),
            "latency_max_s": float(lat[-1]), "jobs": len(jobs), "span_s": span, "body_updates": total}


def run_serve(args, dist: Dist):
    from nbodysimulation_gb300 import build as nbbuild
    if dist.local_rank == 0:
        nbbuild.build()
    dist.barrier()
    import nbodysimulation_gb300 as nb
    dev = dist.local_rank
    jobs = serve_jobs(nb, args.serve_rate, args.serve_seconds, SERVE["seed"] + dist.rank)
    clocks = ClockSampler(dev)
    dist.barrier()
    clocks.start()
    served = run_serve_arm(nb, jobs, SERVE["dt"], dev)
    clk = clocks.stop()
    plain = run_plain_arm(nb, jobs, SERVE["dt"], dev) if not args.skip_plain else None
    dist.barrier()
    total = dist.sum(served["body_updates"])
    span = dist.max(served["span_s"])
    if dist.rank != 0:
        return None
    offered = sum(c.num_of_bodies * s for _, c, s in jobs) / args.serve_seconds
    out = {
        "metric": "served body-updates/s and job latency p50/p99, Poisson job stream",
        "value": total / span,
        "unit": "body-updates/s",
        "n_gpus": dist.world,
        "steps": None,
        "warmup": 0,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded job stream; initial conditions generated by the server)",
        "config": {"workload": f"serve_poisson{args.serve_rate:g}_{args.serve_seconds:g}s_n1k_1m",
                   "stream": (f"the first {args.serve_seconds:g} s of the configuration's 60 s of arrivals (60 s offer "
                              f"about 5e11 body-updates: over 10 minutes of GPU time per arm at these rates)"),
                   "rate_jobs_per_s": args.serve_rate,
                   "stream_seconds": args.serve_seconds, "jobs": len(jobs),
                   "n_range": [SERVE["n_min"], SERVE["n_max"]], "steps_range": [SERVE["steps_min"], SERVE["steps_max"]],
                   "thetas": list(SERVE["thetas"]), "eps": SERVE["eps"], "dt": SERVE["dt"],
                   "direct_below": SERVE["direct_below"], "hbm_budget_bytes": SERVE["budget"],
                   "snapshot_every": SERVE["snapshot_every"], "offered_body_updates_per_s": offered,
                   "parallelism": f"replicas x{dist.world}"},
        "served": served,
        "plain": plain,
        "served_over_plain": (served["value"] / plain["value"]) if plain else None,
        "clocks": clk,
    }
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--n", type=int, default=WORKLOAD["n"],
                    help="bodies per system (default the 4M workload; smaller sizes for profiling)")
    ap.add_argument("--skip-cpu", action="store_true", help="omit the CPU baseline leg")
    ap.add_argument("--skip-fp32", action="store_true", help="omit the plain-FP32 accumulation run")
    ap.add_argument("--mode", choices=("step", "batch", "serve", "direct"), default="step",
                    help="step: the 4M Barnes-Hut system; batch: 512 batched systems vs plain solves; "
                         "serve: a Poisson job stream through the job server vs plain solves")
    ap.add_argument("--serve-rate", type=float, default=SERVE["rate"])
    ap.add_argument("--serve-seconds", type=float, default=None,
                    help=f"length of the job stream (default {SERVE['seconds']} s in serve mode, "
                         f"{SERVE['seconds_in_step']} s beside the step bench)")
    ap.add_argument("--skip-extras", action="store_true",
                    help="step mode: omit the direct-sum, batched and serving measurements")
    ap.add_argument("--skip-plain", action="store_true", help="serve mode: omit the plain-solve arm")
    ap.add_argument("--systems", type=int, default=BATCH["systems"])
    ap.add_argument("--batch-steps", type=int, default=BATCH["steps"])
    ap.add_argument("--plain-steps", type=int, default=BATCH["plain_steps"])
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    dist = Dist()
    try:
        if args.impl == "reference":
            out = run_reference(args, dist)
        elif args.mode == "batch":
            out = run_batch(args, dist)
        elif args.mode == "serve":
            if args.serve_seconds is None:
                args.serve_seconds = SERVE["seconds"]
            out = run_serve(args, dist)
        elif args.mode == "direct":
            out = run_direct(args, dist)
        else:
            out = run_ours(args, dist)
            if not args.skip_extras:
                # the other measurements of the workload family, each its own
                # timed region (see their modes): direct sum, batched systems
                # against plain solves, the job server against plain solves
                extra = {"bh_configs": run_bh_configs(args, dist), "direct": run_direct(args, dist),
                         "collision": run_collision(args, dist), "batched": run_batch(args, dist)}
                if args.serve_seconds is None:
                    args.serve_seconds = SERVE["seconds_in_step"]
                extra["serving"] = run_serve(args, dist)
                if out is not None:
                    out.update(extra)
        if dist.rank == 0 and out is not None:
            print(json.dumps(out), flush=True)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
