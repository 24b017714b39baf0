"""Benchmark of the coupled IB-LBM step on GB300.

Workload (default): the dense red-cell suspension in a channel -- lattice 512x128x128,
periodic x, halfway bounce-back walls on y and z, body force 1e-6, 400 Evans-Fung cells of
642 vertices (20 % haematocrit) at seeded random non-overlapping positions and
orientations, Skalak + dihedral bending + global area / volume penalties, D3Q19 BGK with
Guo forcing, tau = 1.  Populations are stored as FP16 deviations f - t_i (fixed scale),
collision runs in FP32; vertex positions and the area / volume reductions stay FP64.

One step = velocity interpolation to all vertices, membrane forces, vertex motion,
spreading, fused collide-and-stream (the reference's step order).  Populations are
638 MB, larger than the 129 MB L2, so no flush is needed between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--storage f16|f32|f64]
    python bench.py --impl reference ...   (the CPU port of the reference's step)
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "MLUPS (coupled IB-LBM step) + membrane vertex-updates/s, FP16/FP32 storage vs FP64, 1 GB300"
# Algorithmic bytes per lattice update of the coupled collide-and-stream (the roofline's
# `achieved`): 19 populations read and written, the spread force read, the velocity field
# written (FP32 fields for FP32 / FP16 storage, FP64 for FP64); no phase byte at viscosity
# ratio 1.
BYTES_PER_LU = {"f64": 19 * 8 * 2 + 2 * 3 * 8, "f32": 19 * 4 * 2 + 2 * 3 * 4, "f16": 19 * 2 * 2 + 2 * 3 * 4}
# What the kernel moves per cell with the default (dense) reset of the previous force field:
# 19 populations read and written, the spread force read, that previous field read and rewritten
# with the body force (the reference's computeVelocity takes the previous force,
# setExternalVector resets it) and the velocity field written as four values per cell (FP64 /
# FP32 / FP16: FP16 storage keeps the velocity field in FP16, 8 bytes per cell).
KERNEL_BYTES_PER_LU = {st: 19 * s * 2 + 3 * 3 * fb + 4 * ub
                       for st, s, fb, ub in (("f64", 8, 8, 8), ("f32", 4, 4, 4), ("f16", 2, 4, 2))}
# Steps of the precision comparison: the run lengths of the benchmark configurations
COMPARE_STEPS = {"channel": 2000, "capsule": 2000, "rbc": 5000}
# complete runs of the end-to-end driver loop; the median is reported
E2E_RUNS = 3


def env_rank():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


class Ranks:
    """The ranks of a torchrun launch: one independent replica of the workload per GPU (the step
    has no exchange between replicas), a barrier around the timed region and the maximum of the
    ranks' times.  NCCL on the GPUs; gloo (CPU tensors) where a test runs the ranks on the host."""

    def __init__(self, backend=None):
        self.rank, self.world, self.local = env_rank()
        self.dist = None
        self.device = "cpu"
        if self.world > 1:
            import torch
            import torch.distributed as dist

            backend = backend or "nccl"
            if backend == "nccl":
                torch.cuda.set_device(self.local)
                self.device = "cuda"
            if not dist.is_initialized():
                dist.init_process_group(backend)
            self.dist = dist

    def barrier(self):
        if self.dist is not None:
            self.dist.barrier()

    def max(self, v):
        if self.dist is None:
            return v
        import torch

        t = torch.tensor([v], dtype=torch.float64, device=self.device)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())


class _Nvml:
    """Read-only NVML queries through ctypes (the SM clock, its maximum and the active clock
    event reasons); nothing is set.  None when the library is absent."""

    # nvmlClocksEventReason* bits
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown",
               0x80: "hw_power_brake_slowdown"}

    def __init__(self, index):
        import ctypes as C

        self.C = C
        self.lib = C.CDLL("libnvidia-ml.so.1")
        if self.lib.nvmlInit_v2() != 0:
            raise OSError("nvmlInit failed")
        self.h = C.c_void_p()
        uuid = _cuda_uuid(index)
        if not (uuid and self.lib.nvmlDeviceGetHandleByUUID(uuid.encode(), C.byref(self.h)) == 0):
            if self.lib.nvmlDeviceGetHandleByIndex_v2(C.c_uint(_nvml_index(index)), C.byref(self.h)) != 0:
                raise OSError("no NVML device for CUDA device %d" % index)
        reasons = getattr(self.lib, "nvmlDeviceGetCurrentClocksEventReasons", None)
        self._reasons = reasons or self.lib.nvmlDeviceGetCurrentClocksThrottleReasons
        v = C.c_uint()
        self.max_mhz = float(v.value) if self.lib.nvmlDeviceGetMaxClockInfo(self.h, 1, C.byref(v)) == 0 else None

    def sample(self):
        C = self.C
        mhz, bits = C.c_uint(), C.c_ulonglong()
        if self.lib.nvmlDeviceGetClockInfo(self.h, 1, C.byref(mhz)) != 0:  # NVML_CLOCK_SM
            return None
        if self._reasons(self.h, C.byref(bits)) != 0:
            bits.value = 0
        return float(mhz.value), int(bits.value)


def _cuda_uuid(device):
    """NVML's name ("GPU-<uuid>") of CUDA device `device`, or None."""
    try:
        import torch

        u = getattr(torch.cuda.get_device_properties(device), "uuid", None)
        return None if u is None else "GPU-" + str(u)
    except Exception:
        return None


def _nvml_index(device):
    vis = os.environ.get("CUDA_VISIBLE_DEVICES", "")
    ids = [v.strip() for v in vis.split(",") if v.strip()]
    if ids and all(v.isdigit() for v in ids) and device < len(ids):
        return int(ids[device])
    return device


class ClockSampler:
    """SM clock and clock event reasons sampled every 2 ms while running (NVML, read only),
    with one sample right at the start and one at the end; nvidia-smi every 100 ms where
    NVML cannot be loaded."""

    FIELDS = ["index", "clocks.sm", "clocks.max.sm", "power.draw", "clocks_event_reasons.active",
              "clocks_event_reasons.hw_slowdown", "clocks_event_reasons.hw_thermal_slowdown",
              "clocks_event_reasons.sw_thermal_slowdown", "clocks_event_reasons.sw_power_cap"]

    def __init__(self, device):
        self.device, self.proc, self.lines = device, None, []
        self.nvml, self.samples, self.stop = None, [], threading.Event()
        self.source = "unsampled"

    def __enter__(self):
        try:
            self.nvml = _Nvml(self.device)
            self.source = "nvml"
        except (OSError, AttributeError):
            self.nvml = None
        if self.nvml is not None:
            self._take()
            self.t = threading.Thread(target=self._poll, daemon=True)
            self.t.start()
            return self
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + ",".join(self.FIELDS),
                                          "--format=csv,noheader,nounits", "-lms", "100"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.source = "nvidia-smi"
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _take(self):
        s = self.nvml.sample()
        if s is not None:
            self.samples.append(s)

    def _poll(self):
        while not self.stop.wait(0.002):
            self._take()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.nvml is not None:
            self.stop.set()
            self.t.join(timeout=2)
            self._take()
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.t.join(timeout=2)

    def summary(self):
        sm, mx, reasons = [], [], set()
        if self.nvml is not None:
            for mhz, bits in self.samples:
                sm.append(mhz)
                reasons.update(nm for b, nm in _Nvml.REASONS.items() if bits & b)
            mx = [self.nvml.max_mhz] if self.nvml.max_mhz else sm
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if p[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0, "source": self.source}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm), "source": self.source}


def build_instance(bib, ctx, wl, storage):
    nx, ny, nz = wl["dims"]
    lat = ctx.add_domain(nx, ny, nz, storage=storage, **wl["lattice"])
    if wl.get("initial_velocity") is not None:
        lat.initialize_at_equilibrium(None, wl["initial_velocity"])
    shapes = bib.ParticleShapeLibrary(ctx)
    sid = shapes.store_mesh(wl["rest"], wl["tri"], "cell")
    fsi = bib.ImmersedBoundaryDynamics3D(lat, shapes)
    for pos in wl["positions"]:
        fsi.add_particle(sid, wl["model"], wl["params"], pos)
    return lat, fsi


def taylor_and_volume(bib, fsi, wl):
    pos, stats = fsi.download()
    nv = wl["rest"].shape[0]
    V0 = float(wl.get("V0") or stats[0, 1])
    return pos.reshape(-1, nv, 3), stats, V0


def cpu_sample(wl, steps, warmup=1):
    """The oracle (CPU port of the reference's step) on the same instance, all host threads:
    `warmup` untimed coupled steps, then `steps` timed ones."""
    from oracle import oracle as O

    nx, ny, nz = wl["dims"]
    lp = wl["lattice"]
    L = O.lattice((nx, ny, nz), lp["periodic"], lp["collision"], lp["omega"], lp["omega"],
                  wall_y=lp.get("wall_y", "none"), wall_z=lp.get("wall_z", "none"), wall_u=lp.get("wall_u"))
    S = O.System(L, "roma", -1.0)
    if wl.get("initial_velocity") is not None:
        f0 = O.init_equilibrium(L, None, wl["initial_velocity"])
        if lp.get("wall_y") == "fd_velocity":
            f0 = O.apply_fd_walls(L, f0, np.zeros((3, nz, ny, nx)))
        S.f[...] = f0
    S.set_body_force(np.asarray(lp.get("body_force", (0, 0, 0)), dtype=np.float64))
    sid = S.add_shape(wl["rest"], wl["tri"])
    for pos in wl["positions"]:
        S.add_particle(sid, wl["model"], wl["params"], pos)
    if warmup:
        S.step(warmup)
    t0 = time.perf_counter()
    S.step(steps)
    dt = time.perf_counter() - t0
    cells = nx * ny * nz
    nvt = wl["positions"].shape[0] * wl["positions"].shape[1]
    return dict(mlups=cells * steps / dt / 1e6, vups=nvt * steps / dt, seconds=dt, steps=steps, threads=O.threads())


def workload_config(wl, storage, world=1):
    """The `config` object of a bench line (the same for both arms)."""
    nx, ny, nz = wl["dims"]
    cells = nx * ny * nz
    walls = {"halfway_bb": "halfway bounce-back", "fd_velocity": "finite-difference velocity walls"}
    lp = wl["lattice"]
    wall_txt = ", ".join("%s %s" % (walls.get(lp.get(k), lp.get(k)), k[-1]) for k in ("wall_y", "wall_z")
                         if lp.get(k, "none") not in ("none", None))
    return {"workload": wl["name"], "cells": cells, "vertices": int(wl["positions"].size // 3), "storage": storage,
            "collision": "BGK + Guo forcing", "walls": wall_txt or "none", "dirac": "Roma 3-point",
            "l2": "populations %.0f MB > 129 MB L2, no flush" % (cells * 19 * 2 * {"f16": 2, "f32": 4, "f64": 8}[storage] / 1e6),
            "parallelism": "replicas" if world > 1 else "1 GPU"}


def run_reference(args, wl):
    """The reference arm: the CPU oracle (the FP64 port of the reference's coupled step) on the
    same instance, rank 0 only, `--warmup` untimed steps then `--steps` timed ones."""
    rank, world, _ = env_rank()
    if rank != 0:
        return
    t0 = time.perf_counter()
    r = cpu_sample(wl, max(1, args.steps), warmup=args.warmup)
    line = {
        "impl": "reference", "metric": METRIC, "value": r["mlups"], "unit": "MLUPS", "n_gpus": args.gpus,
        "steps": r["steps"], "warmup": args.warmup, "ms_per_step": 1e3 * r["seconds"] / r["steps"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(wl, args.storage, world),
        "vertex_updates_per_s": r["vups"],
        "cpu_baseline": {"value": r["mlups"], "unit": "MLUPS", "cores": r["threads"], "kind": "port",
                         "sample": "%d coupled FP64 steps of the full workload after %d warm-up steps"
                                   % (r["steps"], args.warmup)},
        "e2e": {"value": r["mlups"], "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "wall_s": time.perf_counter() - t0,
    }
    print(json.dumps(line), flush=True)


def run_batch(args):
    """64 independent capsule-in-shear instances (cubic edges 32..96, radius edge/6, 162 / 642
    vertices, Ca log-uniform in [0.01, 1], seed 4), FP32 storage, stepped as one batch after the
    autotuner picked its schedule; the same instances stepped one lattice at a time for
    comparison."""
    import biblbm_gb300 as bib
    from biblbm_gb300 import workloads

    wl = workloads.batched_capsules()
    K, W = args.steps, args.warmup
    storage = "f32" if args.storage == "f16" else args.storage
    ctx = bib.Context(0)
    built = [build_instance(bib, ctx, w, storage) for w in wl["instances"]]
    batch = bib.Batch(ctx, [b[0] for b in built])
    if args.ncu:  # profiling run: default schedule, plain launches
        ctx.set_graph_mode(False)
        batch.step(W)
        ctx.sync()
        ctx.close()
        return
    chosen = batch.autotune(steps=3)
    batch.step(W)
    ctx.sync()
    with ClockSampler(0) as clk:
        ms = batch.step_timed(K)
    cells, verts = wl["cells"], wl["vertices"]
    mlups = cells * K / (ms * 1e-3) / 1e6
    # one lattice at a time (each with its own two-step graphs), same number of steps
    k2 = max(2, K // 10)
    ms_solo = sum(f.step_timed(k2) for _, f in built) / k2 * K
    launches = K * 6
    line = {
        "metric": METRIC, "value": mlups, "unit": "MLUPS", "n_gpus": 1, "steps": K, "warmup": W,
        "ms_per_step": ms / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded instance sizes, meshes and capillary numbers, seed 4)",
        "config": {"workload": wl["name"], "instances": len(wl["instances"]), "cells": cells, "vertices": verts,
                   "storage": storage, "l2": "%d lattices, %.1f M cells: populations %.2f GB > L2, no flush" % (
                       len(wl["instances"]), cells / 1e6, cells * 19 * 2 * {"f64": 8, "f32": 4, "f16": 2}[storage] / 1e9),
                   "parallelism": "1 GPU"},
        "vertex_updates_per_s": verts * K / (ms * 1e-3),
        "autotuned": chosen,
        "one_lattice_at_a_time": {"mlups": cells * K / (ms_solo * 1e-3) / 1e6, "ms_per_step": ms_solo / K},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "kernel": "whole batched step (6 launches)", "achieved":
                     200 * cells / (ms / K * 1e-3) / 1e9, "peak": float(json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))).get("hbm_gbs", 6800.0)) if os.path.exists(os.path.join(ROOT, "MEASURED_PEAKS.json")) else 6800.0,
                     "unit": "GB/s", "traffic": None},
        "clocks": clk.summary(),
        "e2e": None,
        "cpu_baseline": None,
    }
    line["roofline"]["frac"] = line["roofline"]["achieved"] / line["roofline"]["peak"]
    print(json.dumps(line))


def run_tgv(args):
    """Lattice-only TRT (magic 1/4) Taylor-Green vortex in periodic cubes of 128, 256 and 384,
    u0 = 0.02: MLUPS and the relative error of the decay against exp(-2 nu k^2 t) after the
    timed steps, for the chosen storage (all three with --storage all is not offered: run
    three times)."""
    import biblbm_gb300 as bib

    K, W = args.steps, args.warmup
    ctx = bib.Context(0)
    res = {}
    peak = 6800.0
    if os.path.exists(os.path.join(ROOT, "MEASURED_PEAKS.json")):
        peak = float(json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))).get("hbm_gbs", peak))
    # lattice-only TRT: the 19 populations read and written; no force field is read (nothing is
    # spread) and no velocity field is written (the decay is measured after the timed steps)
    bytes_lu = {"f64": 2 * 19 * 8, "f32": 2 * 19 * 4, "f16": 2 * 19 * 2}[args.storage]
    for n in (128, 256, 384):
        tau, u0 = 0.8, 0.02
        lat = ctx.add_domain(n, n, n, periodic=(1, 1, 1), collision="trt", omega=1 / tau, trt_magic=0.25,
                             storage=args.storage)
        k = 2 * np.pi / n
        x = np.arange(n)
        X, Y = np.meshgrid(x, x, indexing="xy")
        u = np.zeros((3, n, n, n))
        u[0] = (u0 * np.sin(k * X) * np.cos(k * Y))[None]
        u[1] = (-u0 * np.cos(k * X) * np.sin(k * Y))[None]
        rho = np.broadcast_to((1.0 + 0.75 * u0 * u0 * (np.cos(2 * k * X) + np.cos(2 * k * Y)))[None], (n, n, n))
        lat.initialize_at_equilibrium(np.ascontiguousarray(rho), u)
        lat.collide_and_stream(W)
        ctx.sync()
        t0 = time.perf_counter()
        lat.collide_and_stream(K)
        ctx.sync()
        dt = time.perf_counter() - t0
        ux = lat.compute_velocity()[0]
        nu = (tau - 0.5) / 3
        expect = u0 * np.exp(-2 * nu * k * k * (W + K))
        res[str(n)] = {"mlups": n ** 3 * K / dt / 1e6, "achieved_gbs": bytes_lu * n ** 3 * K / dt / 1e9,
                       "decay_rel_error": float(abs(np.abs(ux).max() - expect) / expect)}
        ctx.sync()
        del lat
    best = res["384"]
    line = {
        "metric": METRIC, "value": best["mlups"], "unit": "MLUPS", "n_gpus": 1, "steps": K, "warmup": W,
        "ms_per_step": 384 ** 3 / best["mlups"] / 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": args.storage, "data": "synthetic (Taylor-Green vortex, u0 = 0.02)",
        "config": {"workload": "tgv_trt_sweep", "edges": [128, 256, 384], "storage": args.storage,
                   "l2": "populations > L2 from 128^3 on", "parallelism": "1 GPU"},
        "sweep": res,
        "roofline": {"bound": "hbm", "kernel": "collide-and-stream (lattice-only)", "achieved": best["achieved_gbs"],
                     "peak": peak, "unit": "GB/s", "frac": best["achieved_gbs"] / peak, "traffic": None},
        "gpu_launches": K, "e2e": None, "cpu_baseline": None,
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="native", choices=["native", "reference"])
    ap.add_argument("--storage", default="f16", choices=["f16", "f32", "f64"])
    ap.add_argument("--workload", default="channel", choices=["channel", "channel_small", "capsule", "rbc", "batch", "tgv"],
                    help="channel: 400 RBCs in 512x128x128 (the headline); channel_small: the same density and rows, "
                         "200 RBCs in 512x128x64 (profiling captures); capsule: one capsule in shear, 64^3; "
                         "rbc: one RBC in shear, 128x64x64; batch: 64 capsule instances stepped as one batch; "
                         "tgv: TRT Taylor-Green bandwidth sweep, 128^3 / 256^3 / 384^3")
    ap.add_argument("--cpu-steps", type=int, default=2)
    ap.add_argument("--compare-steps", type=int, default=0,
                    help="steps of the FP64 / FP32 / FP16 comparison (default: the configuration's run length)")
    ap.add_argument("--no-variants", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--ncu", action="store_true",
                    help="profiling run: build the instance, run --warmup plain (non-graph) steps, print nothing")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    from biblbm_gb300 import workloads

    if args.workload in ("batch", "tgv") and args.impl == "native":
        return run_batch(args) if args.workload == "batch" else run_tgv(args)
    wl = {"channel": workloads.channel_suspension,
          "channel_small": lambda: workloads.channel_suspension(nx=512, ny=128, nz=64, n_cells=200),
          "capsule": workloads.capsule_shear, "rbc": workloads.rbc_shear,
          "batch": lambda: workloads.batched_capsules()["instances"][0],
          "tgv": workloads.capsule_shear}[args.workload]()
    if args.impl == "reference":
        run_reference(args, wl)
        return

    ranks = Ranks()
    rank, world, local = ranks.rank, ranks.world, ranks.local
    import biblbm_gb300 as bib

    barrier, max_over_ranks = ranks.barrier, ranks.max

    nx, ny, nz = wl["dims"]
    cells = nx * ny * nz
    nvt = int(wl["positions"].shape[0] * wl["positions"].shape[1])
    K, W = args.steps, args.warmup

    if args.ncu:
        ctx = bib.Context(local)
        lat, fsi = build_instance(bib, ctx, wl, args.storage)
        ctx.set_graph_mode(False)
        fsi.step(W)
        ctx.sync()
        ctx.close()
        return

    # ---------------- timed region: K coupled steps, graph replays, device events
    ctx = bib.Context(0 if world == 1 else local)
    lat, fsi = build_instance(bib, ctx, wl, args.storage)
    fsi.step(W)
    ctx.sync()
    barrier()
    with ClockSampler(local) as clk:
        ms = fsi.step_timed(K)
    barrier()
    ms = max_over_ranks(ms)
    mlups = cells * K * world / (ms * 1e-3) / 1e6
    vups = nvt * K * world / (ms * 1e-3)
    lat.check_health()
    kernels_per_step = fsi.kernels_per_step()

    # ---------------- per-kernel device time over K more steps (events between kernels)
    ctx.set_profiling(True)
    fsi.step(K)
    prof = ctx.profile()
    ctx.set_profiling(False)
    coll_ms = prof["collide_stream"] / K
    bytes_lu = BYTES_PER_LU[args.storage]
    achieved = bytes_lu * cells / (coll_ms * 1e-3) / 1e9
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except OSError:
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    traffic = None
    try:
        tr = json.load(open(os.path.join(ROOT, "profiles", "collide_stream_traffic.json")))
        if args.storage in tr.get("bytes_per_cell", {}):
            traffic = tr["bytes_per_cell"][args.storage] * cells
    except (OSError, ValueError):
        pass

    pos_main, stats_main, V0 = taylor_and_volume(bib, fsi, wl)
    u_main = lat.compute_velocity() if args.storage != "f64" else None
    steps_main = W + 2 * K
    ctx.close()
    del lat, fsi

    # ---------------- same-GPU variants and their error against the FP64 path, over the run
    # length of the workload's configuration (independent of --steps)
    variants = {}
    if not args.no_variants:
        n_cmp = args.compare_steps or COMPARE_STEPS.get(args.workload, 2000)
        for st in ["f64", "f32", "f16"]:
            c2 = bib.Context(0 if world == 1 else local)
            l2, f2 = build_instance(bib, c2, wl, st)
            mass0 = cells + float(l2.receive().sum())  # rho = 1 + sum of f-bar
            f2.step(W)
            c2.sync()
            kk = min(max(3, K // 2) if st == "f64" else K, n_cmp - W)
            t = f2.step_timed(kk)
            f2.step(n_cmp - W - kk)
            l2.check_health()
            variants[st] = {"mlups": cells * kk / (t * 1e-3) / 1e6, "vertex_updates_per_s": nvt * kk / (t * 1e-3),
                            "ms_per_step": t / kk, "timed_steps": kk}
            pos_v, stats_v, _ = taylor_and_volume(bib, f2, wl)
            variants[st]["_u"] = l2.compute_velocity()
            variants[st]["_stats"] = stats_v
            variants[st]["_mass"] = (mass0, cells + float(l2.receive().sum()))
            I = bib.api.moments_of_inertia(pos_v, wl["tri"])
            variants[st]["_D"] = np.array([bib.taylor_deformation(Ik) for Ik in I])
            c2.close()
        ref_u, ref_stats, ref_mass = variants["f64"]["_u"], variants["f64"]["_stats"], variants["f64"]["_mass"]
        for st in ["f32", "f16"]:
            u = variants[st]["_u"]
            variants[st]["velocity_rel_l2_vs_f64"] = float(np.linalg.norm(u - ref_u) / np.linalg.norm(ref_u))
            variants[st]["volume_rel_diff_vs_f64_max"] = float(
                np.abs(variants[st]["_stats"][:, 1] - ref_stats[:, 1]).max() / V0)
            dD = np.abs(variants[st]["_D"] - variants["f64"]["_D"])
            variants[st]["taylor_D_abs_diff_vs_f64"] = {"max": float(dD.max()), "mean": float(dD.mean())}
            variants[st]["mass_rel_diff_vs_f64"] = float((variants[st]["_mass"][1] - ref_mass[1]) / ref_mass[0])
        for st in ["f64", "f32", "f16"]:
            v = variants[st]
            v["volume_drift_max"] = float(np.abs(v["_stats"][:, 1] - V0).max() / V0)
            v["taylor_D_mean"] = float(v["_D"].mean())
            v["mass_drift_rel"] = float((v["_mass"][1] - v["_mass"][0]) / v["_mass"][0])
            for key in ("_u", "_stats", "_D", "_mass"):
                v.pop(key)
        variants["steps_compared"] = n_cmp
        variants["f64"]["speedup_f16_over_f64"] = variants["f16"]["mlups"] / variants["f64"]["mlups"]
        variants["f64"]["speedup_f32_over_f64"] = variants["f32"]["mlups"] / variants["f64"]["mlups"]

    # ---------------- end to end through the C ABI with host buffers
    e2e = None
    if not args.no_e2e:
        try:
            import torch

            def pinned(shape):
                return torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()
        except Exception:  # torch without CUDA pinning: pageable buffers
            def pinned(shape):
                return np.empty(shape, dtype=np.float64)
        f_host = pinned((19, nz, ny, nx))
        pos_host = pinned(wl["positions"].shape)
        pos_host[...] = wl["positions"]
        pos_out = pinned((nvt, 3))
        stats_out = pinned((wl["positions"].shape[0], 5))
        f_out = pinned((19, nz, ny, nx))
        c3 = bib.Context(0 if world == 1 else local)
        nxx = wl["dims"]
        l3 = c3.add_domain(*nxx, storage=args.storage, **wl["lattice"])
        shapes = bib.ParticleShapeLibrary(c3)
        sid = shapes.store_mesh(wl["rest"], wl["tri"], "cell")
        f3 = bib.ImmersedBoundaryDynamics3D(l3, shapes)
        # the populations the round trip sends: the library's equilibrium of the initial velocity
        # field, read back before the timed region
        u_init = pinned((3, nz, ny, nx))
        u_init[...] = 0.0 if wl.get("initial_velocity") is None else wl["initial_velocity"]
        l3.initialize_at_equilibrium(None, u_init)
        c3.check(c3.lib.bib_lattice_receive(c3.h, l3.h, f_host.ctypes.data, f_host.nbytes, 0))
        # warm the path once (graphs, kernel modules) on a throwaway step
        l3.send(f_host)
        for p in pos_host:
            f3.add_particle(sid, wl["model"], wl["params"], p)
        f3.step(W)
        c3.sync()
        import ctypes as C

        lib, h = c3.lib, c3.h
        barrier()
        t0 = time.perf_counter()
        c3.check(lib.bib_lattice_send(h, l3.h, f_host.ctypes.data, f_host.nbytes, 0))
        c3.check(lib.bib_particles_upload(h, l3.h, pos_host.ctypes.data_as(C.POINTER(C.c_double))))
        dpd = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))  # noqa: E731
        stats_buf = [stats_out, pinned(stats_out.shape)]
        for k in range(K):
            c3.check(lib.bib_step(h, l3.h, 1))
            # the step's result: area, volume and centre of every cell (what a driver reads to
            # follow the deformation), copied behind the step; the host waits for step k-1's copy
            # while step k runs (double-buffered pinned buffers)
            c3.check(lib.bib_particles_download_async(h, l3.h, None, dpd(stats_buf[k % 2]), k % 2))
            if k:
                c3.check(lib.bib_download_wait(h, (k - 1) % 2))
        c3.check(lib.bib_download_wait(h, (K - 1) % 2))
        c3.check(lib.bib_particles_download(h, l3.h, dpd(pos_out), None))
        c3.check(lib.bib_lattice_receive(h, l3.h, f_out.ctypes.data, f_out.nbytes, 0))
        dt = time.perf_counter() - t0
        barrier()
        dt = max_over_ranks(dt)
        h2d = f_host.nbytes + pos_host.nbytes
        d2h = K * stats_out.nbytes + pos_out.nbytes + f_out.nbytes
        # the population transfers alone (after the timed region), pinned and pageable
        tx = {}
        pageable = np.zeros_like(f_out)
        for name, buf in (("pinned", f_out), ("pageable", pageable)):
            t1 = time.perf_counter()
            c3.check(lib.bib_lattice_send(h, l3.h, buf.ctypes.data, buf.nbytes, 0))
            t2 = time.perf_counter()
            c3.check(lib.bib_lattice_receive(h, l3.h, buf.ctypes.data, buf.nbytes, 0))
            t3 = time.perf_counter()
            tx["send_gbs_" + name] = buf.nbytes / (t2 - t1) / 1e9
            tx["receive_gbs_" + name] = buf.nbytes / (t3 - t2) / 1e9
        rt = {"value": cells * K * world / dt / 1e6, "unit": "MLUPS", "h2d_bytes_per_step": int(h2d // K),
               "d2h_bytes_per_step": int(d2h // K), "seconds": dt, **tx,
               "what": "bib_lattice_send of the FP64 initial populations + bib_particles_upload of the vertex positions, K x (bib_step + "
                       "bib_particles_download_async of the per-cell area/volume/centre, waited for one step "
                       "later), final download of all "
                       "vertex positions and bib_lattice_receive of the populations; pinned host buffers"}
        # The loop of the reference's own channel driver (rbcs_in_channel.cpp: initializeAtEquilibrium
        # from a velocity field, then steps; it writes velocity fields and particle data, not
        # populations): bib_lattice_init_equilibrium from the host velocity field, K x (bib_step +
        # cell statistics), final vertex positions and bib_lattice_get_velocity.
        u0 = pinned((3, nz, ny, nx))
        u0[...] = 0.0 if wl.get("initial_velocity") is None else wl["initial_velocity"]
        u_out = pinned((3, nz, ny, nx))

        def driver_loop():
            barrier()
            t0 = time.perf_counter()
            c3.check(lib.bib_lattice_init_equilibrium(h, l3.h, None, dpd(u0)))
            c3.check(lib.bib_particles_upload(h, l3.h, dpd(pos_host)))
            for k in range(K):
                c3.check(lib.bib_step(h, l3.h, 1))
                c3.check(lib.bib_particles_download_async(h, l3.h, None, dpd(stats_buf[k % 2]), k % 2))
                if k:
                    c3.check(lib.bib_download_wait(h, (k - 1) % 2))
            c3.check(lib.bib_download_wait(h, (K - 1) % 2))
            c3.check(lib.bib_particles_download(h, l3.h, dpd(pos_out), None))
            c3.check(lib.bib_lattice_get_velocity(h, l3.h, dpd(u_out)))
            return max_over_ranks(time.perf_counter() - t0)

        # three complete runs of the loop (each from the host velocity field to the host results);
        # the median is reported: one run of a few milliseconds varies with host scheduling
        runs = [driver_loop() for _ in range(E2E_RUNS)]
        dt2 = float(np.median(runs))
        barrier()
        # the headline: the reference's own driver loop; the population round trip of the
        # CoProcessor3D boundary (bound by the CPU-GPU link for few steps) beside it
        e2e = {
            "value": cells * K * world / dt2 / 1e6, "unit": "MLUPS", "seconds": dt2,
            "runs": len(runs), "seconds_each": runs,
            "h2d_bytes_per_step": int((u0.nbytes + pos_host.nbytes) // K),
            "d2h_bytes_per_step": int((K * stats_out.nbytes + pos_out.nbytes + u_out.nbytes) // K),
            "what": "the loop of the reference's channel driver (rbcs_in_channel.cpp): bib_lattice_init_equilibrium "
                    "from the FP64 host velocity field + bib_particles_upload of the vertex positions, K x (bib_step + "
                    "bib_particles_download_async of the per-cell area/volume/centre, waited for one step later), final "
                    "vertex positions and bib_lattice_get_velocity (FP64 velocity field); pinned host buffers",
            "coprocessor_round_trip": rt}
        c3.close()

    # ---------------- CPU baseline (the oracle port) on a bounded sample
    cpu = None
    if rank == 0 and not args.no_cpu:
        r = cpu_sample(wl, args.cpu_steps)
        cpu = {"value": r["mlups"], "unit": "MLUPS", "cores": r["threads"], "kind": "port",
               "sample": "%d coupled steps of the full workload (after 1 warm-up), %.1f s" % (r["steps"], r["seconds"]),
               "vertex_updates_per_s": r["vups"]}

    if rank != 0:
        return
    # FP16 / FP32 rows of 512 cells fit the staged tile; 512 FP64 cells do not (row-vectorised kernel)
    staged = nx * {"f64": 8, "f32": 4, "f16": 2}[args.storage] % 16 == 0 and nx <= (256 if args.storage == "f64" else 512)
    kernel = {st: ("k_collide_stream_staged<%s>" if staged else "k_collide_stream_rows<%s>") % t
              for st, t in (("f64", "double"), ("f32", "float"), ("f16", "__half"))}
    line = {
        "metric": METRIC,
        "value": mlups,
        "unit": "MLUPS",
        "n_gpus": world,
        "steps": K,
        "warmup": W,
        "ms_per_step": ms / K,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32" if args.storage != "f64" else "f64",
        "data": "synthetic (seeded: RBC positions/orientations seed %d)" % wl["seed"],
        "config": workload_config(wl, args.storage, world),
        "vertex_updates_per_s": vups,
        # a second pass of K plain (not graph-replayed) steps with events between the kernels
        "kernel_ms_per_step": {k: v / K for k, v in prof.items()},
        "kernel_ms_source": "separate pass of K eager steps, CUDA events between kernels (sums above the graph step)",
        # kernel nodes of the replayed step graph (the library's count) x K
        "gpu_launches": int(K * kernels_per_step),
        "kernels_per_step": kernels_per_step,
        "roofline": {"bound": "hbm", "kernel": kernel[args.storage], "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "algorithmic_bytes_per_cell": bytes_lu,
                     "kernel_bytes_per_cell": KERNEL_BYTES_PER_LU[args.storage],
                     "kernel_gbs": KERNEL_BYTES_PER_LU[args.storage] * cells / (coll_ms * 1e-3) / 1e9,
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs" if peaks else "fallback 6800 GB/s"},
        "clocks": clk.summary(),
        "variants": variants,
        "e2e": e2e,
        "cpu_baseline": cpu,
    }
    print(json.dumps(line), flush=True)
    if ranks.dist is not None:
        ranks.dist.destroy_process_group()


if __name__ == "__main__":
    main()
