"""Benchmark of the fused lattice-Boltzmann step on GB300.

Workload (default): D3Q19 BGK, 256^3 lattice, tau = 0.6, periodic on all six
faces (NATIVE semantics), FP32 populations updated with plbpd's own collision
arithmetic (the FP32 body and the double-precision tail of its AVX2 kernel,
bit for bit), initialized at equilibrium from rho = 1 + 1e-3 N(0,1) and a
Taylor-Green velocity field of amplitude 0.02 plus 1e-4 N(0,1) per component
(seed 20261203).  A step is one time step of the whole lattice; the metric is
MLUPS (lattice cell updates per microsecond).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--arith reference|fp32] [--storage fp32|fp16|fp32dev]
                    [--configs c1,c2,c3,c4,c5 | --configs none]

One JSON line is printed by rank 0.  Under torchrun every rank advances its
own replica of the workload on its own GPU (the time step has no data-parallel
split that needs an exchange: replicas only), the timed region is bracketed by
barriers, and the slowest rank's time is used.

  value      MLUPS of K fused steps with the state resident in HBM (CUDA events
             on the solve's stream); the populations (2.7 GB) are larger than
             L2, so no flush is needed between steps.
  e2e        MLUPS through the C ABI with host buffers: upload n, rho, u from
             pinned memory (plbpd's layout), march K steps, read rho and u back;
             with the achieved host-to-device and device-to-host rates (after
             one untimed pass that loads the layout kernels).
  roofline   achieved = 152 B/cell (19 populations read and written, FP32) x
             cells / mean duration of one fused-kernel launch, against the
             measured HBM copy bandwidth; traffic = the kernel's DRAM bytes per
             launch from the ncu capture named in traffic_source.
  cpu_baseline  the reference itself (plbpd's march_in_time, compiled from its
             own sources with an OpenMP stand-in for TBB) on the host cores, on
             a bounded sample of the workload; the oracle port where the
             reference was not built.
  configs    (N = 1) sub-records measured in the same run for every benchmark
             configuration (plbpd_gb300/configs.py): the 10,000-step channel,
             the 256^3 workload in each arithmetic and storage with its error
             against FP64, the 384^3 FP16 duct with spheres, 512 batched
             domains, and the served stream.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

SEED = 20261203
N_SIDE = 256
Q = 19
BYTES_PER_CELL = 2 * Q * 4          # one read and one write of every FP32 population
# --storage: FP32 (the default and the headline), FP16 deviations (2 B a
# population) or FP32 deviations; name, bytes per cell update
STORAGES = {"fp32": ("STORAGE_FP32", 2 * Q * 4), "fp16": ("STORAGE_FP16_DEV", 2 * Q * 2),
            "fp32dev": ("STORAGE_FP32_DEV", 2 * Q * 4)}
TAU = 0.6
PERIODIC = {f: "periodic" for f in ("east", "west", "north", "south", "up", "down")}
WORKLOAD = "D3Q19 BGK 256^3, tau 0.6, fully periodic, Taylor-Green A=0.02 + noise, FP32"
ARITHS = {"reference": ("ARITH_REFERENCE", "plbpd's arithmetic (FP32 body, double-precision tail, bit-exact)"),
          "fp32": ("ARITH_FP32", "FP32 arithmetic for every direction")}


def nu_for_tau(tau: float) -> float:
    """A float viscosity whose float tau = 3 nu + 0.5 equals float(tau)."""
    target = np.float32(tau)
    nu = np.float32((tau - 0.5) / 3.0)
    for _ in range(64):
        t = np.float32(np.float32(3.0) * nu) + np.float32(0.5)
        if t == target:
            return float(nu)
        nu = np.nextafter(nu, np.float32(np.inf) if t < target else np.float32(-np.inf))
    return float(nu)


# ---------------------------------------------------------------------------
# clocks during a timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    QUERY = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int, period_ms: int = 20):
        self.device = device
        self.period_ms = period_ms
        self.proc = None
        self.lines: list[tuple[float, str]] = []   # (host time, csv line)

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", str(self.period_ms)],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
            t0 = time.perf_counter()   # the first sample arrives before the work starts
            while not self.lines and time.perf_counter() - t0 < 5.0 and self.proc.poll() is None:
                time.sleep(0.01)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.perf_counter(), line.strip()))

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self._t.join(timeout=2)

    def summary(self, t0: float | None = None, t1: float | None = None):
        """Samples taken between host times t0 and t1 (all when None; the
        nearest one each side too, since a sample covers the period before
        it)."""
        lines = self.lines
        if t0 is not None and t1 is not None and lines:
            inside = [i for i, (t, _) in enumerate(lines) if t0 <= t <= t1]
            lo = max((inside[0] if inside else next((i for i, (t, _) in enumerate(lines) if t > t1), len(lines)))
                     - 1, 0)
            hi = min((inside[-1] if inside else lo) + 1, len(lines) - 1)
            lines = lines[lo:hi + 1]
        rows = []
        for _, l in lines:
            parts = [p.strip() for p in l.split(",")]
            if len(parts) < 8:
                continue
            try:
                rows.append((float(parts[0]), float(parts[1]), float(parts[2]), parts[4:8]))
            except ValueError:
                continue
        if not rows:
            return None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i, v in enumerate(r[3]) if v.lower().startswith("active")})
        loaded = [r for r in rows if r[2] > 200.0] or rows
        return {"sm_mhz": float(np.median([r[0] for r in loaded])), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows), "power_w_max": max(r[2] for r in rows)}


# ---------------------------------------------------------------------------
# distributed helpers (torchrun: one process per GPU)
# ---------------------------------------------------------------------------
def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def dist_init(world: int, backend: str):
    if world <= 1:
        return None
    import torch.distributed as dist
    if not dist.is_initialized():
        dist.init_process_group(backend=backend)
    return dist


def barrier(dist, device=None):
    if dist is not None:
        if device is not None:
            dist.barrier(device_ids=[device])
        else:
            dist.barrier()


def aggregate(dist, local_ms: float, local_units: float, device=None):
    """Slowest rank's time and the units of all ranks."""
    if dist is None:
        return local_ms, local_units
    import torch
    dev = torch.device("cuda", device) if device is not None else torch.device("cpu")
    t = torch.tensor([local_ms], dtype=torch.float64, device=dev)
    u = torch.tensor([local_units], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(t.item()), float(u.item())


# ---------------------------------------------------------------------------
# CPU baseline (the reference compiled in oracle/_ref, else the oracle port)
# ---------------------------------------------------------------------------
def _cpu_sim(nz: int, threads: int):
    """The reference's own PLBPD loop where it was built on this host (it
    cannot express z-periodicity, so it runs the nearest setup it can: x/y
    periodic, resting z walls), else the oracle port on the fully periodic
    workload."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as po
    nu = nu_for_tau(TAU)
    if po.ref_available("omp"):
        sim = po.RefSim("D3Q19", N_SIDE, N_SIDE, nz, nu, 1.0, (0, 0, 0), (0, 0, 0), 1.0,
                        {"east": "periodic", "west": "periodic", "north": "periodic", "south": "periodic",
                         "up": "noslip", "down": "noslip"}, {"up": (0, 0, 0), "down": (0, 0, 0)},
                        variant="omp", threads=threads)
        path = "AVX2" if os.uname().machine == "x86_64" else "scalar (its AVX2 kernel is x86-only)"
        return sim, "reference", (f"plbpd's PLBPD::march_in_time, {path} collision path, OpenMP stand-in for TBB; "
                                  "x/y periodic, z walls (plbpd has no z-periodicity)")
    sim = po.Port("D3Q19", N_SIDE, N_SIDE, nz, nu, 1.0, (0, 0, 0), (0, 0, 0), 1.0, PERIODIC, {},
                  mode=po.MODE_NATIVE, arith=po.ARITH_AVX2, threads=threads)
    return sim, "port", "oracle restatement of the reference's operator sequence, fully periodic"


def cpu_baseline(seconds: float = 12.0, slab: int | None = None):
    threads = os.cpu_count() or 1
    nz = slab or N_SIDE
    sim, kind, setup = _cpu_sim(nz, threads)
    sim.initialize()
    sim.step(1)
    steps, t0 = 0, time.perf_counter()
    while True:
        sim.step(1)
        steps += 1
        el = time.perf_counter() - t0
        if el >= seconds or (steps >= 3 and el >= 0.5 * seconds and el / steps > seconds / 4):
            break
    cells = N_SIDE * N_SIDE * nz
    val = cells * steps / el / 1e6
    return {"value": round(val, 2), "unit": "MLUPS", "cores": threads, "kind": kind,
            "sample": f"D3Q19 {N_SIDE}x{N_SIDE}x{nz}, {steps} time steps, {setup}; {el:.1f} s"}


def run_reference_arm(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return 0
    # each step: one time step of a 256x256x16 slab (the same per-cell work,
    # sized so that K steps end within a few minutes)
    threads = os.cpu_count() or 1
    slab = 16
    sim, kind, setup = _cpu_sim(slab, threads)
    sim.initialize()
    sim.step(max(args.warmup, 0))
    t0 = time.perf_counter()
    sim.step(args.steps)
    el = time.perf_counter() - t0
    cells = N_SIDE * N_SIDE * slab
    val = cells * args.steps / el / 1e6
    sample = f"D3Q19 {N_SIDE}x{N_SIDE}x{slab} slab per step, {args.steps} steps, {setup}"
    line = {"impl": "reference", "metric": "MLUPS", "value": round(val, 2), "unit": "MLUPS", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(el * 1e3 / max(args.steps, 1), 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": {"workload": WORKLOAD, "sample": f"{N_SIDE}x{N_SIDE}x{slab}"},
            "cpu_baseline": {"value": round(val, 2), "unit": "MLUPS", "cores": threads, "kind": kind,
                             "sample": sample},
            "e2e": {"value": round(val, 2), "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# The fused-step kernel of the D3Q19 256^3 periodic workload, per arithmetic,
# storage and autotuner variant, and its DRAM bytes per launch from an ncu
# capture (dram__bytes_read.sum + dram__bytes_write.sum) of the committed
# summary named beside it.
KERNELS = {("reference", "fp32", 0): "nat_fused_k<19,fp32,nomask,reference> (one node a thread)",
           ("reference", "fp32", 1): "nat_fused_h2_k<19,fp32,nomask,reference,form 2> (two nodes a thread, scalar update)",
           ("fp32", "fp32", 0): "nat_fused_k<19,fp32,nomask,fp32> (one node a thread)",
           ("fp32", "fp32", 1): "nat_fused_h2_k<19,fp32,nomask,form 0> (two nodes a thread, paired FP32)",
           ("fp32", "fp32", 2): "nat_fused_h2_k<19,fp32,nomask,form 1> (two nodes a thread, paired FP32)",
           ("fp32", "fp32", 3): "nat_fused_h2_k<19,fp32,nomask,form 2> (two nodes a thread, scalar update)"}
TRAFFIC = {("reference", "fp32", 0): (2495973034, "profiles/nat_fused_ref_d3q19_256.md"),
           ("reference", "fp32", 1): (2491876522, "profiles/nat_fused_h2_ref_d3q19_256.md"),
           ("fp32", "fp32", 0): (2495234680, "profiles/nat_fused_d3q19_256.md"),
           ("fp32", "fp32", 1): (2494710954, "profiles/nat_fused_d3q19_256.md"),
           ("fp32", "fp32", 2): (2494610944, "profiles/nat_fused_d3q19_256.md"),
           ("fp32", "fp32", 3): (2494349141, "profiles/nat_fused_d3q19_256.md")}


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def golden_channel_digest():
    """SHA-256 of the reference's own fields after 10,000 steps of the
    128x64 channel (tests/golden, made from the reference by
    tests/golden/make_golden.py)."""
    try:
        with open(os.path.join(ROOT, "tests", "golden", "golden.json")) as f:
            return json.load(f)["channel_10000"]
    except (OSError, KeyError, ValueError):
        return None


def run_configs(which: list[str], peak: float, log) -> dict:
    from plbpd_gb300 import configs as cf
    fns = {"c1": lambda: cf.config1(golden_channel_digest()), "c2": lambda: cf.config2(peak),
           "c3": lambda: cf.config3(peak), "c4": lambda: cf.config4(), "c5": lambda: cf.config5()}
    out = {}
    for c in which:
        t0 = time.perf_counter()
        try:
            out[c] = fns[c]()
        except Exception as e:   # one configuration's failure does not lose the others
            out[c] = {"error": f"{type(e).__name__}: {e}"}
        out[c]["wall_seconds"] = round(time.perf_counter() - t0, 1)
        log(f"config {c}: {json.dumps(out[c])}")
    return out


def run_gpu_arm(args):
    world, rank, local = dist_env()
    import torch
    torch.cuda.set_device(local)
    dist = dist_init(world, "nccl")
    from plbpd_gb300 import capi

    nu = nu_for_tau(TAU)
    params = capi.make_params("D3Q19", N_SIDE, N_SIDE, N_SIDE, nu, rho0=1.0, face_type=PERIODIC,
                              semantics=capi.SEMANTICS_NATIVE, arith=getattr(capi, ARITHS[args.arith][0]),
                              storage=getattr(capi, STORAGES[args.storage][0]), device=local)
    cells = N_SIDE ** 3
    full = (N_SIDE + 2,) * 3
    pin_n = capi.PinnedBuffer(full + (Q,))
    pin_rho = capi.PinnedBuffer(full + (1,))
    pin_u = capi.PinnedBuffer(full + (3,))
    out_rho = capi.PinnedBuffer(full + (1,))
    out_u = capi.PinnedBuffer(full + (3,))
    from plbpd_gb300.workloads import taylor_green_state
    taylor_green_state(N_SIDE, pin_n.array, pin_rho.array, pin_u.array, seed=SEED)

    s = capi.Solve(params)
    stream = torch.cuda.ExternalStream(s.stream(), device=torch.device("cuda", local))

    def upload():
        s.set(capi.FIELD_N, pin_n.array)
        s.set(capi.FIELD_RHO, pin_rho.array)
        s.set(capi.FIELD_U, pin_u.array)

    upload()
    s.step(args.warmup)                       # RAW -> steady fused steps
    s.tune()                                  # kernel variant timed on this state, before the timed steps
    s.synchronize()

    clk = ClockSampler(local).__enter__()
    # ---- value: K fused steps, device resident --------------------------------
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier(dist, local)
    torch.cuda.synchronize()
    h0 = time.perf_counter()
    e0.record(stream)
    s.step_async(args.steps)
    e1.record(stream)
    s.synchronize()
    torch.cuda.synchronize()
    h1 = time.perf_counter()
    barrier(dist, local)
    local_ms = e0.elapsed_time(e1)
    ms, units = aggregate(dist, local_ms, float(cells) * args.steps, local)
    value = units / (ms * 1e-3) / 1e6

    # ---- mean duration of one fused-kernel launch -----------------------------
    launches = 20
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(launches)]
    for a, b in evs:
        a.record(stream)
        s.step_async(1)
        b.record(stream)
    s.synchronize()
    kms = float(np.mean([a.elapsed_time(b) for a, b in evs]))

    # ---- e2e through the C ABI with host buffers -------------------------------
    # one untimed pass first: the layout and read-back kernels load on their
    # first launch (lazy module loading), which took 30 ms of a 40 ms pass
    upload()
    s.step(min(args.steps, 64))
    s.get(capi.FIELD_RHO, out_rho.array)
    s.get(capi.FIELD_U, out_u.array)
    e2e_iters = max(1, args.e2e_iters)
    barrier(dist, local)
    torch.cuda.synchronize()
    t_up = t_down = 0.0
    t0 = time.perf_counter()
    for _ in range(e2e_iters):
        a0 = time.perf_counter()
        upload()
        a1 = time.perf_counter()
        s.step(args.steps)
        a2 = time.perf_counter()
        s.get(capi.FIELD_RHO, out_rho.array)
        s.get(capi.FIELD_U, out_u.array)
        a3 = time.perf_counter()
        t_up += a1 - a0
        t_down += a3 - a2
    t1 = time.perf_counter()
    barrier(dist, local)
    e2e_ms, e2e_units = aggregate(dist, (t1 - t0) * 1e3, float(cells) * args.steps * e2e_iters, local)
    e2e_val = e2e_units / (e2e_ms * 1e-3) / 1e6
    up_bytes = pin_n.nbytes + pin_rho.nbytes + pin_u.nbytes
    down_bytes = out_rho.nbytes + out_u.nbytes
    h2d = up_bytes / args.steps
    d2h = down_bytes / args.steps
    mass = s.conservation()[0]
    variant = s.variant()
    s.close()
    for b in (pin_n, pin_rho, pin_u, out_rho, out_u):
        b.free()

    if rank != 0:
        clk.__exit__(None, None, None)
        return 0
    peak, peak_kind = measured_peak()
    bytes_per_cell = STORAGES[args.storage][1]
    achieved = bytes_per_cell * cells / (kms * 1e-3) / 1e9
    key = (args.arith, args.storage, variant)
    traffic = TRAFFIC.get(key)
    wl = WORKLOAD if args.storage == "fp32" else WORKLOAD.replace(
        "FP32", {"fp16": "FP16 storage of f - w", "fp32dev": "FP32 storage of f - w"}[args.storage])
    line = {
        "metric": "MLUPS", "value": round(value, 1), "unit": "MLUPS", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": wl, "lattice": "D3Q19", "cells": cells, "tau": TAU,
                   "boundaries": "periodic x/y/z", "storage": args.storage, "semantics": "native",
                   "arithmetic": ARITHS[args.arith][1],
                   "l2": "no flush: populations 2.7 GB > 129 MB L2", "parallelism": f"replicas x{world}",
                   "e2e": f"{e2e_iters} x (upload n/rho/u, {args.steps} steps, read rho/u) after one untimed pass"},
        "e2e": {"value": round(e2e_val, 1), "unit": "MLUPS", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h),
                "h2d_gbs": round(up_bytes * e2e_iters / t_up / 1e9, 1),
                "d2h_gbs": round(down_bytes * e2e_iters / t_down / 1e9, 1),
                "transfer": ("pinned host buffers: one DMA copy through a device staging buffer, layout converted "
                             "on the device" if os.environ.get("PLB_PINNED_TRANSFER") != "direct" else
                             "pinned host buffers read and written in place by the layout kernels")},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": traffic[0] if traffic else None,
                     "traffic_source": (f"ncu capture, {traffic[1]}" if traffic else None),
                     "peak_source": peak_kind,
                     "kernel": KERNELS.get(key, f"fused step, {args.storage} storage, autotuner variant {variant}"),
                     "variant": variant, "bytes_per_cell": bytes_per_cell, "kernel_ms": round(kms, 4)},
        "gpu_launches": int(args.steps),
        "clocks": clk.summary(h0, h1),
        "mass_after": mass,
    }
    if world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline()
    which = [c for c in args.configs.split(",") if c and c != "none"]
    if world == 1 and which:
        line["configs"] = run_configs(which, peak, lambda m: print(m, file=sys.stderr, flush=True))
    clk.__exit__(None, None, None)
    line["clocks_whole_run"] = clk.summary()
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--e2e-iters", type=int, default=2)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--arith", choices=sorted(ARITHS), default="reference",
                    help="collision arithmetic of the GPU arm (default: plbpd's, bit-exact)")
    ap.add_argument("--storage", choices=sorted(STORAGES), default="fp32",
                    help="population storage of the GPU arm (default fp32, the headline)")
    ap.add_argument("--configs", default="c1,c2,c3,c4,c5",
                    help="benchmark configurations measured as sub-records at N=1 ('none' to skip)")
    args = ap.parse_args(argv)
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference_arm(args)
    return run_gpu_arm(args)


if __name__ == "__main__":
    sys.exit(main())
