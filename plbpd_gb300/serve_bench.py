"""Served stream of mixed solves: the solve server against serial plain solves.

    python -m plbpd_gb300.serve_bench --requests 200 --rate 200

Requests (seeded): Poisson arrivals at --rate per second; 60% D2Q9 with a
square grid of edge log-uniform in [64, 2048], 40% D3Q19 with a cube of edge
log-uniform in [32, 160]; FP32 (f - w by default) or FP16 storage 50/50; tau uniform in
[0.55, 1.5]; random 2x2x2 obstacles at 0-20% solid; 500-5000 steps; periodic
x, resting walls on the other moving axes, a body force.  The server admits
by device bytes under --budget-gb (and by its own running-cells cap and
smallest-work-first order).  Printed: solves/s and p50/p99 latency (arrival
to result) of the server, the median wait for admission and run time, the
median latency of the smaller half of the requests, solves/s of the same
requests run one after another as plain solves, and the relative L2 error of
u against an FP64 run for a sample of the requests.
"""
from __future__ import annotations

import argparse
import json
import threading
import time

import numpy as np

from . import capi
from .workloads import porous_mask


def make_requests(n: int, rate: float, seed: int, min_steps: int = 500, max_steps: int = 5000):
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for i in range(n):
        t += float(rng.exponential(1.0 / rate))
        fp16 = bool(rng.random() < 0.5)
        if rng.random() < 0.6:
            L = int(round(float(np.exp(rng.uniform(np.log(64), np.log(2048))))))
            model, nx, ny, nz = "D2Q9", L + (L % 2 if fp16 else 0), 1, L
            faces = {"east": "periodic", "west": "periodic", "up": "noslip", "down": "noslip"}
            vel = {"up": (0.0, 0.0, 0.0), "down": (0.0, 0.0, 0.0)}
        else:
            L = int(round(float(np.exp(rng.uniform(np.log(32), np.log(160))))))
            model, nx, ny, nz = "D3Q19", L + (L % 2 if fp16 else 0), L, L
            faces = {"east": "periodic", "west": "periodic", "north": "noslip", "south": "noslip", "up": "noslip",
                     "down": "noslip"}
            vel = {f: (0.0, 0.0, 0.0) for f in ("north", "south", "up", "down")}
        tau = float(rng.uniform(0.55, 1.5))
        nu = (tau - 0.5) / 3.0
        h = max(nz - 2, 1)
        force = 8.0 * nu * 0.02 / (h * h)
        solid = float(rng.uniform(0.0, 0.2))
        steps = int(rng.integers(min_steps, max_steps + 1))
        out.append(dict(t=t, model=model, dims=(nx, ny, nz), tau=tau, nu=nu, force=force, faces=faces, vel=vel,
                        fp16=fp16, solid=solid, mask_seed=seed + 7 + i, steps=steps))
    return out


FP32_STORAGE = {"dev": capi.STORAGE_FP32_DEV, "plain": capi.STORAGE_FP32}
_fp32 = [capi.STORAGE_FP32_DEV]


def params_of(r, storage=None):
    st = storage if storage is not None else (capi.STORAGE_FP16_DEV if r["fp16"] else _fp32[0])
    nx, ny, nz = r["dims"]
    return capi.make_params(r["model"], nx, ny, nz, r["nu"], force=(r["force"], 0.0, 0.0), face_type=r["faces"],
                            face_vel=r["vel"], semantics=capi.SEMANTICS_NATIVE, arith=capi.ARITH_FP32, storage=st)


def mask_of(r):
    nx, ny, nz = r["dims"]
    return porous_mask(nx, ny, nz, 1.0 - r["solid"], r["mask_seed"]) if r["solid"] > 0 else None


def run_plain(r, storage=None):
    with capi.Solve(params_of(r, storage)) as s:
        m = mask_of(r)
        if m is not None:
            s.set_mask(m)
        s.initialize()
        s.step(r["steps"])
        return s.get(capi.FIELD_U)


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--requests", type=int, default=200)
    ap.add_argument("--rate", type=float, default=200.0)
    ap.add_argument("--budget-gb", type=float, default=150.0)
    ap.add_argument("--tick", type=int, default=250)
    ap.add_argument("--seed", type=int, default=20261203)
    ap.add_argument("--plain", type=int, default=-1, help="requests run as serial plain solves (default: all)")
    ap.add_argument("--accuracy-sample", type=int, default=6)
    ap.add_argument("--max-steps", type=int, default=5000)
    ap.add_argument("--fp32-storage", choices=sorted(FP32_STORAGE), default="dev",
                    help="storage of the FP32 half: f - w (dev) or f (plain, plbpd's)")
    a = ap.parse_args(argv)
    _fp32[0] = FP32_STORAGE[a.fp32_storage]
    reqs = make_requests(a.requests, a.rate, a.seed, max_steps=a.max_steps)
    masks = [mask_of(r) for r in reqs]
    cell_updates = sum(np.prod(r["dims"]) * r["steps"] for r in reqs)

    # ---- served ------------------------------------------------------------------
    lat, waits, runs, results = {}, {}, {}, {}
    with capi.Server(budget_bytes=int(a.budget_gb * (1 << 30)), tick_steps=a.tick) as srv:
        ids = [None] * len(reqs)
        t0 = time.perf_counter()

        def producer():
            for i, r in enumerate(reqs):
                delay = r["t"] - (time.perf_counter() - t0)
                if delay > 0:
                    time.sleep(delay)
                ids[i] = srv.submit(params_of(r), r["steps"], masks[i])

        th = threading.Thread(target=producer)
        th.start()
        th.join()
        for i in range(len(reqs)):
            srv.wait(ids[i], 3600.0)
            rho, u, (ts, tadm, tdone) = srv.result(ids[i])
            lat[i] = tdone - ts
            waits[i] = tadm - ts
            runs[i] = tdone - tadm
            if i < a.accuracy_sample:
                results[i] = u
        t_served = time.perf_counter() - t0
        _, peak = srv.memory()
    lats = np.array([lat[i] for i in range(len(reqs))])
    work = np.array([float(np.prod(r["dims"])) * r["steps"] for r in reqs])
    small = work <= np.median(work)

    # ---- serial plain solves ---------------------------------------------------------
    nplain = len(reqs) if a.plain < 0 else min(a.plain, len(reqs))
    t0 = time.perf_counter()
    for r in reqs[:nplain]:
        run_plain(r)
    t_plain = time.perf_counter() - t0
    plain_rate = nplain / t_plain if nplain else float("nan")

    # ---- accuracy against FP64 runs of the same requests -------------------------------
    errs = {"fp32": [], "fp16": []}
    for i in range(min(a.accuracy_sample, len(reqs))):
        r = reqs[i]
        u64 = run_plain(r, capi.STORAGE_FP64)[1:-1, 1:-1, 1:-1].astype(np.float64)
        u = results[i][1:-1, 1:-1, 1:-1].astype(np.float64)
        e = float(np.linalg.norm(u - u64) / max(np.linalg.norm(u64), 1e-300))
        errs["fp16" if r["fp16"] else "fp32"].append(e)

    served_rate = len(reqs) / t_served
    print(json.dumps({
        "workload": "served stream", "requests": len(reqs), "arrival_rate": a.rate, "fp32_storage": a.fp32_storage,
        "cell_updates": float(cell_updates), "served_seconds": round(t_served, 2),
        "served_solves_per_s": round(served_rate, 3), "served_mlups": round(cell_updates / t_served / 1e6, 1),
        "latency_p50_s": round(float(np.percentile(lats, 50)), 3),
        "latency_p99_s": round(float(np.percentile(lats, 99)), 3), "peak_budget_bytes": int(peak),
        "wait_p50_s": round(float(np.median([waits[i] for i in range(len(reqs))])), 3),
        "run_p50_s": round(float(np.median([runs[i] for i in range(len(reqs))])), 3),
        "latency_p50_smaller_half_s": round(float(np.percentile(lats[small], 50)), 3),
        "plain_requests": nplain, "plain_seconds": round(t_plain, 2), "plain_solves_per_s": round(plain_rate, 3),
        "speedup": round(served_rate / plain_rate, 2) if nplain else None,
        "u_rel_l2_vs_fp64": {k: [float(f"{x:.3g}") for x in v] for k, v in errs.items()},
    }))


if __name__ == "__main__":
    main()
