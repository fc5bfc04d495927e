"""Served stream of mixed solves: the solve server against serial plain solves.

    python -m plbpd_gb300.serve_bench --requests 200 --rate 200 [--small]

Requests (seeded): Poisson arrivals at --rate per second; 60% D2Q9 with a
square grid of edge log-uniform in [64, 2048], 40% D3Q19 with a cube of edge
log-uniform in [32, 160] (--small: edges up to 256 and 48, the requests that
alone leave most of the GPU idle); FP32 storage (f - w by default) or FP16
storage 50/50; tau uniform in [0.55, 1.5]; random 2x2x2 obstacles at 0-20%
solid; 500-5000 steps; periodic x, resting walls on the other moving axes, a
body force.  The server admits by device bytes under --budget-gb (and by its
own running-cells cap and smallest-work-first order).

Printed (one JSON line): solves/s and p50/p99 latency (arrival to result) of
the server; the same requests run one after another as plain solves (one
solve, its own launches, at a time), their solves/s and the p50/p99 latency
they would see arriving on the same trace (a first-come first-served queue
with the measured service times); and the relative L2 error of u against an
FP64 run of the same request for --accuracy-sample requests (spread over the
trace), with the number meeting --tolerance per storage and the served
solves/s and latencies of the compliant requests alone.
"""
from __future__ import annotations

import argparse
import json
import threading
import time

import numpy as np

from . import capi
from .workloads import porous_mask

TOLERANCE = 1e-4   # relative L2 of u against the FP64 run


def make_requests(n: int, rate: float, seed: int, min_steps: int = 500, max_steps: int = 5000, small: bool = False):
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    d2_hi, d3_hi = (256, 48) if small else (2048, 160)
    for i in range(n):
        t += float(rng.exponential(1.0 / rate))
        fp16 = bool(rng.random() < 0.5)
        if rng.random() < 0.6:
            L = int(round(float(np.exp(rng.uniform(np.log(64), np.log(d2_hi))))))
            model, nx, ny, nz = "D2Q9", L + (L % 2 if fp16 else 0), 1, L
            faces = {"east": "periodic", "west": "periodic", "up": "noslip", "down": "noslip"}
            vel = {"up": (0.0, 0.0, 0.0), "down": (0.0, 0.0, 0.0)}
        else:
            L = int(round(float(np.exp(rng.uniform(np.log(32), np.log(d3_hi))))))
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


def params_of(r, storage=None, fp32_storage=capi.STORAGE_FP32_DEV):
    st = storage if storage is not None else (capi.STORAGE_FP16_DEV if r["fp16"] else fp32_storage)
    nx, ny, nz = r["dims"]
    return capi.make_params(r["model"], nx, ny, nz, r["nu"], force=(r["force"], 0.0, 0.0), face_type=r["faces"],
                            face_vel=r["vel"], semantics=capi.SEMANTICS_NATIVE, arith=capi.ARITH_FP32, storage=st)


def mask_of(r):
    nx, ny, nz = r["dims"]
    return porous_mask(nx, ny, nz, 1.0 - r["solid"], r["mask_seed"]) if r["solid"] > 0 else None


def run_plain(r, storage=None, fp32_storage=capi.STORAGE_FP32_DEV, mask=None):
    with capi.Solve(params_of(r, storage, fp32_storage)) as s:
        m = mask if mask is not None else mask_of(r)
        if m is not None:
            s.set_mask(m)
        s.initialize()
        s.step(r["steps"])
        return s.get(capi.FIELD_U)


def serve(reqs, masks, budget_gb: float = 150.0, tick: int = 250, fp32_storage=capi.STORAGE_FP32_DEV, keep=()):
    """Submits every request at its arrival time; returns per-request
    latency, admission wait and run time, the served wall time, the peak
    budget use, and u of the requests in `keep`."""
    n = len(reqs)
    lat, waits, runs = np.zeros(n), np.zeros(n), np.zeros(n)
    results = {}
    keep = set(keep)
    with capi.Server(budget_bytes=int(budget_gb * (1 << 30)), tick_steps=tick) as srv:
        ids = [None] * n
        t0 = time.perf_counter()

        def producer():
            for i, r in enumerate(reqs):
                delay = r["t"] - (time.perf_counter() - t0)
                if delay > 0:
                    time.sleep(delay)
                ids[i] = srv.submit(params_of(r, None, fp32_storage), r["steps"], masks[i])

        th = threading.Thread(target=producer)
        th.start()
        th.join()
        for i in range(n):
            srv.wait(ids[i], 3600.0)
            _, u, (ts, tadm, tdone) = srv.result(ids[i])
            lat[i], waits[i], runs[i] = tdone - ts, tadm - ts, tdone - tadm
            if i in keep:
                results[i] = u
        t_served = time.perf_counter() - t0
        _, peak = srv.memory()
    return dict(lat=lat, wait=waits, run=runs, seconds=t_served, peak=peak, results=results)


def plain(reqs, masks, fp32_storage=capi.STORAGE_FP32_DEV, keep=()):
    """The requests one after another as plain solves: each solve's service
    time, the total, and u of the requests in `keep`.  Latency on the trace:
    a first-come first-served queue, finish_i = max(arrival_i, finish_{i-1})
    + service_i."""
    n = len(reqs)
    service = np.zeros(n)
    results = {}
    keep = set(keep)
    t0 = time.perf_counter()
    for i, r in enumerate(reqs):
        ts = time.perf_counter()
        u = run_plain(r, None, fp32_storage, masks[i])
        service[i] = time.perf_counter() - ts
        if i in keep:
            results[i] = u
    total = time.perf_counter() - t0
    finish, lat = 0.0, np.zeros(n)
    for i, r in enumerate(reqs):
        finish = max(r["t"], finish) + service[i]
        lat[i] = finish - r["t"]
    return dict(service=service, seconds=total, lat=lat, results=results)


def rel_l2_u(u, u64) -> float:
    a = np.asarray(u[1:-1, 1:-1, 1:-1], np.float64)
    b = np.asarray(u64[1:-1, 1:-1, 1:-1], np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def accuracy(reqs, masks, idx, results) -> dict:
    """Relative L2 of u against an FP64 run of the same request."""
    return {i: rel_l2_u(results[i], run_plain(reqs[i], capi.STORAGE_FP64, mask=masks[i])) for i in idx}


def pct(a, q):
    return round(float(np.percentile(a, q)), 4) if len(a) else None


def summarize(reqs, served, plain_run, errs, tolerance: float = TOLERANCE) -> dict:
    n = len(reqs)
    work = np.array([float(np.prod(r["dims"])) * r["steps"] for r in reqs])
    served_rate = n / served["seconds"]
    plain_rate = n / plain_run["seconds"]
    out = {
        "requests": n, "cell_updates": float(work.sum()),
        "served": {"seconds": round(served["seconds"], 3), "solves_per_s": round(served_rate, 3),
                   "mlups": round(work.sum() / served["seconds"] / 1e6, 1),
                   "latency_p50_s": pct(served["lat"], 50), "latency_p99_s": pct(served["lat"], 99),
                   "wait_p50_s": pct(served["wait"], 50), "run_p50_s": pct(served["run"], 50),
                   "peak_budget_bytes": int(served["peak"])},
        "plain": {"seconds": round(plain_run["seconds"], 3), "solves_per_s": round(plain_rate, 3),
                  "mlups": round(work.sum() / plain_run["seconds"] / 1e6, 1),
                  "latency_p50_s": pct(plain_run["lat"], 50), "latency_p99_s": pct(plain_run["lat"], 99),
                  "service_p50_s": pct(plain_run["service"], 50)},
        "speedup_solves_per_s": round(served_rate / plain_rate, 2),
    }
    if errs:
        acc = {"tolerance": tolerance, "sampled": len(errs)}
        for name, want in (("fp32", False), ("fp16", True)):
            e = [errs[i] for i in errs if reqs[i]["fp16"] == want]
            acc[name] = {"sampled": len(e), "compliant": int(sum(x <= tolerance for x in e)),
                         "rel_l2_u_max": float(f"{max(e):.3g}") if e else None,
                         "rel_l2_u_median": float(f"{np.median(e):.3g}") if e else None}
        ok = [i for i in errs if errs[i] <= tolerance]
        acc["compliant_served_latency_p50_s"] = pct(served["lat"][ok], 50) if ok else None
        acc["compliant_served_latency_p99_s"] = pct(served["lat"][ok], 99) if ok else None
        acc["compliant_plain_latency_p50_s"] = pct(plain_run["lat"][ok], 50) if ok else None
        acc["compliant_plain_latency_p99_s"] = pct(plain_run["lat"][ok], 99) if ok else None
        if len(errs) == n:
            # every request checked: solves/s of the compliant requests alone
            # (their share of the served and plain wall times, by work)
            frac = work[ok].sum() / work.sum() if ok else 0.0
            acc["compliant_served_solves_per_s"] = round(len(ok) / (served["seconds"] * frac), 3) if ok else None
            acc["compliant_plain_solves_per_s"] = round(len(ok) / plain_run["service"][ok].sum(), 3) if ok else None
        out["accuracy_vs_fp64"] = acc
    return out


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--requests", type=int, default=200)
    ap.add_argument("--rate", type=float, default=200.0)
    ap.add_argument("--budget-gb", type=float, default=150.0)
    ap.add_argument("--tick", type=int, default=250)
    ap.add_argument("--seed", type=int, default=20261203)
    ap.add_argument("--small", action="store_true", help="only the small requests (D2Q9 <= 256^2, D3Q19 <= 48^3)")
    ap.add_argument("--accuracy-sample", type=int, default=50, help="requests checked against FP64 (-1: all)")
    ap.add_argument("--max-steps", type=int, default=5000)
    ap.add_argument("--fp32-storage", choices=sorted(FP32_STORAGE), default="dev",
                    help="storage of the FP32 half: f - w (dev) or f (plain, plbpd's)")
    a = ap.parse_args(argv)
    st32 = FP32_STORAGE[a.fp32_storage]
    reqs = make_requests(a.requests, a.rate, a.seed, max_steps=a.max_steps, small=a.small)
    masks = [mask_of(r) for r in reqs]
    n_acc = len(reqs) if a.accuracy_sample < 0 else min(a.accuracy_sample, len(reqs))
    idx = sorted(set(np.linspace(0, len(reqs) - 1, n_acc).round().astype(int).tolist())) if n_acc else []
    served = serve(reqs, masks, a.budget_gb, a.tick, st32, keep=idx)
    plain_run = plain(reqs, masks, st32)
    errs = accuracy(reqs, masks, idx, served["results"])
    print(json.dumps({"workload": "served stream" + (" (small requests)" if a.small else ""), "arrival_rate": a.rate,
                      "fp32_storage": a.fp32_storage, **summarize(reqs, served, plain_run, errs)}))


if __name__ == "__main__":
    main()
