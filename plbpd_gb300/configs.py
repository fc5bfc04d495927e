"""Measurements of the five benchmark configurations, one dict each: the
sub-records of bench.py's JSON line, and quick runs by hand:

    python -m plbpd_gb300.configs --only c1,c2,c3,c4,c5

c1  D2Q9 128x64 channel, tau 0.8, body force 2.08e-6, 10,000 steps under
    plbpd's semantics and arithmetic: MLUPS, bit-exactness against the
    reference's own 10,000-step output (SHA-256 of n, ntmp, rho, u, passed in
    by the caller), and the relative L2 of the x-averaged velocity against the
    startup-Poiseuille series.
c2  D3Q19 256^3 periodic Taylor-Green start, tau 0.6, 2,000 steps, in four
    forms -- plbpd's arithmetic (bit-exact operator), FP32 arithmetic, FP16
    storage of f - w, FP32 storage of f - w: MLUPS, fraction of the measured
    copy bandwidth at the form's bytes per cell, and the relative L2 of rho
    and u against an FP64 run of the same start and step count.
c3  D3Q27 384^3 duct (walls on y and z, periodic x) with 15 % random spheres,
    tau 0.55, FP16 storage of f - w, 5,000 steps: MLUPS and fraction at
    109 B/cell (108 population bytes + the node-type byte); FP32 storage over
    500 steps; L2 of rho and u against FP64 after --c3-accuracy-steps steps
    (an FP64 run of all 5,000 steps takes minutes).
c4  512 D3Q19 domains (edges log-uniform in [16, 96], porosity 0.7-0.9),
    1,000 steps: one batch (a launch a step, graph-replayed; and all steps in
    one cooperative launch) against per-domain solves, FP32 and FP16.
c5  the served stream: a prefix of the mixed trace and a trace of small
    requests (at 200/s, and arriving at once to measure capacity), each
    served and run as plain solves one after another, with accuracy against
    FP64 runs (plbpd_gb300.serve_bench).

Every solve is closed before the next configuration starts.
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import time

import numpy as np

from . import capi
from .accuracy import DUCT, REST, channel_profile_error, errors, wall_layers
from .run import nu_for_tau
from .workloads import sphere_mask, taylor_green_state

TG_SEED = 20261203


def _mlups(cells: int, steps: int, seconds: float) -> float:
    return round(cells * steps / seconds / 1e6, 1)


def _frac(bytes_per_cell: float, mlups: float, peak_gbs: float) -> float:
    return round(bytes_per_cell * mlups * 1e6 / (peak_gbs * 1e9), 4)


def _timed(s: capi.Solve, steps: int) -> float:
    s.synchronize()
    t0 = time.perf_counter()
    s.step(steps)
    return time.perf_counter() - t0


# ---- c1 ------------------------------------------------------------------------
CHANNEL = dict(model="D2Q9", nx=128, ny=1, nz=64, nu=0.1, rho0=1.0, u0=(0.0, 0.0, 0.0), force=(2.08e-6, 0.0, 0.0),
               rho_solid=1.0, face_type={"east": "periodic", "west": "periodic", "up": "noslip", "down": "noslip"},
               face_vel={"up": (0.0, 0.0, 0.0), "down": (0.0, 0.0, 0.0)})


def config1(expected_sha256: dict | None = None, steps: int = 10000) -> dict:
    p = capi.make_params(**CHANNEL, semantics=capi.SEMANTICS_REFERENCE, arith=capi.ARITH_REFERENCE)
    cells = 128 * 64
    with capi.Solve(p) as s:
        s.initialize()
        s.step(steps)                       # first march: captures the step graphs
        digests = {k: hashlib.sha256(s.get(w).tobytes()).hexdigest()
                   for k, w in (("n", 0), ("ntmp", 1), ("rho", 2), ("u", 3))}
        u = s.get(capi.FIELD_U)
        s.initialize()
        sec = _timed(s, steps)
        s.synchronize()
    out = {"workload": "D2Q9 128x64 channel, tau 0.8, F 2.08e-6, plbpd semantics and arithmetic", "steps": steps,
           "mlups": _mlups(cells, steps, sec), "seconds": round(sec, 4),
           "u_rel_l2_vs_startup_poiseuille": float(f"{channel_profile_error(u, steps, 0.1, 2.08e-6):.3g}")}
    if expected_sha256:
        out["bit_exact_vs_reference"] = all(digests[k] == expected_sha256.get(k) for k in digests)
    return out


# ---- c2 ------------------------------------------------------------------------
C2_FORMS = (("reference_arith", capi.STORAGE_FP32, capi.ARITH_REFERENCE, 152),
            ("fp32_arith", capi.STORAGE_FP32, capi.ARITH_FP32, 152),
            ("fp16_storage", capi.STORAGE_FP16_DEV, capi.ARITH_FP32, 76),
            ("fp32dev_storage", capi.STORAGE_FP32_DEV, capi.ARITH_FP32, 152))


def _periodic_solve(n_side: int, storage: int, arith: int, start) -> capi.Solve:
    faces = {f: "periodic" for f in capi.FACES}
    s = capi.Solve.create("D3Q19", n_side, n_side, n_side, nu_for_tau(0.6), face_type=faces,
                          semantics=capi.SEMANTICS_NATIVE, arith=arith, storage=storage)
    s.set(capi.FIELD_N, start[0])
    s.set(capi.FIELD_RHO, start[1])
    s.set(capi.FIELD_U, start[2])
    return s


def _fields(s: capi.Solve):
    rho = s.get(capi.FIELD_RHO)[1:-1, 1:-1, 1:-1, 0].astype(np.float64)
    u = s.get(capi.FIELD_U)[1:-1, 1:-1, 1:-1, :].astype(np.float64)
    return rho, u


def config2(peak_gbs: float, steps: int = 2000, n_side: int = 256, forms=None) -> dict:
    start = taylor_green_state(n_side, seed=TG_SEED)
    cells = n_side ** 3
    t0 = time.perf_counter()
    with _periodic_solve(n_side, capi.STORAGE_FP64, capi.ARITH_FP32, start) as s:
        s.step(steps)
        rho64, u64 = _fields(s)
    fp64_sec = time.perf_counter() - t0
    fluid = np.ones(rho64.shape, bool)
    out = {"workload": f"D3Q19 {n_side}^3 periodic, Taylor-Green A=0.02 + noise, tau 0.6", "steps": steps,
           "accuracy_reference": f"FP64 storage and arithmetic, same start, {steps} steps ({fp64_sec:.1f} s)"}
    warm = 3
    for name, storage, arith, bpc in C2_FORMS:
        if forms and name not in forms:
            continue
        with _periodic_solve(n_side, storage, arith, start) as s:
            s.step(warm)
            s.tune()
            sec = _timed(s, steps - warm)
            rho, u = _fields(s)
            mlups = _mlups(cells, steps - warm, sec)
            e = errors(rho, u, rho64, u64, fluid)
            out[name] = {"mlups": mlups, "bytes_per_cell": bpc, "frac_of_copy": _frac(bpc, mlups, peak_gbs),
                         "rel_l2_u_vs_fp64": float(f"{e['rel_l2_u']:.3g}"),
                         "rel_l2_rho_vs_fp64": float(f"{e['rel_l2_rho']:.3g}"), "variant": s.variant()}
    return out


# ---- c3 ------------------------------------------------------------------------
def _duct_solve(n: int, storage: int, mask) -> capi.Solve:
    s = capi.Solve.create("D3Q27", n, n, n, nu_for_tau(0.55), u0=(0.03, 0.0, 0.0), force=(2.7e-8, 0.0, 0.0),
                          face_type=DUCT, face_vel=REST, semantics=capi.SEMANTICS_NATIVE, arith=capi.ARITH_FP32,
                          storage=storage)
    s.set_mask(mask)
    s.initialize()
    return s


def config3(peak_gbs: float, steps: int = 5000, fp32_steps: int = 500, accuracy_steps: int = 300,
            n: int = 384) -> dict:
    mask = sphere_mask(n, n, n)
    cells = n ** 3
    out = {"workload": f"D3Q27 {n}^3 duct, walls y/z, periodic x, {mask.mean() * 100:.1f} % spheres, tau 0.55",
           "solid_fraction": round(float(mask.mean()), 4)}
    for name, storage, st_steps, bpc in (("fp16_storage", capi.STORAGE_FP16_DEV, steps, 109),
                                         ("fp32_storage", capi.STORAGE_FP32, fp32_steps, 217)):
        with _duct_solve(n, storage, mask) as s:
            s.step(3)
            s.tune()
            sec = _timed(s, st_steps)
            mlups = _mlups(cells, st_steps, sec)
            out[name] = {"steps": st_steps, "mlups": mlups, "bytes_per_cell": bpc,
                         "frac_of_copy": _frac(bpc, mlups, peak_gbs), "variant": s.variant()}
    fluid = ~wall_layers(DUCT, n, n, n) & ~mask.astype(bool)
    with _duct_solve(n, capi.STORAGE_FP64, mask) as s:
        s.step(accuracy_steps)
        rho64, u64 = _fields(s)
    with _duct_solve(n, capi.STORAGE_FP16_DEV, mask) as s:
        s.step(accuracy_steps)
        rho, u = _fields(s)
    e = errors(rho, u, rho64, u64, fluid)
    out["fp16_storage"].update({"accuracy_steps": accuracy_steps, "rel_l2_u_vs_fp64": float(f"{e['rel_l2_u']:.3g}"),
                                "rel_l2_rho_vs_fp64": float(f"{e['rel_l2_rho']:.3g}")})
    return out


# ---- c4 ------------------------------------------------------------------------
def config4(steps: int = 1000, domains: int = 512, storages=("fp32", "fp16"), seed: int = 20261203) -> dict:
    from .batch_bench import build
    out = {"workload": f"{domains} D3Q19 domains, edges 16-96 log-uniform, porosity 0.7-0.9", "steps": steps}
    for st_name in storages:
        storage = capi.STORAGE_FP16_DEV if st_name == "fp16" else capi.STORAGE_FP32
        t0 = time.perf_counter()
        solves = build(domains, storage, seed)
        setup = time.perf_counter() - t0
        cells = sum(s.nx * s.ny * s.nz for s in solves)
        with capi.Batch(solves) as b:
            b.step(2)
            b.step(64)
            b.synchronize()
            t0 = time.perf_counter()
            b.step(steps)
            tb = time.perf_counter() - t0
        # the same steps as one cooperative launch with grid barriers
        prev = os.environ.get("PLB_BATCH_MULTI")
        os.environ["PLB_BATCH_MULTI"] = "1"
        try:
            with capi.Batch(solves) as b:
                b.step(2)
                b.synchronize()
                t0 = time.perf_counter()
                b.step(steps)
                tm = time.perf_counter() - t0
        finally:
            if prev is None:
                del os.environ["PLB_BATCH_MULTI"]
            else:
                os.environ["PLB_BATCH_MULTI"] = prev
        # each size class's kernel variant timed before the per-domain steps
        classes = set()
        for s in solves:
            c = (s.nx * s.ny * s.nz).bit_length()
            if c not in classes:
                classes.add(c)
                s.tune()
        for s in solves:
            s.synchronize()
        t0 = time.perf_counter()
        for s in solves:
            s.step_async(steps)
        for s in solves:
            s.synchronize()
        tp = time.perf_counter() - t0
        for s in solves:
            s.close()
        out[st_name] = {"cells": int(cells), "batch_mlups": _mlups(cells, steps, tb),
                        "batch_one_launch_mlups": _mlups(cells, steps, tm),
                        "per_domain_mlups": _mlups(cells, steps, tp), "speedup": round(tp / tb, 3),
                        "setup_seconds": round(setup, 1)}
    return out


# ---- c5 ------------------------------------------------------------------------
def config5(mixed_requests: int = 150, small_requests: int = 300, mixed_accuracy: int = 20,
            seed: int = 20261203) -> dict:
    from . import serve_bench as sb
    out = {"workload": "Poisson arrivals at 200/s; 60 % D2Q9, 40 % D3Q19; FP32 (f - w) or FP16 (f - w) 50/50; "
                       "tau 0.55-1.5; 0-20 % solid; 500-5000 steps; 150 GB admission budget",
           "tolerance_rel_l2_u_vs_fp64": sb.TOLERANCE}
    for label, n, small, n_acc, rate in (("mixed_prefix", mixed_requests, False, mixed_accuracy, 200.0),
                                         ("small_requests", small_requests, True, small_requests, 200.0),
                                         ("small_saturated", small_requests, True, 0, 5000.0)):
        reqs = sb.make_requests(n, rate, seed, small=small)
        masks = [sb.mask_of(r) for r in reqs]
        idx = sorted(set(np.linspace(0, n - 1, n_acc).round().astype(int).tolist())) if n_acc else []
        served = sb.serve(reqs, masks, 150.0, 250, keep=idx)
        plain_run = sb.plain(reqs, masks)
        errs = sb.accuracy(reqs, masks, idx, served["results"])
        rec = sb.summarize(reqs, served, plain_run, errs)
        rec["trace"] = (f"first {n} requests of the seeded trace" if not small else
                        f"{n} requests, D2Q9 edges 64-256 and D3Q19 edges 32-48, own seeded trace, "
                        f"arrivals at {rate:g}/s" + (" (all within ~0.1 s: the server's capacity)"
                                                    if rate > 1000 else ""))
        out[label] = rec
    return out


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--only", default="c1,c2,c3,c4,c5")
    ap.add_argument("--peak-gbs", type=float, default=0.0)
    ap.add_argument("--c3-accuracy-steps", type=int, default=300)
    a = ap.parse_args(argv)
    peak = a.peak_gbs
    if peak <= 0:
        try:
            import os
            with open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                                   "MEASURED_PEAKS.json")) as f:
                peak = float(json.load(f)["hbm_gbs"])
        except (OSError, KeyError, ValueError):
            peak = 6800.0
    for c in a.only.split(","):
        t0 = time.perf_counter()
        rec = {"c1": lambda: config1(), "c2": lambda: config2(peak),
               "c3": lambda: config3(peak, accuracy_steps=a.c3_accuracy_steps),
               "c4": lambda: config4(), "c5": lambda: config5()}[c]()
        rec["wall_seconds"] = round(time.perf_counter() - t0, 1)
        print(json.dumps({c: rec}), flush=True)


if __name__ == "__main__":
    main()
