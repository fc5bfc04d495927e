"""Batched uneven domains: one batch of many D3Q19 domains against the same
domains advanced one solve (one launch) at a time.

    python -m plbpd_gb300.batch_bench --domains 512 --steps 1000

Domains (plbpd_gb300.workloads.batch_domains): cubes with edges log-uniform
in [16, 96], tau uniform in [0.55, 1.2], random 2x2x2 obstacles at porosity
uniform in [0.7, 0.9], periodic in x and resting walls elsewhere, body force
for a channel velocity of 0.02, started at equilibrium with rho = 1.
Prints one JSON line: MLUPS of the batch (tile-list kernel, graph-captured
step loop) and of the per-domain launches, and their ratio.
"""
from __future__ import annotations

import argparse
import json
import time

from . import capi
from .workloads import batch_domains, porous_mask

DUCT = {"east": "periodic", "west": "periodic", "north": "noslip", "south": "noslip", "up": "noslip",
        "down": "noslip"}
REST = {f: (0.0, 0.0, 0.0) for f in ("north", "south", "up", "down")}


def build(count: int, storage: int, seed: int):
    solves = []
    for (L, tau, por, force, mseed) in batch_domains(count, seed):
        nx = L + (L % 2 if storage == capi.STORAGE_FP16_DEV else 0)
        s = capi.Solve.create("D3Q19", nx, L, L, (tau - 0.5) / 3.0, force=(force, 0.0, 0.0), face_type=DUCT,
                              face_vel=REST, semantics=capi.SEMANTICS_NATIVE, arith=capi.ARITH_FP32,
                              storage=storage)
        s.set_mask(porous_mask(nx, L, L, por, mseed))
        s.initialize()
        solves.append(s)
    return solves


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--domains", type=int, default=512)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--plain-steps", type=int, default=0, help="steps of the per-domain form (default: --steps)")
    ap.add_argument("--storage", default="fp32", choices=["fp32", "fp16"])
    ap.add_argument("--seed", type=int, default=20261203)
    a = ap.parse_args(argv)
    storage = capi.STORAGE_FP16_DEV if a.storage == "fp16" else capi.STORAGE_FP32
    t0 = time.perf_counter()
    solves = build(a.domains, storage, a.seed)
    setup = time.perf_counter() - t0
    cells = sum(s.nx * s.ny * s.nz for s in solves)
    with capi.Batch(solves) as b:
        b.step(2)                      # first collision + one step, graphs not yet involved
        b.step(64)                     # capture the graph chunk
        t0 = time.perf_counter()
        b.step(a.steps)
        tb = time.perf_counter() - t0
    plain_steps = a.plain_steps or a.steps
    for s in solves:
        s.synchronize()
    t0 = time.perf_counter()
    for _ in range(plain_steps):
        for s in solves:
            s.step_async(1)
    for s in solves:
        s.synchronize()
    tp = time.perf_counter() - t0
    batch = cells * a.steps / tb / 1e6
    plain = cells * plain_steps / tp / 1e6
    print(json.dumps({"workload": "batched uneven domains", "domains": a.domains, "cells": cells,
                      "storage": a.storage, "steps": a.steps, "batch_seconds": round(tb, 3),
                      "batch_mlups": round(batch, 1), "plain_steps": plain_steps, "plain_seconds": round(tp, 3),
                      "plain_mlups": round(plain, 1), "speedup": round(batch / plain, 2),
                      "setup_seconds": round(setup, 1)}))
    for s in solves:
        s.close()


if __name__ == "__main__":
    main()
