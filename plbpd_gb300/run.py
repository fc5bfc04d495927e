"""Runs one named workload through the C ABI and prints its MLUPS.

    python -m plbpd_gb300.run --workload periodic --model D3Q19 --n 128 --steps 20

Workloads
  periodic  NATIVE semantics, every face periodic (the fused pull kernel
            without a node-type mask)
  duct      NATIVE semantics, periodic x, no-slip walls on y and z, body force
  channel   REFERENCE semantics, D2Q9-style channel: periodic x, walls up/down
            (plbpd's own operator sequence, bit-exact)
Used for quick measurements and for small profiler captures.
"""
from __future__ import annotations

import argparse
import json
import time

from . import capi


def params_for(workload: str, model: str, n: int, storage: str, arith: str):
    nx = ny = nz = n
    if model == "D2Q9":
        ny = 1
    st = capi.STORAGE_FP16_DEV if storage == "fp16" else capi.STORAGE_FP32
    ar = capi.ARITH_REFERENCE if arith == "reference" else capi.ARITH_FP32
    if workload == "periodic":
        faces = {f: "periodic" for f in capi.FACES}
        return capi.make_params(model, nx, ny, nz, 0.0333333, face_type=faces, u0=(0.01, 0.0, 0.0),
                                semantics=capi.SEMANTICS_NATIVE, arith=ar, storage=st)
    if workload == "duct":
        faces = {"east": "periodic", "west": "periodic", "north": "noslip", "south": "noslip", "up": "noslip",
                 "down": "noslip"}
        vel = {f: (0.0, 0.0, 0.0) for f in ("north", "south", "up", "down")}
        return capi.make_params(model, nx, ny, nz, 0.0166667, force=(1e-6, 0.0, 0.0), face_type=faces, face_vel=vel,
                                semantics=capi.SEMANTICS_NATIVE, arith=ar, storage=st)
    if workload == "channel":
        faces = {"east": "periodic", "west": "periodic", "up": "noslip", "down": "noslip"}
        vel = {"up": (0.0, 0.0, 0.0), "down": (0.0, 0.0, 0.0)}
        return capi.make_params(model, nx, ny, nz, 0.1, force=(1e-6, 0.0, 0.0), face_type=faces, face_vel=vel,
                                semantics=capi.SEMANTICS_REFERENCE, arith=ar)
    raise SystemExit(f"unknown workload {workload}")


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="periodic", choices=["periodic", "duct", "channel"])
    ap.add_argument("--model", default="D3Q19", choices=["D2Q9", "D3Q19", "D3Q27"])
    ap.add_argument("--n", type=int, default=128)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--storage", default="fp32", choices=["fp32", "fp16"])
    ap.add_argument("--arith", default="fp32", choices=["fp32", "reference"])
    a = ap.parse_args(argv)
    p = params_for(a.workload, a.model, a.n, a.storage, a.arith)
    cells = int(p.nx) * int(p.ny) * int(p.nz)
    with capi.Solve(p) as s:
        s.initialize()
        s.step(a.warmup)
        t0 = time.perf_counter()
        s.step(a.steps)
        dt = time.perf_counter() - t0
        print(json.dumps({"workload": a.workload, "model": a.model, "n": a.n, "storage": a.storage,
                          "arith": a.arith, "steps": a.steps, "mlups": round(cells * a.steps / dt / 1e6, 1),
                          "mass": s.conservation()[0]}))


if __name__ == "__main__":
    main()
