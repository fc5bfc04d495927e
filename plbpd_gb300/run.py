"""Runs one named workload through the C ABI and prints its MLUPS.

    python -m plbpd_gb300.run --workload periodic --model D3Q19 --n 128 --steps 20

Workloads
  periodic  NATIVE semantics, every face periodic (the fused pull kernel
            without a node-type mask)
  duct      NATIVE semantics, periodic x, no-slip walls on y and z, body force;
            --spheres adds the seeded random-sphere obstacles (15% solid)
  channel   REFERENCE semantics, periodic x (and y in 3D), walls up/down
            (plbpd's own operator sequence, bit-exact with the reference)
--nx/--ny/--nz override --n per axis.  Used for quick measurements and for
small profiler captures.
"""
from __future__ import annotations

import argparse
import json
import time

from . import capi


def nu_for_tau(tau: float) -> float:
    import numpy as np
    target = np.float32(tau)
    nu = np.float32((tau - 0.5) / 3.0)
    for _ in range(64):
        t = np.float32(np.float32(3.0) * nu) + np.float32(0.5)
        if t == target:
            break
        nu = np.nextafter(nu, np.float32(np.inf) if t < target else np.float32(-np.inf))
    return float(nu)


def params_for(a):
    nx, ny, nz = a.nx or a.n, a.ny or a.n, a.nz or a.n
    if a.model == "D2Q9":
        ny = 1
    st = {"fp32": capi.STORAGE_FP32, "fp16": capi.STORAGE_FP16_DEV, "fp32dev": capi.STORAGE_FP32_DEV,
          "fp64": capi.STORAGE_FP64}[a.storage]
    ar = capi.ARITH_REFERENCE if a.arith == "reference" else capi.ARITH_FP32
    col = dict(collision=capi.COLLISION_TRT if a.collision == "trt" else capi.COLLISION_BGK)
    if getattr(a, "streaming", "ab") == "aa":
        col["streaming"] = capi.STREAMING_AA
    nu = nu_for_tau(a.tau)
    if a.workload == "periodic":
        faces = {f: "periodic" for f in capi.FACES}
        return capi.make_params(a.model, nx, ny, nz, nu, face_type=faces, u0=(0.01, 0.0, 0.0),
                                semantics=capi.SEMANTICS_NATIVE, arith=ar, storage=st, **col)
    if a.workload == "duct":
        # D2Q9 moves in x-z only: its channel has walls up and down
        walls = ("up", "down") if a.model == "D2Q9" else ("north", "south", "up", "down")
        faces = {"east": "periodic", "west": "periodic", **{f: "noslip" for f in walls}}
        vel = {f: (0.0, 0.0, 0.0) for f in walls}
        return capi.make_params(a.model, nx, ny, nz, nu, force=(a.force, 0.0, 0.0), face_type=faces, face_vel=vel,
                                semantics=capi.SEMANTICS_NATIVE, arith=ar, storage=st, **col)
    if a.workload == "channel":
        # walls up and down, periodic x (and y: a face left out would be open,
        # and an open face loses mass until the flow fails)
        faces = {"east": "periodic", "west": "periodic", "up": "noslip", "down": "noslip"}
        if a.model != "D2Q9":
            faces.update(north="periodic", south="periodic")
        vel = {"up": (0.0, 0.0, 0.0), "down": (0.0, 0.0, 0.0)}
        return capi.make_params(a.model, nx, ny, nz, nu, force=(a.force, 0.0, 0.0), face_type=faces, face_vel=vel,
                                semantics=capi.SEMANTICS_REFERENCE, arith=ar, **col)
    raise SystemExit(f"unknown workload {a.workload}")


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="periodic", choices=["periodic", "duct", "channel"])
    ap.add_argument("--model", default="D3Q19", choices=["D2Q9", "D3Q19", "D3Q27"])
    ap.add_argument("--n", type=int, default=128)
    ap.add_argument("--nx", type=int, default=0)
    ap.add_argument("--ny", type=int, default=0)
    ap.add_argument("--nz", type=int, default=0)
    ap.add_argument("--tau", type=float, default=0.6)
    ap.add_argument("--force", type=float, default=1e-6)
    ap.add_argument("--spheres", action="store_true")
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--no-tune", action="store_true",
                    help="no timed trials after the warm-up: keep the variant of the first fused step (for profiling)")
    ap.add_argument("--storage", default="fp32", choices=["fp32", "fp16", "fp32dev", "fp64"])
    ap.add_argument("--collision", default="bgk", choices=["bgk", "trt"])
    ap.add_argument("--arith", default="fp32", choices=["fp32", "reference"])
    ap.add_argument("--streaming", default="ab", choices=["ab", "aa"],
                    help="two population buffers (ab) or one updated in place (aa)")
    a = ap.parse_args(argv)
    p = params_for(a)
    cells = int(p.nx) * int(p.ny) * int(p.nz)
    with capi.Solve(p) as s:
        if a.spheres:
            from .workloads import sphere_mask
            s.set_mask(sphere_mask(int(p.nx), int(p.ny), int(p.nz)))
        s.initialize()
        s.step(a.warmup)
        if not a.no_tune:
            s.tune()   # the kernel variant timed on the warmed-up state, before the timed steps
        s.synchronize()
        t0 = time.perf_counter()
        s.step(a.steps)
        dt = time.perf_counter() - t0
        print(json.dumps({"workload": a.workload, "model": a.model, "dims": [int(p.nx), int(p.ny), int(p.nz)],
                          "storage": a.storage, "arith": a.arith, "streaming": a.streaming, "spheres": a.spheres,
                          "steps": a.steps,
                          "seconds": round(dt, 4), "mlups": round(cells * a.steps / dt / 1e6, 1),
                          "mass": s.conservation()[0], "device_bytes": s.device_bytes(), "variant": s.variant()}))


if __name__ == "__main__":
    main()
