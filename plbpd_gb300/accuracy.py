"""Accuracy of each benchmark configuration against an FP64 run of the same method.

    python -m plbpd_gb300.accuracy --config 2 --storages fp32,fp16,fp32dev

Each storage runs the configuration's workload on the GPU from the same start
as a run in FP64 storage (FP64 populations, FP64 arithmetic, exact weights:
the same method without rounding to speak of), and one JSON line per storage
gives, over the fluid nodes,
    rel_l2_u      ||u - u64|| / ||u64||
    rel_l2_rho    ||rho - rho64|| / ||rho64||
    rel_l2_drho   ||rho - rho64|| / ||rho64 - 1||   (the density deviation)
and the largest |u - u64|.

Configurations (NATIVE semantics throughout; REFERENCE semantics is
bit-exact with plbpd itself):
    1  D2Q9 128 x 64 channel, tau 0.8, body force 2.08e-6, 10,000 steps
    2  D3Q19 256^3 periodic Taylor-Green start, tau 0.6, 2,000 steps
    3  D3Q27 384^3 duct with 15 % random spheres, tau 0.55, started at the
       inlet velocity u = (0.03, 0, 0) and driven by the body force that holds
       it as a duct flow (2.7e-8), 5,000 steps
    4  a sample of the batched domains (a batch advances each exactly as a
       single solve), 1,000 steps
--n and --steps shrink a configuration for a quick look.
"""
from __future__ import annotations

import argparse
import json

import numpy as np

from . import capi
from .run import nu_for_tau
from .workloads import batch_domains, porous_mask, sphere_mask, taylor_green_state

STORAGES = {"fp32": capi.STORAGE_FP32, "fp16": capi.STORAGE_FP16_DEV, "fp32dev": capi.STORAGE_FP32_DEV,
            "fp64": capi.STORAGE_FP64}
DUCT = {"east": "periodic", "west": "periodic", "north": "noslip", "south": "noslip", "up": "noslip",
        "down": "noslip"}
REST = {f: (0.0, 0.0, 0.0) for f in ("north", "south", "up", "down")}


def poiseuille_startup(zeta, t: float, nu: float, g: float, h: float, terms: int = 4001) -> np.ndarray:
    """Plane Poiseuille flow started from rest: the velocity at distance zeta
    from one wall of a channel of width h, t time units after an acceleration
    g is switched on (kinematic viscosity nu).  The series solution of the
    diffusion equation with no-slip walls:
        u = g h^2 / (2 nu) [ (zeta/h)(1 - zeta/h)
                             - sum_{n odd} 8/(n pi)^3 sin(n pi zeta/h) exp(-(n pi)^2 nu t / h^2) ]"""
    zeta = np.asarray(zeta, np.float64)
    x = zeta / h
    s = x * (1.0 - x)
    for n in range(1, terms, 2):
        a = (n * np.pi) ** 2 * nu * t / (h * h)
        if a > 700.0:
            break
        s = s - 8.0 / (n * np.pi) ** 3 * np.sin(n * np.pi * x) * np.exp(-a)
    return g * h * h / (2.0 * nu) * s


def channel_profile_error(u: np.ndarray, steps: int, nu: float, force: float) -> float:
    """Relative L2 error of the x-averaged velocity profile of a body-force
    driven channel (plbpd's field layout (nz+2, ny+2, nx+2, 3), wall layers on
    the first and last interior z layers, half-way walls 1.5 and nz + 0.5)
    against poiseuille_startup.  plbpd's velocity is the moment sum c f / rho
    (src/CalcMoments.hpp:28-36), which the forcing scheme (u + F tau / rho in
    the equilibrium) leaves half a force step behind the fluid velocity, so
    F/2 is added before comparing."""
    nz = u.shape[0] - 2
    prof = np.asarray(u[2:nz, 1, 1:-1, 0], np.float64).mean(axis=1) + 0.5 * force
    zeta = np.arange(2, nz, dtype=np.float64) - 1.5
    ref = poiseuille_startup(zeta, float(steps), nu, force, float(nz - 2))
    return float(np.linalg.norm(prof - ref) / np.linalg.norm(ref))


def wall_layers(faces: dict, nx: int, ny: int, nz: int) -> np.ndarray:
    solid = np.zeros((nz, ny, nx), bool)
    if faces.get("east") == "noslip": solid[:, :, -1] = True
    if faces.get("west") == "noslip": solid[:, :, 0] = True
    if faces.get("north") == "noslip": solid[:, -1, :] = True
    if faces.get("south") == "noslip": solid[:, 0, :] = True
    if faces.get("up") == "noslip": solid[-1, :, :] = True
    if faces.get("down") == "noslip": solid[0, :, :] = True
    return solid


def run_case(model, dims, nu, faces, vel, force, u0, storage, steps, mask=None, start=None):
    nx, ny, nz = dims
    p = capi.make_params(model, nx, ny, nz, nu, u0=u0, force=force, face_type=faces, face_vel=vel,
                         semantics=capi.SEMANTICS_NATIVE, arith=capi.ARITH_FP32, storage=storage)
    with capi.Solve(p) as s:
        if mask is not None:
            s.set_mask(mask)
        s.initialize()
        if start is not None:
            s.set(capi.FIELD_N, start[0])
            s.set(capi.FIELD_RHO, start[1])
            s.set(capi.FIELD_U, start[2])
        s.step(steps)
        rho = s.get(capi.FIELD_RHO)[1:-1, 1:-1, 1:-1, 0].astype(np.float64)
        u = s.get(capi.FIELD_U)[1:-1, 1:-1, 1:-1, :].astype(np.float64)
    return rho, u


def errors(rho, u, rho64, u64, fluid):
    dr = (rho - rho64)[fluid]
    du = (u - u64)[fluid]
    n_u64 = np.linalg.norm(u64[fluid])
    n_r64 = np.linalg.norm(rho64[fluid])
    n_d64 = np.linalg.norm(rho64[fluid] - 1.0)
    # the density deviation is meaningless where FP64 keeps rho at 1 to float precision
    resolved = n_d64 > 1e-6 * np.sqrt(max(dr.size, 1))
    return {"rel_l2_u": float(np.linalg.norm(du) / max(n_u64, 1e-300)),
            "rel_l2_rho": float(np.linalg.norm(dr) / max(n_r64, 1e-300)),
            "rel_l2_drho": float(np.linalg.norm(dr) / n_d64) if resolved else None,
            "max_abs_u": float(np.abs(du).max()) if du.size else 0.0,
            "u64_rms": float(n_u64 / max(np.sqrt(du.size / 3), 1.0))}


def cases(config: int, n: int | None, sample: int):
    """Yields (label, model, dims, nu, faces, vel, force, u0, mask, start, steps)."""
    if config == 1:
        faces = {"east": "periodic", "west": "periodic", "up": "noslip", "down": "noslip"}
        vel = {"up": (0.0, 0.0, 0.0), "down": (0.0, 0.0, 0.0)}
        nx, nz = (n or 128), (n or 128) // 2
        yield ("D2Q9 channel", "D2Q9", (nx, 1, nz), nu_for_tau(0.8), faces, vel, (2.08e-6, 0.0, 0.0), (0.0, 0.0, 0.0),
               None, None, 10000)
    elif config == 2:
        N = n or 256
        start = taylor_green_state(N)
        faces = {f: "periodic" for f in capi.FACES}
        yield ("D3Q19 periodic Taylor-Green", "D3Q19", (N, N, N), nu_for_tau(0.6), faces, {}, (0.0, 0.0, 0.0),
               (0.0, 0.0, 0.0), None, start, 2000)
    elif config == 3:
        N = n or 384
        mask = sphere_mask(N, N, N)
        yield ("D3Q27 duct with spheres", "D3Q27", (N, N, N), nu_for_tau(0.55), DUCT, REST, (2.7e-8, 0.0, 0.0),
               (0.03, 0.0, 0.0), mask, None, 5000)
    elif config == 4:
        for (L, tau, por, force, mseed) in batch_domains(512)[:sample]:
            nx = L + L % 2
            yield (f"batched domain L={L}", "D3Q19", (nx, L, L), (tau - 0.5) / 3.0, DUCT, REST, (force, 0.0, 0.0),
                   (0.0, 0.0, 0.0), porous_mask(nx, L, L, por, mseed), None, 1000)
    else:
        raise SystemExit(f"unknown config {config}")


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", type=int, required=True, choices=[1, 2, 3, 4])
    ap.add_argument("--storages", default="fp32,fp16,fp32dev")
    ap.add_argument("--n", type=int, default=0, help="edge length override (smaller, quicker)")
    ap.add_argument("--steps", type=int, default=0, help="step count override")
    ap.add_argument("--sample", type=int, default=8, help="config 4: domains compared")
    a = ap.parse_args(argv)
    storages = [x for x in a.storages.split(",") if x]
    for (label, model, dims, nu, faces, vel, force, u0, mask, start, steps) in cases(a.config, a.n or None, a.sample):
        steps = a.steps or steps
        nx, ny, nz = dims
        fluid = ~wall_layers(faces, nx, ny, nz)
        if mask is not None:
            fluid &= ~mask.astype(bool)
        rho64, u64 = run_case(model, dims, nu, faces, vel, force, u0, capi.STORAGE_FP64, steps, mask, start)
        for st in storages:
            rho, u = run_case(model, dims, nu, faces, vel, force, u0, STORAGES[st], steps, mask, start)
            print(json.dumps({"config": a.config, "case": label, "dims": list(dims), "steps": steps, "storage": st,
                              "vs": "fp64", **errors(rho, u, rho64, u64, fluid)}), flush=True)


if __name__ == "__main__":
    main()
