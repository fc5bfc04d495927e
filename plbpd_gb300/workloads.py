"""Seeded synthetic geometry for the benchmark configurations.

sphere_mask: random spheres (radius uniform in [rmin, rmax]) dropped at
uniform positions until the solid fraction reaches the target; periodic axes
wrap, the others clip.  porous_mask: the same with small radii, to a target
porosity (fluid fraction).  Both return uint8 arrays (nz, ny, nx), 1 = solid.
taylor_green_state: the D3Q19 Taylor-Green start of the 256^3 periodic
workload in plbpd's Field layout.
"""
from __future__ import annotations

import numpy as np


def sphere_mask(nx: int, ny: int, nz: int, solid_fraction: float = 0.15, rmin: float = 4.0, rmax: float = 12.0,
                seed: int = 20261203, wrap=(True, False, False)) -> np.ndarray:
    rng = np.random.default_rng(seed)
    mask = np.zeros((nz, ny, nx), np.uint8)
    target = solid_fraction * mask.size
    solid = 0
    while solid < target:
        r = rng.uniform(rmin, rmax)
        c = rng.uniform((0, 0, 0), (nx, ny, nz))
        R = int(np.ceil(r))
        ranges = []
        for ax, (n, w) in enumerate(zip((nx, ny, nz), wrap)):
            lo, hi = int(np.floor(c[ax])) - R, int(np.floor(c[ax])) + R + 1
            idx = np.arange(lo, hi)
            if w:
                idx = np.mod(idx, n)
                d = np.arange(lo, hi) + 0.5 - c[ax]
            else:
                keep = (idx >= 0) & (idx < n)
                d = (idx + 0.5 - c[ax])[keep]
                idx = idx[keep]
            ranges.append((idx, d))
        (ix, dx), (iy, dy), (iz, dz) = ranges
        if ix.size == 0 or iy.size == 0 or iz.size == 0:
            continue
        inside = (dz[:, None, None] ** 2 + dy[None, :, None] ** 2 + dx[None, None, :] ** 2) <= r * r
        sub = mask[np.ix_(iz, iy, ix)]
        before = int(sub.sum())
        sub |= inside.astype(np.uint8)
        mask[np.ix_(iz, iy, ix)] = sub
        solid += int(sub.sum()) - before
    return mask


def porous_mask(nx: int, ny: int, nz: int, porosity: float, seed: int) -> np.ndarray:
    """Random obstacles of 2x2x2 cells: a coarse random field at half
    resolution, solid where below 1 - porosity, upsampled."""
    rng = np.random.default_rng(seed)
    coarse = rng.random(((nz + 1) // 2, (ny + 1) // 2, (nx + 1) // 2)) < (1.0 - porosity)
    fine = np.repeat(np.repeat(np.repeat(coarse, 2, axis=0), 2, axis=1), 2, axis=2)
    return np.ascontiguousarray(fine[:nz, :ny, :nx]).astype(np.uint8)


def batch_domains(count: int = 512, seed: int = 20261203, lmin: int = 16, lmax: int = 96):
    """The batched workload: `count` cubes with edges log-uniform in
    [lmin, lmax], tau uniform in [0.55, 1.2], porosity uniform in [0.7, 0.9],
    periodic in x with resting walls elsewhere, body force for a channel
    velocity of 0.02.  Yields (edge, tau, porosity, force_x, mask_seed)."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        L = int(round(float(np.exp(rng.uniform(np.log(lmin), np.log(lmax))))))
        tau = float(rng.uniform(0.55, 1.2))
        por = float(rng.uniform(0.7, 0.9))
        nu = (tau - 0.5) / 3.0
        h = max(L - 2, 1)
        force = 8.0 * nu * 0.02 / (h * h)
        out.append((L, tau, por, force, seed + 1 + i))
    return out


def taylor_green_state(n_side: int, out_n=None, out_rho=None, out_u=None, seed: int = 20261203):
    """rho = 1 + 1e-3 N(0,1), u = Taylor-Green of amplitude 0.02 + 1e-4 N(0,1)
    per component on a 2 pi / n grid, and n = EqlbDist(rho, u) with the
    rounding of src/EqlbDist.hpp:26-38, on the interior of plbpd-layout D3Q19
    arrays (n+2, n+2, n+2, V).  Returns (n, rho, u)."""
    from . import capi
    q = 19
    rng = np.random.default_rng(seed)
    N = n_side
    shape3 = (N, N, N)
    rho = (1.0 + 1e-3 * rng.standard_normal(shape3)).astype(np.float32)
    ax = 2.0 * np.pi * np.arange(N) / N
    zc, yc, xc = np.meshgrid(ax, ax, ax, indexing="ij")
    A = 0.02
    ux = (A * np.sin(xc) * np.cos(yc) * np.cos(zc) + 1e-4 * rng.standard_normal(shape3)).astype(np.float32)
    uy = (-A * np.cos(xc) * np.sin(yc) * np.cos(zc) + 1e-4 * rng.standard_normal(shape3)).astype(np.float32)
    uz = (1e-4 * rng.standard_normal(shape3)).astype(np.float32)
    del zc, yc, xc
    full = (N + 2, N + 2, N + 2)
    n_arr = out_n if out_n is not None else np.zeros(full + (q,), np.float32)
    r_arr = out_rho if out_rho is not None else np.zeros(full + (1,), np.float32)
    u_arr = out_u if out_u is not None else np.zeros(full + (3,), np.float32)
    r_arr[1:-1, 1:-1, 1:-1, 0] = rho
    u_arr[1:-1, 1:-1, 1:-1, 0] = ux
    u_arr[1:-1, 1:-1, 1:-1, 1] = uy
    u_arr[1:-1, 1:-1, 1:-1, 2] = uz
    c, w, _, _ = capi.model_tables("D3Q19")
    usq = (ux * ux + uy * uy) + uz * uz
    for k in range(q):
        cu = (np.float32(c[k, 0]) * ux + np.float32(c[k, 1]) * uy) + np.float32(c[k, 2]) * uz
        wr = (w[k] * rho).astype(np.float64)
        cud = cu.astype(np.float64)
        br = 1.0 + 3.0 * cud + 4.5 * cud * cud - 1.5 * usq.astype(np.float64)
        n_arr[1:-1, 1:-1, 1:-1, k] = (wr * br).astype(np.float32)
    return n_arr, r_arr, u_arr
