"""Seeded synthetic geometry for the benchmark configurations.

sphere_mask: random spheres (radius uniform in [rmin, rmax]) dropped at
uniform positions until the solid fraction reaches the target; periodic axes
wrap, the others clip.  porous_mask: the same with small radii, to a target
porosity (fluid fraction).  Both return uint8 arrays (nz, ny, nx), 1 = solid.
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


def porous_mask(nx: int, ny: int, nz: int, porosity: float, seed: int, wrap=(True, False, False)) -> np.ndarray:
    return sphere_mask(nx, ny, nz, solid_fraction=1.0 - porosity, rmin=1.0, rmax=3.0, seed=seed, wrap=wrap)
