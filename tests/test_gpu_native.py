"""GPU parity under NATIVE semantics (fused pull kernel, periodic wrap on any
axis, wall layers and obstacle masks with bounce-back) against the oracle."""
import numpy as np
import pytest

import pyoracle as po
from conftest import assert_bitexact, rel_l2

pytestmark = pytest.mark.gpu

PERIODIC3 = {"east": "periodic", "west": "periodic", "north": "periodic", "south": "periodic",
             "up": "periodic", "down": "periodic"}

NATIVE_CASES = {
    "torus_d3q19": dict(model="D3Q19", nx=12, ny=10, nz=9, nu=0.0333333, rho0=1.0, u0=(0.01, -0.005, 0.002),
                        force=(0.0, 0.0, 0.0), rho_solid=1.0, face_type=PERIODIC3, face_vel={}),
    "torus_d3q27": dict(model="D3Q27", nx=9, ny=8, nz=11, nu=0.05, rho0=1.0, u0=(0.0, 0.01, 0.01),
                        force=(1e-5, 0.0, 0.0), rho_solid=1.0, face_type=PERIODIC3, face_vel={}),
    "channel_d2q9": dict(model="D2Q9", nx=16, ny=1, nz=10, nu=0.1, rho0=1.0, u0=(0.0, 0.0, 0.0),
                         force=(1e-5, 0.0, 0.0), rho_solid=1.0,
                         face_type={"east": "periodic", "west": "periodic", "up": "noslip", "down": "noslip"},
                         face_vel={"up": (0.05, 0.0, 0.0), "down": (0.0, 0.0, 0.0)}),
    "duct_d3q27": dict(model="D3Q27", nx=10, ny=7, nz=8, nu=0.0166667, rho0=1.0, u0=(0.01, 0.0, 0.0),
                       force=(2e-5, 0.0, 0.0), rho_solid=1.0,
                       face_type={"east": "periodic", "west": "periodic", "north": "noslip", "south": "noslip",
                                  "up": "noslip", "down": "noslip"},
                       face_vel={"up": (0.02, 0.0, 0.0), "down": (0.0, 0.0, 0.0), "north": (0.0, 0.0, 0.01),
                                 "south": (0.0, 0.0, 0.0)}),
    "obstacles_d3q19": dict(model="D3Q19", nx=14, ny=12, nz=10, nu=0.1, rho0=1.0, u0=(0.0, 0.0, 0.0),
                            force=(1e-4, 0.0, 0.0), rho_solid=1.0,
                            face_type={"east": "periodic", "west": "periodic", "north": "noslip",
                                       "south": "noslip", "up": "noslip", "down": "noslip"},
                            face_vel={"up": (0.0, 0.0, 0.0), "down": (0.0, 0.0, 0.0), "north": (0.0, 0.0, 0.0),
                                      "south": (0.0, 0.0, 0.0)}),
    "obstacles_torus_d3q27": dict(model="D3Q27", nx=10, ny=9, nz=8, nu=0.2, rho0=1.0, u0=(0.01, 0.0, 0.0),
                                  force=(1e-5, 1e-5, 0.0), rho_solid=1.0, face_type=PERIODIC3, face_vel={}),
}


def mask_for(case, cfg):
    if not case.startswith("obstacles"):
        return None
    rng = np.random.default_rng(3)
    return (rng.random((cfg["nz"], cfg["ny"], cfg["nx"])) < 0.15).astype(np.uint8)


def perturbed_start(port, seed):
    """A non-uniform RAW start: perturbed populations and fields."""
    rng = np.random.default_rng(seed)
    n = port.get(po.N)
    n = n * (1 + rng.normal(0, 1e-3, n.shape)).astype(np.float32)
    rho = port.get(po.RHO) + rng.normal(0, 1e-3, port.shape(po.RHO)).astype(np.float32)
    u = port.get(po.U) + rng.normal(0, 1e-3, port.shape(po.U)).astype(np.float32)
    return n.astype(np.float32), rho.astype(np.float32), u.astype(np.float32)


def fluid_of(port):
    solid = np.zeros((port.nz + 2, port.ny + 2, port.nx + 2), bool)
    return solid


def compare(s, p, mask, what):
    # interior only: NATIVE holds no halo state
    ns, npo = s.get(0)[1:-1, 1:-1, 1:-1], p.get(po.N)[1:-1, 1:-1, 1:-1]
    solid = np.zeros(ns.shape[:3], bool)
    if mask is not None:
        solid |= mask.astype(bool)
    ft = p_face_solid(p)
    solid |= ft
    assert_bitexact(ns[~solid], npo[~solid], f"{what} n (fluid)")
    assert_bitexact(s.get(2)[1:-1, 1:-1, 1:-1], p.get(po.RHO)[1:-1, 1:-1, 1:-1], f"{what} rho")
    assert_bitexact(s.get(3)[1:-1, 1:-1, 1:-1], p.get(po.U)[1:-1, 1:-1, 1:-1], f"{what} u")


def p_face_solid(p):
    cfg = p._cfg
    solid = np.zeros((p.nz, p.ny, p.nx), bool)
    ft = cfg["face_type"]
    if ft.get("east") == "noslip": solid[:, :, -1] = True
    if ft.get("west") == "noslip": solid[:, :, 0] = True
    if ft.get("north") == "noslip": solid[:, -1, :] = True
    if ft.get("south") == "noslip": solid[:, 0, :] = True
    if ft.get("up") == "noslip": solid[-1, :, :] = True
    if ft.get("down") == "noslip": solid[0, :, :] = True
    return solid


@pytest.mark.parametrize("arith", ["fp32", "reference", "fp16", "fp64", "fp32dev"])
@pytest.mark.parametrize("case", sorted(NATIVE_CASES))
def test_native_matches_oracle(case, arith):
    """FP32 storage with either arithmetic, FP16 deviation storage and FP64
    storage, each bit-exact against the oracle's matching mode."""
    from plbpd_gb300 import capi
    cfg = NATIVE_CASES[case]
    mask = mask_for(case, cfg)
    port_kw = {"fp32": dict(arith=po.ARITH_FP32), "reference": dict(arith=po.ARITH_AVX2),
               "fp16": dict(arith=po.ARITH_FP16DEV), "fp64": dict(precision=1),
               "fp32dev": dict(arith=po.ARITH_FP32DEV)}[arith]
    gpu_kw = {"fp32": dict(arith=capi.ARITH_FP32), "reference": dict(arith=capi.ARITH_REFERENCE),
              "fp16": dict(storage=capi.STORAGE_FP16_DEV), "fp64": dict(storage=capi.STORAGE_FP64),
              "fp32dev": dict(storage=capi.STORAGE_FP32_DEV)}[arith]
    p = po.Port(**cfg, mode=po.MODE_NATIVE, mask=mask, **port_kw)
    p._cfg = cfg
    p.initialize()
    n, rho, u = perturbed_start(p, 11)
    p.set(po.N, n); p.set(po.RHO, rho); p.set(po.U, u)
    with capi.Solve.create(**cfg, semantics=capi.SEMANTICS_NATIVE, **gpu_kw) as s:
        if mask is not None:
            s.set_mask(mask)
        s.initialize()
        s.set(0, n); s.set(2, rho); s.set(3, u)
        done = 0
        for target in (1, 7, 150):
            p.step(target - done)
            s.step(target - done)
            done = target
            compare(s, p, mask, f"{case} step {target}")
        np.testing.assert_allclose(s.conservation(), p.conservation(), rtol=1e-11, atol=1e-12)


def test_native_initialize_matches_oracle():
    from plbpd_gb300 import capi
    cfg = NATIVE_CASES["duct_d3q27"]
    p = po.Port(**cfg, mode=po.MODE_NATIVE, arith=po.ARITH_FP32)
    p._cfg = cfg
    p.initialize()
    with capi.Solve.create(**cfg, semantics=capi.SEMANTICS_NATIVE, arith=capi.ARITH_FP32) as s:
        s.initialize()
        compare(s, p, None, "init")
        p.step(5)
        s.step(5)
        compare(s, p, None, "5 steps")


@pytest.mark.parametrize("case", ["torus_d3q19", "duct_d3q27", "obstacles_d3q19"])
def test_fp16_storage_tracks_fp64_oracle(case):
    """FP16 storage of f - w with FP32 arithmetic stays close to an FP64 run."""
    from plbpd_gb300 import capi
    cfg = NATIVE_CASES[case]
    mask = mask_for(case, cfg)
    d = po.Port(**cfg, mode=po.MODE_NATIVE, precision=1, mask=mask)
    d.initialize()
    d.step(200)
    with capi.Solve.create(**cfg, semantics=capi.SEMANTICS_NATIVE, storage=capi.STORAGE_FP16_DEV) as s:
        if mask is not None:
            s.set_mask(mask)
        s.initialize()
        s.step(200)
        u16 = s.get(3)[1:-1, 1:-1, 1:-1]
        u64 = d.get64(po.U)[1:-1, 1:-1, 1:-1]
        r16 = s.get(2)[1:-1, 1:-1, 1:-1]
        r64 = d.get64(po.RHO)[1:-1, 1:-1, 1:-1]
        assert rel_l2(u16, u64) < 2e-2, rel_l2(u16, u64)
        assert rel_l2(r16, r64) < 1e-4, rel_l2(r16, r64)


def test_fp32_deviation_storage_accuracy():
    """A slow flow (u ~ 1e-5): FP32 storage of f loses most digits of u to the
    rounding of f ~ w, FP32 storage of f - w keeps them."""
    from plbpd_gb300 import capi
    cfg = dict(NATIVE_CASES["obstacles_d3q19"], force=(1e-7, 0.0, 0.0))
    mask = mask_for("obstacles_d3q19", cfg)
    d = po.Port(**cfg, mode=po.MODE_NATIVE, precision=1, mask=mask)
    d.initialize()
    d.step(300)
    u64 = d.get64(po.U)[1:-1, 1:-1, 1:-1]
    err = {}
    for name, st in (("fp32", capi.STORAGE_FP32), ("fp32dev", capi.STORAGE_FP32_DEV)):
        with capi.Solve.create(**cfg, semantics=capi.SEMANTICS_NATIVE, arith=capi.ARITH_FP32, storage=st) as s:
            s.set_mask(mask)
            s.initialize()
            s.step(300)
            err[name] = rel_l2(s.get(3)[1:-1, 1:-1, 1:-1], u64)
    assert err["fp32dev"] < 1e-4, err
    assert err["fp32dev"] < err["fp32"] / 10, err


@pytest.mark.parametrize("storage", ["fp32", "fp16"])
def test_pinned_host_buffers_transfer_directly(storage):
    """Page-locked host buffers are read and written by the layout kernels
    directly; the bytes equal the staged path's for every field."""
    from plbpd_gb300 import capi
    cfg = NATIVE_CASES["obstacles_d3q19"]
    mask = mask_for("obstacles_d3q19", cfg)
    st = capi.STORAGE_FP16_DEV if storage == "fp16" else capi.STORAGE_FP32
    with capi.Solve.create(**cfg, semantics=capi.SEMANTICS_NATIVE, arith=capi.ARITH_FP32, storage=st) as s:
        s.set_mask(mask)
        s.initialize()
        s.step(5)
        for w in (capi.FIELD_N, capi.FIELD_RHO, capi.FIELD_U):
            pinned = capi.PinnedBuffer(s.shape(w))
            s.get(w, pinned.array)
            assert_bitexact(pinned.array, s.get(w), f"get {w}")
            pinned.free()
        n = s.get(capi.FIELD_N)
        n[1:-1, 1:-1, 1:-1] *= np.float32(1.0001)
        pn = capi.PinnedBuffer(s.shape(capi.FIELD_N))
        pn.array[...] = n
        s.set(capi.FIELD_N, pn.array)
        got = s.get(capi.FIELD_N)
        with capi.Solve.create(**cfg, semantics=capi.SEMANTICS_NATIVE, arith=capi.ARITH_FP32, storage=st) as t:
            t.set_mask(mask)
            t.initialize()
            t.step(5)
            t.set(capi.FIELD_N, n)
            assert_bitexact(got, t.get(capi.FIELD_N), "set n")
        pn.free()


@pytest.mark.parametrize("case", ["obstacles_d3q19", "torus_d3q27", "channel_d2q9"])
def test_moments_read_without_populations(case):
    """rho and u read straight after a march (a gather of the moments alone,
    no population read first) equal the oracle's, and a later read of n still
    does."""
    from plbpd_gb300 import capi
    cfg = NATIVE_CASES[case]
    mask = mask_for(case, cfg)
    p = po.Port(**cfg, mode=po.MODE_NATIVE, mask=mask, arith=po.ARITH_FP32)
    p._cfg = cfg
    p.initialize()
    n, rho, u = perturbed_start(p, 5)
    p.set(po.N, n); p.set(po.RHO, rho); p.set(po.U, u)
    p.step(23)
    with capi.Solve.create(**cfg, semantics=capi.SEMANTICS_NATIVE, arith=capi.ARITH_FP32) as s:
        if mask is not None:
            s.set_mask(mask)
        s.initialize()
        s.set(0, n); s.set(2, rho); s.set(3, u)
        s.step(23)
        assert_bitexact(s.get(3)[1:-1, 1:-1, 1:-1], p.get(po.U)[1:-1, 1:-1, 1:-1], f"{case} u first")
        assert_bitexact(s.get(2)[1:-1, 1:-1, 1:-1], p.get(po.RHO)[1:-1, 1:-1, 1:-1], f"{case} rho")
        compare(s, p, mask, f"{case} after the moment reads")
