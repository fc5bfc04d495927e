"""TRT collision on the GPU (NATIVE semantics) against the oracle's TRT, bit
for bit, for FP32, FP16-deviation and FP64 storage; the GPU's FP64 run
reproduces plane Poiseuille flow; batches with TRT members equal each member
run alone; TRT is refused where it is not defined."""
import numpy as np
import pytest

import pyoracle as po
from conftest import assert_bitexact
from test_gpu_native import NATIVE_CASES, compare, mask_for, perturbed_start

pytestmark = pytest.mark.gpu

# torus_d3q27 has odd nx: FP16 storage then runs the one-node kernel, not the pair kernel
CASES = ["channel_d2q9", "duct_d3q27", "obstacles_d3q19", "torus_d3q19", "torus_d3q27"]
MAGIC = {"channel_d2q9": 0.0, "duct_d3q27": 0.25, "obstacles_d3q19": 0.0, "torus_d3q19": 1.0 / 12.0,
         "torus_d3q27": 0.0}


@pytest.mark.parametrize("storage", ["fp32", "fp16", "fp64", "fp32dev"])
@pytest.mark.parametrize("case", CASES)
def test_trt_matches_oracle(case, storage):
    from plbpd_gb300 import capi
    cfg = NATIVE_CASES[case]
    mask = mask_for(case, cfg)
    port_kw = {"fp32": dict(arith=po.ARITH_FP32), "fp16": dict(arith=po.ARITH_FP16DEV),
               "fp64": dict(precision=1), "fp32dev": dict(arith=po.ARITH_FP32DEV)}[storage]
    gpu_kw = {"fp32": dict(arith=capi.ARITH_FP32), "fp16": dict(storage=capi.STORAGE_FP16_DEV, arith=capi.ARITH_FP32),
              "fp64": dict(storage=capi.STORAGE_FP64, arith=capi.ARITH_FP32),
              "fp32dev": dict(storage=capi.STORAGE_FP32_DEV, arith=capi.ARITH_FP32)}[storage]
    p = po.Port(**cfg, mode=po.MODE_NATIVE, mask=mask, trt=MAGIC[case], **port_kw)
    p._cfg = cfg
    p.initialize()
    n, rho, u = perturbed_start(p, 5)
    p.set(po.N, n); p.set(po.RHO, rho); p.set(po.U, u)
    with capi.Solve.create(**cfg, semantics=capi.SEMANTICS_NATIVE, collision=capi.COLLISION_TRT,
                           trt_magic=MAGIC[case], **gpu_kw) as s:
        if mask is not None:
            s.set_mask(mask)
        s.initialize()
        s.set(0, n); s.set(2, rho); s.set(3, u)
        done = 0
        for target in (1, 8, 120):
            p.step(target - done)
            s.step(target - done)
            done = target
            compare(s, p, mask, f"TRT {case} {storage} step {target}")
        np.testing.assert_allclose(s.conservation(), p.conservation(), rtol=1e-11, atol=1e-12)


@pytest.mark.parametrize("case", sorted(["d2q9_channel", "d3q19_xy_periodic"]))
def test_trt_reference_semantics_matches_oracle(case):
    """plbpd's operator sequence (push streaming, serial no-slip, halo
    periodicity) with the TRT collision, fused and operator by operator."""
    from cases import CASES
    from plbpd_gb300 import capi
    cfg = CASES[case]
    p = po.Port(**cfg, arith=po.ARITH_FP32, trt=0.0)
    p.initialize()
    with capi.Solve.create(**cfg, collision=capi.COLLISION_TRT) as s:
        s.initialize()
        done = 0
        for target in (1, 6, 40):
            p.step(target - done)
            s.step(target - done)
            done = target
            for name, w in (("n", 0), ("ntmp", 1), ("rho", 2), ("u", 3)):
                assert_bitexact(s.get(w), p.get(w), f"TRT {case} step {target} {name}")
        s.collide(); p.collide()
        assert_bitexact(s.get(0), p.get(0), f"TRT {case} collide")


def test_set_collision_switches_operator():
    from cases import CASES
    from plbpd_gb300 import capi
    cfg = CASES["d2q9_channel"]
    p = po.Port(**cfg, arith=po.ARITH_FP32, trt=0.25)
    p.initialize()
    with capi.Solve.create(**cfg) as s:
        s.set_collision(capi.COLLISION_TRT, 0.25)
        s.initialize()
        p.step(9)
        s.step(9)
        assert_bitexact(s.get(0), p.get(0), "TRT after plb_set_collision")


def test_trt_poiseuille_on_gpu():
    """FP64 storage, magic 3/16, tau 1.5: the steady profile is the parabola
    with walls half way between wall layer and first fluid layer."""
    from plbpd_gb300 import capi
    nz, force, tau = 18, 1e-6, 1.5
    nu = (tau - 0.5) / 3.0
    with capi.Solve.create("D2Q9", 4, 1, nz, nu, force=(force, 0, 0),
                           face_type={"east": "periodic", "west": "periodic", "up": "noslip", "down": "noslip"},
                           face_vel={"up": (0, 0, 0), "down": (0, 0, 0)}, semantics=capi.SEMANTICS_NATIVE,
                           arith=capi.ARITH_FP32, storage=capi.STORAGE_FP64, collision=capi.COLLISION_TRT) as s:
        s.initialize()
        s.step(int(40 * (nz - 2) ** 2 / nu))
        ux = s.get(capi.FIELD_U)[2:-2, 1, 2, 0].astype(np.float64)
        rho = s.get(capi.FIELD_RHO)[2:-2, 1, 2, 0].astype(np.float64)
    z = np.arange(2, nz, dtype=np.float64)
    exact = force / rho / (2 * nu) * (z - 1.5) * (nz - 0.5 - z)
    err = np.max(np.abs(ux + force / (2 * rho) - exact)) / exact.max()
    assert err < 1e-5, err


@pytest.mark.parametrize("storage", ["fp32", "fp16"])
def test_trt_batch_equals_alone(storage):
    from plbpd_gb300 import capi
    from plbpd_gb300.workloads import porous_mask
    st = capi.STORAGE_FP16_DEV if storage == "fp16" else capi.STORAGE_FP32
    rng = np.random.default_rng(9)
    faces = {"east": "periodic", "west": "periodic", "north": "noslip", "south": "noslip", "up": "noslip",
             "down": "noslip"}
    vel = {f: (0.0, 0.0, 0.0) for f in ("north", "south", "up", "down")}
    specs = []
    for i in range(5):
        L = int(rng.integers(8, 20)) * 2
        specs.append(dict(dims=(L, L - 2, L + 2), nu=float(rng.uniform(0.02, 0.2)), mask_seed=100 + i))

    def make(sp):
        nx, ny, nz = sp["dims"]
        s = capi.Solve.create("D3Q19", nx, ny, nz, sp["nu"], force=(1e-5, 0, 0), face_type=faces, face_vel=vel,
                              semantics=capi.SEMANTICS_NATIVE, arith=capi.ARITH_FP32, storage=st,
                              collision=capi.COLLISION_TRT)
        s.set_mask(porous_mask(nx, ny, nz, 0.85, sp["mask_seed"]))
        s.initialize()
        return s

    solves = [make(sp) for sp in specs]
    with capi.Batch(solves) as b:
        b.step(37)
    for sp, s in zip(specs, solves):
        with make(sp) as a:
            a.step(37)
            assert np.array_equal(s.get(capi.FIELD_U).view(np.uint32), a.get(capi.FIELD_U).view(np.uint32))
        s.close()


def test_trt_refused_where_undefined():
    from plbpd_gb300 import capi
    faces = {"east": "periodic", "west": "periodic", "up": "noslip", "down": "noslip"}
    vel = {"up": (0, 0, 0), "down": (0, 0, 0)}
    with pytest.raises(capi.PlbError):      # no such operator
        capi.Solve.create("D2Q9", 8, 1, 6, 0.1, face_type=faces, face_vel=vel, collision=7)
    with pytest.raises(capi.PlbError):      # tau must exceed 1/2
        capi.Solve.create("D2Q9", 8, 1, 6, 0.0, face_type=faces, face_vel=vel, semantics=capi.SEMANTICS_NATIVE,
                          arith=capi.ARITH_FP32, collision=capi.COLLISION_TRT)
