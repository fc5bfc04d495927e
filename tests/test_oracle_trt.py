"""The oracle's TRT operator (an extension through plbpd's Collision base,
src/Collision.hpp:10-21).  plbpd has no TRT, so the operator is pinned on
physics: with magic 3/16 the half-way bounce-back wall sits exactly half way
between the wall layer and the first fluid layer, so steady plane Poiseuille
flow is reproduced for any tau, where BGK's wall slip grows with tau."""
import numpy as np
import pytest

import pyoracle as po

CHANNEL = {"east": "periodic", "west": "periodic", "up": "noslip", "down": "noslip"}
STILL = {"up": (0.0, 0.0, 0.0), "down": (0.0, 0.0, 0.0)}


def poiseuille_error(tau, trt, nz=18, force=1e-6, precision=1, arith=po.ARITH_FP32):
    nu = (tau - 0.5) / 3.0
    steps = int(40 * (nz - 2) ** 2 / nu)          # 40 viscous times: steady
    p = po.Port("D2Q9", 4, 1, nz, nu, 1.0, (0, 0, 0), (force, 0, 0), 1.0, CHANNEL, STILL, mode=po.MODE_NATIVE,
                arith=arith, precision=precision, trt=trt)
    p.initialize()
    p.step(steps)
    ux = p.get64(po.U)[2:-2, 1, 2, 0]            # fluid layers z = 2 .. nz-1
    rho = p.get64(po.RHO)[2:-2, 1, 2, 0]
    z = np.arange(2, nz, dtype=np.float64)
    exact = force / rho / (2 * nu) * (z - 1.5) * (nz - 0.5 - z)   # walls half way
    # u reported as sum(c f)/rho; the physical velocity adds F/(2 rho)
    return float(np.max(np.abs(ux + force / (2 * rho) - exact)) / exact.max())


@pytest.mark.parametrize("tau", [0.6, 1.5, 3.0])
def test_trt_poiseuille_exact_for_any_tau(tau):
    assert poiseuille_error(tau, trt=0.0) < 1e-5


def test_bgk_wall_slip_grows_with_tau():
    # the contrast that TRT removes: BGK's error at tau = 3 is large
    assert poiseuille_error(3.0, trt=None) > 5e-2


@pytest.mark.parametrize("arith,tol", [(po.ARITH_FP32, 5e-3), (po.ARITH_FP16DEV, 5e-2)])
def test_trt_float_paths_track_the_exact_profile(arith, tol):
    # FP32 arithmetic, and FP16-deviation storage, with TRT
    assert poiseuille_error(1.0, trt=0.0, precision=0, arith=arith, force=1e-5) < tol


def test_trt_rejected_where_undefined():
    with pytest.raises(ValueError):   # plbpd's own arithmetic is BGK only
        po.Port("D2Q9", 4, 1, 6, 0.1, 1.0, (0, 0, 0), (0, 0, 0), 1.0, CHANNEL, STILL, mode=po.MODE_NATIVE,
                arith=po.ARITH_AVX2, trt=0.0)
    with pytest.raises(ValueError):   # tau must exceed 1/2
        po.Port("D2Q9", 4, 1, 6, 0.0, 1.0, (0, 0, 0), (0, 0, 0), 1.0, CHANNEL, STILL, mode=po.MODE_NATIVE,
                arith=po.ARITH_FP32, trt=0.0)


def test_trt_conserves_mass_and_momentum_without_force():
    p = po.Port("D3Q19", 6, 5, 4, 0.05, 1.0, (0.01, 0.0, 0.0), (0, 0, 0), 1.0,
                {f: "periodic" for f in ("east", "west", "north", "south", "up", "down")}, {},
                mode=po.MODE_NATIVE, precision=1, trt=0.25)
    p.initialize()
    before = p.conservation()
    p.step(50)
    after = p.conservation()
    np.testing.assert_allclose(after, before, rtol=1e-12, atol=1e-13)
