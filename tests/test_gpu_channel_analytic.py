"""The 128 x 64 D2Q9 channel (tau 0.8, body force 2.08e-6, 10,000 steps)
against plane Poiseuille flow started from rest (the series solution,
plbpd_gb300.accuracy.poiseuille_startup), walls half way between the wall
layers and the fluid (z = 1.5 and 63.5 in plbpd's coordinates, width 62), the
velocity compared half a force step ahead (u + F/2: plbpd reports the moment
sum c f / rho, src/CalcMoments.hpp:28-36, which its forcing, u + F tau / rho
in the equilibrium, leaves F/2 behind the fluid velocity).

Under plbpd's semantics and arithmetic the run is bit-exact with plbpd, so its
distance from the series is plbpd's own: FP32 storage of populations near the
weights rounds u ~ 1e-2 to about 3e-3 relative (the FP64 form of the same
operator sequence, in the oracle, is 1.8e-5 from the series).  NATIVE
semantics with FP32 storage of f - w or FP64 storage keeps the digits and
shows the method's own error: BGK with half-way bounce-back at tau = 0.8 on a
62-node channel, 1.5e-4 (FP64), 1.1e-4 (FP32 of f - w)."""
import pytest

from cases import CHANNEL

pytestmark = pytest.mark.gpu

STEPS = 10000


def channel_u(capi, semantics, **kw):
    with capi.Solve.create(**CHANNEL, semantics=semantics, **kw) as s:
        s.initialize()
        s.step(STEPS)
        return s.get(capi.FIELD_U)


def test_reference_semantics_channel_vs_startup_poiseuille():
    from plbpd_gb300 import capi
    from plbpd_gb300.accuracy import channel_profile_error
    u = channel_u(capi, capi.SEMANTICS_REFERENCE, arith=capi.ARITH_REFERENCE)
    err = channel_profile_error(u, STEPS, 0.1, 2.08e-6)
    assert err < 4e-3, err          # 3.03e-3: plbpd's FP32 rounding, bit for bit


@pytest.mark.parametrize("storage,bound", [("fp64", 2.5e-4), ("fp32dev", 2.5e-4)])
def test_native_channel_vs_startup_poiseuille(storage, bound):
    from plbpd_gb300 import capi
    from plbpd_gb300.accuracy import channel_profile_error
    st = {"fp64": capi.STORAGE_FP64, "fp32dev": capi.STORAGE_FP32_DEV}[storage]
    u = channel_u(capi, capi.SEMANTICS_NATIVE, arith=capi.ARITH_FP32, storage=st)
    err = channel_profile_error(u, STEPS, 0.1, 2.08e-6)
    assert err < bound, err
