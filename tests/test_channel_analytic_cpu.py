"""The startup-Poiseuille series itself and the oracle's channel against it,
on the CPU: the series converges to the steady parabola, and plbpd's operator
sequence in double precision (the oracle, pinned bit-exact to the reference
in float) follows it to 2e-5 after 10,000 steps of the 128 x 64 channel."""
import numpy as np

import pyoracle as po
from cases import CHANNEL


def test_series_limits():
    from plbpd_gb300.accuracy import poiseuille_startup
    z = np.linspace(0.5, 61.5, 62)
    steady = 2.08e-6 / (2 * 0.1) * z * (62.0 - z)
    np.testing.assert_allclose(poiseuille_startup(z, 1e9, 0.1, 2.08e-6, 62.0), steady, rtol=1e-12)
    assert np.abs(poiseuille_startup(z, 0.0, 0.1, 2.08e-6, 62.0)).max() < 1e-3 * steady.max()


def test_oracle_double_channel_follows_series():
    from plbpd_gb300.accuracy import channel_profile_error
    p = po.Port(**CHANNEL, precision=1)
    p.initialize()
    p.step(10000)
    err = channel_profile_error(p.get64(po.U), 10000, 0.1, 2.08e-6)
    assert err < 5e-5, err
