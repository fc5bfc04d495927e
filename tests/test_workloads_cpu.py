"""Host-side workload generators and metrics (no GPU): the Taylor-Green start
is the reference's equilibrium, the served-stream trace and the batched
domains follow their specifications, and the accuracy metrics are what they
say."""
import numpy as np
import pytest

import pyoracle as po


@pytest.fixture(scope="module")
def built():
    from plbpd_gb300 import build
    build.build()


def test_taylor_green_start_is_eqlbdist(built):
    """n = EqlbDist(rho, u) with the oracle's (and plbpd's) rounding, cell by cell."""
    from plbpd_gb300.workloads import taylor_green_state
    n, rho, u = taylor_green_state(6, seed=3)
    assert n.shape == (8, 8, 8, 19) and rho.shape == (8, 8, 8, 1) and u.shape == (8, 8, 8, 3)
    assert not n[0].any() and not n[:, :, -1].any()          # halo left at zero
    rng = np.random.default_rng(0)
    for _ in range(25):
        z, y, x = (int(v) for v in rng.integers(1, 7, 3))
        want = po.eqlb("D3Q19", float(rho[z, y, x, 0]), u[z, y, x])
        assert np.array_equal(n[z, y, x].view(np.uint32), want.astype(np.float32).view(np.uint32))
    # the same seed gives the same start
    n2, _, _ = taylor_green_state(6, seed=3)
    assert np.array_equal(n, n2)


def test_taylor_green_amplitude(built):
    from plbpd_gb300.workloads import taylor_green_state
    _, rho, u = taylor_green_state(32)
    ui = u[1:-1, 1:-1, 1:-1]
    assert abs(float(np.abs(ui[..., 0]).max()) - 0.02) < 2e-3
    assert float(np.abs(ui[..., 2]).max()) < 1e-3               # noise only
    assert abs(float(rho[1:-1, 1:-1, 1:-1].mean()) - 1.0) < 1e-4


def test_served_trace_follows_config():
    """60 % D2Q9 with L in [64, 2048], 40 % D3Q19 with L in [32, 160], FP16
    half the time with even nx, tau in [0.55, 1.5], 0-20 % solid, 500-5000
    steps, Poisson arrivals at the given rate; seeded."""
    from plbpd_gb300.serve_bench import make_requests
    reqs = make_requests(4000, 200.0, 20261203)
    assert reqs == make_requests(4000, 200.0, 20261203)
    d2 = [r for r in reqs if r["model"] == "D2Q9"]
    d3 = [r for r in reqs if r["model"] == "D3Q19"]
    assert abs(len(d2) / len(reqs) - 0.6) < 0.03
    assert all(64 <= r["dims"][0] <= 2049 and r["dims"][1] == 1 for r in d2)
    assert all(32 <= r["dims"][1] <= 160 for r in d3)
    assert all(r["dims"][0] % 2 == 0 for r in reqs if r["fp16"])
    assert abs(np.mean([r["fp16"] for r in reqs]) - 0.5) < 0.03
    assert all(0.55 <= r["tau"] <= 1.5 and 0.0 <= r["solid"] <= 0.2 and 500 <= r["steps"] <= 5000 for r in reqs)
    gaps = np.diff([0.0] + [r["t"] for r in reqs])
    assert abs(gaps.mean() - 1.0 / 200.0) < 0.1 / 200.0


def test_batched_domains_follow_config():
    from plbpd_gb300.workloads import batch_domains
    doms = batch_domains(512)
    assert len(doms) == 512
    L = np.array([d[0] for d in doms])
    assert L.min() >= 16 and L.max() <= 96
    assert all(0.55 <= d[1] <= 1.2 and 0.7 <= d[2] <= 0.9 for d in doms)
    # log-uniform edges: the median edge is near the geometric mean of the range
    assert abs(np.median(L) - np.sqrt(16 * 96)) < 6


def test_accuracy_metrics():
    from plbpd_gb300.accuracy import errors, wall_layers
    rng = np.random.default_rng(1)
    rho64 = 1.0 + 1e-3 * rng.standard_normal((4, 5, 6))
    u64 = 1e-2 * rng.standard_normal((4, 5, 6, 3))
    fluid = np.ones((4, 5, 6), bool)
    e = errors(rho64, u64, rho64, u64, fluid)
    assert e["rel_l2_u"] == 0.0 and e["rel_l2_rho"] == 0.0 and e["max_abs_u"] == 0.0
    e = errors(rho64, u64 * 1.001, rho64, u64, fluid)
    assert abs(e["rel_l2_u"] - 1e-3) < 1e-9
    # a density that FP64 keeps at 1 has no meaningful relative deviation
    e = errors(np.ones((4, 5, 6)), u64, np.ones((4, 5, 6)), u64, fluid)
    assert e["rel_l2_drho"] is None
    walls = wall_layers({"north": "noslip", "south": "noslip", "east": "periodic"}, 6, 5, 4)
    assert walls[:, 0, :].all() and walls[:, -1, :].all() and not walls[:, 1:-1, :].any()
