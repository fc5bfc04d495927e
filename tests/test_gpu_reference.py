"""GPU parity under REFERENCE semantics: the CUDA path against the reference's
own outputs (golden fixtures) and against the oracle, bit for bit."""
import hashlib

import numpy as np
import pytest

import pyoracle as po
from cases import CASES, CHANNEL, SOURCEMAP_CASES
from conftest import assert_bitexact, load_npz

pytestmark = pytest.mark.gpu

FIELDS = (("n", 0), ("ntmp", 1), ("rho", 2), ("u", 3))


def gpu_solve(cfg, arith=None, semantics=None):
    from plbpd_gb300 import capi
    return capi.Solve.create(**cfg, semantics=capi.SEMANTICS_REFERENCE if semantics is None else semantics,
                             arith=capi.ARITH_REFERENCE if arith is None else arith)


@pytest.mark.parametrize("pair", ["1", "0"])
@pytest.mark.parametrize("case", sorted(CASES))
def test_steps_match_reference(case, pair, monkeypatch):
    """Steps against the reference's own fields, the step in its two-node
    form wherever nx is even (the default) or in its one-node form
    (PLB_REF_PAIR=0)."""
    monkeypatch.setenv("PLB_REF_PAIR", pair)
    ref = load_npz(f"ref_{case}.npz")
    with gpu_solve(CASES[case]) as s:
        s.initialize()
        for k, w in FIELDS:
            assert_bitexact(s.get(w), ref[f"init_{k}"], f"{case} init {k}")
        done = 0
        for target in (1, 2, 5, 20):
            s.step(target - done)
            done = target
            for k, w in FIELDS:
                assert_bitexact(s.get(w), ref[f"step{target}_{k}"], f"{case} step {target} {k}")


@pytest.mark.parametrize("case", sorted(CASES))
def test_operators_match_reference(case):
    """CollisionSRT, Streaming, Boundary and CalcMoments one by one."""
    ref = load_npz(f"ref_{case}.npz")
    with gpu_solve(CASES[case]) as s:
        s.initialize()
        s.step(20)
        s.collide()
        assert_bitexact(s.get(0), ref["op_collide_n"], "collide")
        s.stream_push()
        assert_bitexact(s.get(0), ref["op_stream_n"], "stream n")
        assert_bitexact(s.get(1), ref["op_stream_ntmp"], "stream ntmp")
        s.apply_noslip()
        assert_bitexact(s.get(0), ref["op_noslip_n"], "noslip")
        s.apply_periodicity()
        assert_bitexact(s.get(0), ref["op_periodic_n"], "periodic")
        s.calc_moments()
        assert_bitexact(s.get(2), ref["op_moments_rho"], "moments rho")
        assert_bitexact(s.get(3), ref["op_moments_u"], "moments u")
        s.reset()
        assert_bitexact(s.get(2), ref["op_reset_rho"], "reset rho")
        assert_bitexact(s.get(3), ref["op_reset_u"], "reset u")


@pytest.mark.parametrize("case", sorted(SOURCEMAP_CASES))
def test_sourcemap_matches_reference(case):
    """Neighbour indexing, wall mask and periodic mapping, integer-encoded."""
    ref = load_npz(f"ref_sourcemap_{case}.npz")
    with gpu_solve(SOURCEMAP_CASES[case]) as s:
        s.initialize()
        shape = s.shape(0)
        idx = np.arange(1, np.prod(shape) + 1, dtype=np.float64)
        s.set(0, idx.astype(np.float32).reshape(shape))
        s.set(1, (-idx).astype(np.float32).reshape(shape))
        s.stream_push()
        s.apply_noslip()
        s.apply_periodicity()
        assert_bitexact(s.get(0), ref["n"], "source map n")
        assert_bitexact(s.get(1), ref["ntmp"], "source map ntmp")


@pytest.mark.parametrize("cluster,pair", [("1", "1"), ("0", "1"), ("0", "0")])
def test_channel_10000_steps_match_reference_digest(golden, monkeypatch, cluster, pair):
    """The 128 x 64 D2Q9 channel, 10,000 steps in one march: every byte of n,
    ntmp, rho and u equals the reference's -- with the march in one cluster
    launch (state in distributed shared memory) and with three launches a
    step (PLB_REF_CLUSTER=0), the step in its two-node or one-node form."""
    monkeypatch.setenv("PLB_REF_CLUSTER", cluster)
    monkeypatch.setenv("PLB_REF_PAIR", pair)
    with gpu_solve(CHANNEL) as s:
        s.initialize()
        s.step(10000)
        for k, w in FIELDS:
            d = hashlib.sha256(s.get(w).tobytes()).hexdigest()
            assert d == golden["channel_10000"][k], f"channel {k} differs from the reference"


@pytest.mark.parametrize("case", ["d3q19_xy_periodic", "d3q27_duct", "d2q9_channel"])
def test_long_march_uses_graphs_and_matches_oracle(case):
    """300 steps in one call (captured CUDA-graph chunks) equal the oracle."""
    cfg = CASES[case]
    p = po.Port(**cfg)
    p.initialize()
    p.step(300)
    with gpu_solve(cfg) as s:
        s.initialize()
        s.step(300)
        for k, w in FIELDS:
            assert_bitexact(s.get(w), p.get(w), f"{case} {k}")


@pytest.mark.parametrize("pair", ["1", "0"])
@pytest.mark.parametrize("case", sorted(CASES))
def test_fp32_arith_matches_oracle(case, pair, monkeypatch):
    """FP32-only collision arithmetic: bit-exact against the oracle's FP32 mode."""
    monkeypatch.setenv("PLB_REF_PAIR", pair)
    from plbpd_gb300 import capi
    cfg = CASES[case]
    p = po.Port(**cfg, arith=po.ARITH_FP32)
    p.initialize()
    p.step(37)
    with gpu_solve(cfg, arith=capi.ARITH_FP32) as s:
        s.initialize()
        s.step(37)
        for k, w in FIELDS:
            assert_bitexact(s.get(w), p.get(w), f"{case} {k}")


def test_user_fields_between_marches():
    """Fields set by the caller are used by the next march's first collision,
    as the reference's public SimData pointers allow."""
    cfg = CASES["d3q19_xy_periodic"]
    rng = np.random.default_rng(7)
    p = po.Port(**cfg)
    p.initialize()
    p.step(3)
    rho = p.get(po.RHO) * np.float32(1.0) + rng.normal(0, 1e-3, p.shape(po.RHO)).astype(np.float32)
    n = p.get(po.N) + rng.normal(0, 1e-4, p.shape(po.N)).astype(np.float32)
    with gpu_solve(cfg) as s:
        s.initialize()
        s.step(3)
        for obj in (p, s):
            obj.set(po.RHO, rho)
            obj.set(po.N, n)
        p.step(4)
        s.step(4)
        for k, w in FIELDS:
            assert_bitexact(s.get(w), p.get(w), k)


def test_conservation_matches_oracle():
    cfg = CASES["d3q19_xy_periodic"]
    p = po.Port(**cfg)
    p.initialize()
    p.step(11)
    with gpu_solve(cfg) as s:
        s.initialize()
        s.step(11)
        np.testing.assert_allclose(s.conservation(), p.conservation(), rtol=1e-12, atol=1e-13)


@pytest.mark.parametrize("case", ["d2q9_channel"])
@pytest.mark.parametrize("split", [(1,), (2, 3, 1), (7, 250, 9)])
def test_cluster_march_equals_three_launch_path(case, split, monkeypatch):
    """D2Q9 marches of various lengths (odd and even, first and last steps,
    caller-set fields between marches) are identical with and without the
    one-launch cluster path."""
    from plbpd_gb300 import capi
    cfg = CASES[case]
    out = {}
    for cluster in ("1", "0"):
        monkeypatch.setenv("PLB_REF_CLUSTER", cluster)
        with gpu_solve(cfg) as s:
            s.initialize()
            for i, n in enumerate(split):
                s.step(n)
                if i == 0:
                    rho = s.get(capi.FIELD_RHO)
                    rho[2:-2, 1, 2:-2, 0] *= np.float32(1.001)
                    s.set(capi.FIELD_RHO, rho)
            out[cluster] = [s.get(w) for _, w in FIELDS]
    for (k, _), a, b in zip(FIELDS, out["1"], out["0"]):
        assert_bitexact(a, b, f"{case} {split} {k}")


@pytest.mark.parametrize("case,dims", [("d3q19_xy_periodic", (130, 5, 4)), ("d3q27_duct", (256, 3, 4)),
                                       ("d3q19_thin_walls", (66, 3, 3))])
def test_pair_step_with_wide_rows(case, dims, monkeypatch):
    """Rows of several warps (and of 128-thread blocks at 256): the two-node
    step's stores across warp and block edges, and at the row's halo ends,
    give the oracle's fields, and the one-node step's."""
    cfg = dict(CASES[case], nx=dims[0], ny=dims[1], nz=dims[2])
    p = po.Port(**cfg)
    p.initialize()
    p.step(9)
    out = {}
    for pair in ("1", "0"):
        monkeypatch.setenv("PLB_REF_PAIR", pair)
        with gpu_solve(cfg) as s:
            s.initialize()
            s.step(9)
            out[pair] = [s.get(w) for _, w in FIELDS]
    for (k, w), a, b in zip(FIELDS, out["1"], out["0"]):
        assert_bitexact(a, p.get(w), f"{case} {dims} {k} pair")
        assert_bitexact(b, p.get(w), f"{case} {dims} {k} one-node")
