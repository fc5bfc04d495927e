"""The oracle (oracle/lbm_oracle.c) against the reference: golden fixtures made
by the reference's own code, the reference's unit-test known answers, and --
where the reference was compiled here -- the reference run live."""
import os

import numpy as np
import pytest

import pyoracle as po
from cases import CASES, CHANNEL, SOURCEMAP_CASES
from conftest import assert_bitexact, load_npz

# TestEqlbDist.cpp:22-26: D2Q9, rho = 1, u = (0.5, 0.5, -0.5), squared error == 0
EQLB_TESTFILE = [-0.05555555597, 0.277777791, -0.05555555597, -0.05555555597, 0.277777791,
                 -0.003472222248, -0.003472222248, 0.2048611194, 0.03819444403]


def port_of(cfg, **kw):
    return po.Port(**cfg, **kw)


def test_eqlb_known_answer(golden):
    got = po.eqlb("D2Q9", 1.0, (0.5, 0.5, -0.5))
    assert_bitexact(got, np.array(EQLB_TESTFILE, np.float32), "TestEqlbDist vector")
    assert_bitexact(got, np.array(golden["eqlb_d2q9_rho1_u_05_05_m05"], np.float32), "reference EqlbDist")


@pytest.mark.parametrize("model", ["D2Q9", "D3Q19", "D3Q27"])
def test_model_tables(golden, model):
    c, w, rev, cs2 = po.model_tables(model)
    g = golden[f"tables_{model}"]
    assert c.ravel().tolist() == g["c"]
    assert w.view(np.uint32).tolist() == g["w_bits"]
    assert rev.tolist() == g["rev"]
    assert int(np.float32(cs2).view(np.uint32)) == g["cs2_bits"]
    # TestLBModel.cpp: cs2 == 1.0f/3.0f, opposite velocities
    assert cs2 == np.float32(1.0) / np.float32(3.0)
    assert np.array_equal(c[rev], -c)


def test_unknown_model_rejected():
    with pytest.raises(ValueError):
        po.Port(model="D3Q19", nx=0, ny=1, nz=1, nu=0.1, rho0=1, u0=(0, 0, 0), force=(0, 0, 0), rho_solid=1,
                face_type={}, face_vel={})


@pytest.mark.parametrize("case", sorted(CASES))
def test_port_matches_reference_fixtures(case):
    ref = load_npz(f"ref_{case}.npz")
    p = port_of(CASES[case])
    p.initialize()
    for k, w in (("n", po.N), ("ntmp", po.NTMP), ("rho", po.RHO), ("u", po.U)):
        assert_bitexact(p.get(w), ref[f"init_{k}"], f"{case} init {k}")
    done = 0
    for target in (1, 2, 5, 20):
        p.step(target - done)
        done = target
        for k, w in (("n", po.N), ("ntmp", po.NTMP), ("rho", po.RHO), ("u", po.U)):
            assert_bitexact(p.get(w), ref[f"step{target}_{k}"], f"{case} step {target} {k}")
    p.collide()
    assert_bitexact(p.get(po.N), ref["op_collide_n"], "collide")
    p.stream()
    assert_bitexact(p.get(po.N), ref["op_stream_n"], "stream n")
    assert_bitexact(p.get(po.NTMP), ref["op_stream_ntmp"], "stream ntmp")
    p.noslip()
    assert_bitexact(p.get(po.N), ref["op_noslip_n"], "noslip")
    p.periodic()
    assert_bitexact(p.get(po.N), ref["op_periodic_n"], "periodic")
    p.moments()
    assert_bitexact(p.get(po.RHO), ref["op_moments_rho"], "moments rho")
    assert_bitexact(p.get(po.U), ref["op_moments_u"], "moments u")
    p.reset()
    assert_bitexact(p.get(po.RHO), ref["op_reset_rho"], "reset rho")
    assert_bitexact(p.get(po.U), ref["op_reset_u"], "reset u")


@pytest.mark.parametrize("case", sorted(SOURCEMAP_CASES))
def test_port_sourcemap(case):
    ref = load_npz(f"ref_sourcemap_{case}.npz")
    p = port_of(SOURCEMAP_CASES[case])
    p.initialize()
    shape = p.shape(po.N)
    idx = np.arange(1, np.prod(shape) + 1, dtype=np.float64)
    p.set(po.N, idx.astype(np.float32).reshape(shape))
    p.set(po.NTMP, (-idx).astype(np.float32).reshape(shape))
    p.stream()
    p.noslip()
    p.periodic()
    assert_bitexact(p.get(po.N), ref["n"], "source map n")
    assert_bitexact(p.get(po.NTMP), ref["ntmp"], "source map ntmp")


def test_port_channel_digest(golden):
    import hashlib
    p = port_of(CHANNEL)
    p.initialize()
    p.step(10000)
    for k, w in (("n", po.N), ("ntmp", po.NTMP), ("rho", po.RHO), ("u", po.U)):
        d = hashlib.sha256(p.get(w).tobytes()).hexdigest()
        assert d == golden["channel_10000"][k], f"channel {k} digest differs from the reference's"


# ---- live reference (only where it was compiled) ------------------------------
needs_ref = pytest.mark.skipif(not po.ref_available("avx2"), reason="reference not compiled here (oracle/_ref)")


def random_config(rng):
    model = rng.choice(["D2Q9", "D3Q19", "D3Q27"])
    nx, nz = int(rng.integers(3, 9)), int(rng.integers(3, 9))
    ny = 1 if model == "D2Q9" else int(rng.integers(3, 8))
    axes = [("east", "west"), ("north", "south"), ("up", "down")]
    face_type, face_vel = {}, {}
    for a, (f0, f1) in enumerate(axes):
        kind = rng.choice(["periodic", "noslip", "open", "mixed"])
        if model == "D2Q9" and a == 1:
            kind = "open"
        if kind == "periodic":
            face_type[f0] = face_type[f1] = "periodic"
        elif kind == "noslip":
            face_type[f0] = face_type[f1] = "noslip"
            face_vel[f0] = tuple(float(v) for v in rng.normal(0, 0.02, 3))
            face_vel[f1] = (0.0, 0.0, 0.0)
        elif kind == "mixed":
            face_type[f0] = "noslip"
            face_vel[f0] = tuple(float(v) for v in rng.normal(0, 0.02, 3))
    return dict(model=model, nx=nx, ny=ny, nz=nz, nu=float(rng.uniform(0.02, 0.4)), rho0=1.0,
                u0=tuple(float(v) for v in rng.normal(0, 0.01, 3)), force=tuple(float(v) for v in rng.normal(0, 1e-4, 3)),
                rho_solid=float(rng.uniform(0.9, 1.1)), face_type=face_type, face_vel=face_vel)


@needs_ref
@pytest.mark.parametrize("seed", range(12))
@pytest.mark.parametrize("variant,arith", [("avx2", po.ARITH_AVX2), ("scalar", po.ARITH_SCALAR)])
def test_port_matches_live_reference(seed, variant, arith):
    cfg = random_config(np.random.default_rng(seed))
    r = po.RefSim(**cfg, variant=variant)
    p = port_of(cfg, arith=arith)
    r.initialize()
    p.initialize()
    r.step(15)
    p.step(15)
    for w in (po.N, po.NTMP, po.RHO, po.U):
        assert_bitexact(p.get(w), r.get(w), f"{cfg['model']} field {w}")


def test_half_rounding_matches_ieee_binary16():
    """orc_round_half is binary16 round-to-nearest-even (numpy's float16 is
    the independent check); orc_store_half keeps d * 2^12 in it."""
    lib = po.port_lib()
    rng = np.random.default_rng(4)
    mags = 10.0 ** rng.uniform(-12, 4.9, 4000)
    vals = (mags * rng.choice([-1.0, 1.0], mags.size)).astype(np.float32)
    edge = np.array([0.0, -0.0, 6.1035156e-05, 5.9604645e-08, 2.9802322e-08, 65504.0, 65520.0, 1e9,
                     1.0 + 2.0 ** -11, 1.0 + 3 * 2.0 ** -11], np.float32)
    for v in np.concatenate([vals, edge]):
        with np.errstate(over="ignore"):
            want = np.float32(np.float16(v))
        got = np.float32(lib.orc_round_half(float(v)))
        assert got.tobytes() == want.tobytes() or (np.isinf(got) and np.isinf(want)), (v, got, want)
        with np.errstate(over="ignore"):
            want_s = np.float32(np.float32(np.float16(np.float32(v) * np.float32(4096.0))) / np.float32(4096.0))
        got_s = np.float32(lib.orc_store_half(float(v)))
        assert got_s.tobytes() == want_s.tobytes() or (np.isinf(got_s) and np.isinf(want_s)), (v, got_s, want_s)
    # the scale keeps 11 bits where binary16 alone has subnormals
    d = np.float32(3.0e-6)
    assert abs(lib.orc_store_half(float(d)) - d) <= d * 2.0 ** -11
    assert abs(np.float32(np.float16(d)) - d) > d * 2.0 ** -9
