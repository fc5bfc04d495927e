"""plbpd's C++ classes (include/plbpd/*.hpp over libplb_gb300.so): a C++
program written against the reference's interface -- the unit-test cases of
src/utest and the flow of src/main.cpp -- compared with the reference."""
import hashlib
import json
import os
import subprocess

import numpy as np
import pytest

from cases import CASES, PRESETS
from conftest import ROOT, assert_bitexact, load_npz

SRC = os.path.join(ROOT, "tests", "cpp", "test_facade.cpp")
BUILD = os.path.join(ROOT, "tests", "cpp", "_build")
EXE = os.path.join(BUILD, "test_facade")
LIBDIR = os.path.join(ROOT, "plbpd_gb300", "_lib")

# TestEqlbDist.cpp:22-26
EQLB_TESTFILE = [-0.05555555597, 0.277777791, -0.05555555597, -0.05555555597, 0.277777791,
                 -0.003472222248, -0.003472222248, 0.2048611194, 0.03819444403]
FACES = ("east", "west", "north", "south", "up", "down")


@pytest.fixture(scope="module")
def exe():
    from plbpd_gb300 import build
    build.build()
    os.makedirs(BUILD, exist_ok=True)
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-I", os.path.join(ROOT, "include", "plbpd"), SRC,
           "-L", LIBDIR, "-lplb_gb300", f"-Wl,-rpath,{LIBDIR}", "-o", EXE]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return EXE


def test_facade_host_side(exe, golden):
    """LBModel, EqlbDist, Field, Domain and the exception types, no GPU."""
    r = subprocess.run([exe, "cpu"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = json.loads(r.stdout)
    for model in ("D2Q9", "D3Q19", "D3Q27"):
        g = golden[f"tables_{model}"]
        assert out[model]["c"] == g["c"]
        assert np.array(out[model]["w"], np.float32).view(np.uint32).tolist() == g["w_bits"]
        assert out[model]["rev"] == g["rev"]
        assert np.float32(out[model]["cs2"]).view(np.uint32) == g["cs2_bits"]
    assert np.array_equal(np.array(out["eqlb"], np.float32), np.array(EQLB_TESTFILE, np.float32))


def case_args(cfg):
    a = [cfg["model"], cfg["nx"], cfg["ny"], cfg["nz"], cfg["nu"], cfg["rho0"], *cfg["u0"], *cfg["force"],
         cfg["rho_solid"]]
    for f in FACES:
        t = {"periodic": 1, "noslip": 2}.get(cfg["face_type"].get(f), 0)
        hv = 1 if f in cfg["face_vel"] else 0
        a += [t, hv, *cfg["face_vel"].get(f, (0.0, 0.0, 0.0))]
    return [repr(float(v)) if isinstance(v, float) else str(v) for v in a]


def read_f32(path, shape):
    return np.fromfile(path, dtype=np.float32).reshape(shape)


@pytest.mark.gpu
@pytest.mark.parametrize("case", sorted(CASES))
def test_facade_matches_reference(exe, tmp_path, case):
    cfg = CASES[case]
    ref = load_npz(f"ref_{case}.npz")
    r = subprocess.run([exe, "case", str(tmp_path)] + case_args(cfg), capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    for key in ("init", "step1", "step2", "step5", "step20"):
        for fld in ("n", "ntmp", "rho", "u"):
            want = ref[f"{key}_{fld}"]
            assert_bitexact(read_f32(tmp_path / f"{key}_{fld}.f32", want.shape), want, f"{case} {key} {fld}")
    for key in ("op_collide_n", "op_stream_n", "op_stream_ntmp", "op_noslip_n", "op_periodic_n",
                "op_moments_rho", "op_moments_u", "op_reset_rho", "op_reset_u"):
        want = ref[key]
        assert_bitexact(read_f32(tmp_path / f"{key}.f32", want.shape), want, f"{case} {key}")


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["d2q9_channel", "d3q19_xy_periodic", "d3q27_duct"])
def test_facade_collision_trt_matches_oracle(exe, tmp_path, case):
    """CollisionTRT through the Collision base in a hand-written plbpd loop
    equals the oracle's REFERENCE-mode run with the TRT operator."""
    import pyoracle as po
    cfg = CASES[case]
    r = subprocess.run([exe, "case", str(tmp_path)] + case_args(cfg), capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    p = po.Port(**cfg, arith=po.ARITH_FP32, trt=0.0)
    p.initialize()
    p.step(6)
    for fld, w in (("n", po.N), ("rho", po.RHO), ("u", po.U)):
        want = p.get(w)
        assert_bitexact(read_f32(tmp_path / f"trt6_{fld}.f32", want.shape), want, f"{case} TRT {fld}")


@pytest.mark.gpu
@pytest.mark.parametrize("preset", sorted(PRESETS))
def test_facade_flow_presets_match_reference(exe, tmp_path, golden, preset):
    """src/main.cpp's flow -- Flow, PLBPD, SimData, initialize, march_in_time
    -- on each preset at its full step count: every byte equals the reference's."""
    r = subprocess.run([exe, "preset", preset, str(tmp_path)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    for fld in ("n", "ntmp", "rho", "u"):
        d = hashlib.sha256((tmp_path / f"final_{fld}.f32").read_bytes()).hexdigest()
        assert d == golden[f"preset_{preset}"][fld], f"{preset} {fld} differs from the reference"
