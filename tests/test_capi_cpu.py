"""The C ABI on a machine without a GPU: the library loads, exports every entry
point include/plb.h declares, and its host-only entry points (lattice tables,
equilibrium, relaxation) agree with the oracle and the reference's known
answers.  Nothing here launches a kernel."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import pyoracle as po
from conftest import ROOT, assert_bitexact

HEADER = os.path.join(ROOT, "include", "plb.h")
EQLB_TESTFILE = [-0.05555555597, 0.277777791, -0.05555555597, -0.05555555597, 0.277777791,
                 -0.003472222248, -0.003472222248, 0.2048611194, 0.03819444403]


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(plb_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from plbpd_gb300 import build, capi
    build.build()
    return capi.lib()


def test_every_declared_symbol_is_exported(lib):
    names = declared_symbols()
    assert len(names) >= 30
    raw = C.CDLL(os.path.join(ROOT, "plbpd_gb300", "_lib", "libplb_gb300.so"))
    missing = [n for n in names if not hasattr(raw, n)]
    assert not missing, missing


def test_binding_covers_every_declared_symbol(lib):
    from plbpd_gb300 import capi
    bound = {name for name, _, _ in capi._SIGS}
    assert set(declared_symbols()) <= bound


@pytest.mark.parametrize("model", ["D2Q9", "D3Q19", "D3Q27"])
def test_tables_match_oracle(lib, model):
    from plbpd_gb300 import capi
    c, w, rev, cs2 = capi.model_tables(model)
    c2, w2, rev2, cs22 = po.model_tables(model)
    assert np.array_equal(c, c2) and np.array_equal(rev, rev2)
    assert_bitexact(w, w2, "weights")
    assert cs2 == cs22


def test_unknown_model(lib):
    from plbpd_gb300 import capi
    with pytest.raises(capi.PlbError) as e:
        capi.model_tables("D2Q5")
    assert e.value.code == capi.EINVAL
    assert "not yet implemented" in str(e.value)


def test_equilibrium_known_answer(lib):
    from plbpd_gb300 import capi
    got = capi.equilibrium(9, 1.0, (0.5, 0.5, -0.5))
    assert_bitexact(got, np.array(EQLB_TESTFILE, np.float32), "TestEqlbDist")
    rng = np.random.default_rng(1)
    for q, model in ((9, "D2Q9"), (19, "D3Q19"), (27, "D3Q27")):
        for _ in range(20):
            rho = float(np.float32(rng.uniform(0.8, 1.2)))
            u = rng.normal(0, 0.05, 3).astype(np.float32)
            assert_bitexact(capi.equilibrium(q, rho, u), po.eqlb(model, rho, u), f"{model} eqlb")


@pytest.mark.parametrize("nu", [0.1, 0.5, 0.0333333, 0.01666667, 0.25, 1e-3])
def test_relaxation_matches_reference_rule(lib, nu):
    from plbpd_gb300 import capi
    tau, omega = capi.relaxation(nu)
    t = np.float32(np.float32(3.0) * np.float32(nu)) + np.float32(0.5)
    assert np.float32(tau) == t
    assert np.float32(omega) == np.float32(1.0 / np.float64(t))


def test_invalid_parameters_rejected_before_any_device_work(lib):
    from plbpd_gb300 import capi
    bad = [dict(model="D3Q19", nx=0, ny=4, nz=4, nu=0.1),
           dict(model="D3Q19", nx=4, ny=4, nz=4, nu=0.1, semantics=capi.SEMANTICS_NATIVE,
                face_type={"east": "periodic", "west": "noslip"}),
           dict(model="D3Q19", nx=4, ny=4, nz=4, nu=0.1, storage=capi.STORAGE_FP16_DEV),
           # non-finite parameters and tau <= 0 never reach a kernel
           dict(model="D3Q19", nx=4, ny=4, nz=4, nu=float("nan")),
           dict(model="D3Q19", nx=4, ny=4, nz=4, nu=0.1, force=(float("inf"), 0.0, 0.0)),
           dict(model="D2Q9", nx=4, ny=1, nz=4, nu=0.1, rho0=float("nan")),
           dict(model="D3Q19", nx=4, ny=4, nz=4, nu=-0.2)]
    for kw in bad:
        with pytest.raises(capi.PlbError) as e:
            capi.Solve.create(**kw)
        assert e.value.code in (capi.EINVAL, capi.EUNSUPPORTED)


def test_tune_force_range(lib):
    from plbpd_gb300 import capi
    n = capi.tune_variants()
    assert n >= 1
    for bad in (-2, n, 1000):
        with pytest.raises(capi.PlbError) as e:
            capi.tune_force(bad)
        assert e.value.code == capi.EINVAL
    capi.tune_force(0)
    capi.tune_force(-1)


def test_solve_bytes_follow_storage_and_streaming(lib):
    """plb_solve_bytes (the server's admission measure, host arithmetic only):
    FP16 populations take half FP32's bytes, AA streaming one buffer instead
    of two, FP64 twice FP32's."""
    from plbpd_gb300 import capi

    def nbytes(**kw):
        p = capi.make_params("D3Q19", 64, 64, 64, 0.1, semantics=capi.SEMANTICS_NATIVE, arith=capi.ARITH_FP32,
                             face_type={f: "periodic" for f in capi.FACES}, **kw)
        return lib.plb_solve_bytes(capi.C.byref(p))

    pop = 64 ** 3 * 19
    fp32, fp16, fp64 = (nbytes(storage=capi.STORAGE_FP32), nbytes(storage=capi.STORAGE_FP16_DEV),
                        nbytes(storage=capi.STORAGE_FP64))
    aa = nbytes(storage=capi.STORAGE_FP32, streaming=capi.STREAMING_AA)
    assert fp32 - fp16 == 2 * pop * 2          # two buffers, 2 bytes a population less
    assert fp64 - fp32 == 2 * pop * 4
    assert fp32 - aa == pop * 4                # one buffer fewer
    assert min(fp32, fp16, fp64, aa) > 0
