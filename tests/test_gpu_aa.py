"""AA in-place streaming (one population buffer) against the oracle and
against the two-buffer kernels, bit for bit: every storage, both collision
operators, odd and even step counts (the buffer's two layouts), graph chunks,
reads and writes of the state between steps, and half the population
memory."""
import numpy as np
import pytest

import pyoracle as po
from conftest import assert_bitexact
from test_gpu_native import NATIVE_CASES, compare, mask_for, perturbed_start

pytestmark = pytest.mark.gpu

STORAGES = ["fp32", "fp16", "fp64", "fp32dev"]


def make(capi, case, storage, streaming, collision):
    cfg = NATIVE_CASES[case]
    st = {"fp32": capi.STORAGE_FP32, "fp16": capi.STORAGE_FP16_DEV, "fp64": capi.STORAGE_FP64,
          "fp32dev": capi.STORAGE_FP32_DEV}[storage]
    s = capi.Solve.create(**cfg, semantics=capi.SEMANTICS_NATIVE, arith=capi.ARITH_FP32, storage=st,
                          streaming=streaming, collision=collision)
    m = mask_for(case, cfg)
    if m is not None:
        s.set_mask(m)
    s.initialize()
    return s


def same_state(a, b, what):
    for w, name in ((0, "n"), (2, "rho"), (3, "u")):
        assert_bitexact(a.get(w), b.get(w), f"{what} {name}")
    np.testing.assert_array_equal(a.conservation(), b.conservation())


@pytest.mark.parametrize("collision", ["bgk", "trt"])
@pytest.mark.parametrize("storage", STORAGES)
@pytest.mark.parametrize("case", sorted(NATIVE_CASES))
def test_aa_equals_ab(case, storage, collision):
    from plbpd_gb300 import capi
    col = capi.COLLISION_TRT if collision == "trt" else capi.COLLISION_BGK
    with make(capi, case, storage, capi.STREAMING_AB, col) as ab, make(capi, case, storage, capi.STREAMING_AA, col) as aa:
        done = 0
        for target in (1, 2, 7, 150):      # odd counts end in the swapped layout
            ab.step(target - done)
            aa.step(target - done)
            done = target
            same_state(aa, ab, f"{case} {storage} {collision} step {target}")


@pytest.mark.parametrize("storage", ["fp32", "fp16"])
def test_aa_state_edits_between_steps(storage):
    """Writing rho and n while the buffer is in either layout."""
    from plbpd_gb300 import capi
    case = "obstacles_d3q19"
    with make(capi, case, storage, capi.STREAMING_AB, 0) as ab, make(capi, case, storage, capi.STREAMING_AA, 0) as aa:
        for steps in (3, 4):                  # swapped, then natural
            ab.step(steps)
            aa.step(steps)
            rho = ab.get(capi.FIELD_RHO)
            rho[1:-1, 1:-1, 1:-1] *= np.float32(1.0001)
            ab.set(capi.FIELD_RHO, rho)
            aa.set(capi.FIELD_RHO, rho)
            ab.step(5)
            aa.step(5)
            same_state(aa, ab, f"after rho edit ({steps} steps)")
        n = ab.get(capi.FIELD_N)
        ab.set(capi.FIELD_N, n)
        aa.set(capi.FIELD_N, n)
        ab.step(9)
        aa.step(9)
        same_state(aa, ab, "after n edit")


def test_aa_halves_population_memory():
    from plbpd_gb300 import capi
    with make(capi, "torus_d3q19", "fp32", capi.STREAMING_AB, 0) as ab, \
            make(capi, "torus_d3q19", "fp32", capi.STREAMING_AA, 0) as aa:
        cfg = NATIVE_CASES["torus_d3q19"]
        pop = ab.device_bytes() - aa.device_bytes()
        assert pop >= 19 * cfg["nx"] * cfg["ny"] * cfg["nz"] * 4
        p_ab = capi.make_params(**cfg, semantics=capi.SEMANTICS_NATIVE, arith=capi.ARITH_FP32)
        p_aa = capi.make_params(**cfg, semantics=capi.SEMANTICS_NATIVE, arith=capi.ARITH_FP32,
                                streaming=capi.STREAMING_AA)
        assert capi.lib().plb_solve_bytes(capi.C.byref(p_ab)) - capi.lib().plb_solve_bytes(capi.C.byref(p_aa)) == pop


def test_aa_refused_where_undefined():
    from plbpd_gb300 import capi
    from cases import CASES
    with pytest.raises(capi.PlbError):      # plbpd's own sequence pushes between two buffers
        capi.Solve.create(**CASES["d2q9_channel"], streaming=capi.STREAMING_AA)
    with make(capi, "torus_d3q19", "fp32", capi.STREAMING_AA, 0) as aa, pytest.raises(capi.PlbError):
        capi.Batch([aa])


ORACLE_MODE = {"fp32": dict(arith=po.ARITH_FP32), "fp16": dict(arith=po.ARITH_FP16DEV), "fp64": dict(precision=1),
               "fp32dev": dict(arith=po.ARITH_FP32DEV)}


@pytest.mark.parametrize("collision", ["bgk", "trt"])
@pytest.mark.parametrize("storage", STORAGES)
@pytest.mark.parametrize("case", sorted(NATIVE_CASES))
def test_aa_matches_oracle(case, storage, collision):
    """AA against the oracle's restatement directly (the oracle has no AA:
    its two-buffer pull step is the definition the in-place update must
    reproduce)."""
    from plbpd_gb300 import capi
    cfg = NATIVE_CASES[case]
    mask = mask_for(case, cfg)
    kw = dict(ORACLE_MODE[storage])
    if collision == "trt":
        kw["trt"] = 0.0
    p = po.Port(**cfg, mode=po.MODE_NATIVE, mask=mask, **kw)
    p._cfg = cfg
    p.initialize()
    # the same non-uniform float start on both sides (FP64 storage computes
    # its initial equilibrium with the exact weights, the oracle's with
    # plbpd's float ones)
    n, rho, u = perturbed_start(p, 17)
    p.set(po.N, n); p.set(po.RHO, rho); p.set(po.U, u)
    col = capi.COLLISION_TRT if collision == "trt" else capi.COLLISION_BGK
    with make(capi, case, storage, capi.STREAMING_AA, col) as aa:
        aa.set(0, n); aa.set(2, rho); aa.set(3, u)
        done = 0
        for target in (1, 2, 7, 150):      # odd counts end in the swapped layout
            p.step(target - done)
            aa.step(target - done)
            done = target
            compare(aa, p, mask, f"AA {case} {storage} {collision} step {target}")
