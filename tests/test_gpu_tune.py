"""The fused-step autotuner: every compiled variant of the fused step (the
FP16 pair kernel's forms; for FP32 and FP32_DEV storage, either arithmetic,
the single-node and the pair kernel) gives the oracle's bits, and a tuned
solve runs one of them and records it."""
import numpy as np
import pytest

import pyoracle as po
from test_gpu_native import NATIVE_CASES, compare, mask_for, perturbed_start

pytestmark = pytest.mark.gpu

# even nx (the pair kernel); duct_d3q27 has moving walls (one variant)
PAIR_CASES = ["torus_d3q19", "obstacles_d3q19", "channel_d2q9", "obstacles_torus_d3q27", "duct_d3q27"]


STORAGE = {"fp16": ("STORAGE_FP16_DEV", "ARITH_FP32", po.ARITH_FP16DEV),
           "fp32": ("STORAGE_FP32", "ARITH_FP32", po.ARITH_FP32),
           "fp32dev": ("STORAGE_FP32_DEV", "ARITH_FP32", po.ARITH_FP32DEV),
           "reference": ("STORAGE_FP32", "ARITH_REFERENCE", po.ARITH_AVX2)}


def oracle_after(case, steps, storage="fp16"):
    cfg = NATIVE_CASES[case]
    mask = mask_for(case, cfg)
    p = po.Port(**cfg, mode=po.MODE_NATIVE, mask=mask, arith=STORAGE[storage][2])
    p._cfg = cfg
    p.initialize()
    start = perturbed_start(p, 11)
    p.set(po.N, start[0]); p.set(po.RHO, start[1]); p.set(po.U, start[2])
    p.step(steps)
    return cfg, mask, start, p


def gpu_solve(capi, cfg, mask, start, steps, storage="fp16"):
    st, ar, _ = STORAGE[storage]
    s = capi.Solve.create(**cfg, semantics=capi.SEMANTICS_NATIVE, storage=getattr(capi, st), arith=getattr(capi, ar))
    if mask is not None:
        s.set_mask(mask)
    s.initialize()
    s.set(0, start[0]); s.set(2, start[1]); s.set(3, start[2])
    s.step(steps)
    return s


@pytest.mark.parametrize("storage", sorted(STORAGE))
@pytest.mark.parametrize("case", PAIR_CASES)
def test_every_variant_matches_oracle(case, storage):
    """FP16: the pair kernel's seven compiled forms; FP32 and FP32_DEV: the
    single-node kernel and the pair kernel's three forms; FP32 storage with
    plbpd's arithmetic: the single-node kernel and the pair kernel's form 2."""
    from plbpd_gb300 import capi
    cfg, mask, start, p = oracle_after(case, 20, storage)
    try:
        for v in range(capi.tune_variants()):
            capi.tune_force(v)
            with gpu_solve(capi, cfg, mask, start, 20, storage) as s:
                assert s.variant() in (v, 0)
                compare(s, p, mask, f"{case} {storage} variant {v}")
    finally:
        capi.tune_force(-1)


def test_tuned_solve_records_its_choice(tmp_path, monkeypatch):
    from plbpd_gb300 import capi
    cache = tmp_path / "tune.txt"
    monkeypatch.setenv("PLB_TUNE_CACHE", str(cache))
    monkeypatch.delenv("PLB_TUNE", raising=False)
    # a size class no other test uses, so this solve tunes rather than reuses
    cfg = dict(NATIVE_CASES["torus_d3q19"], nx=48, ny=40, nz=36)
    p = po.Port(**cfg, mode=po.MODE_NATIVE, arith=po.ARITH_FP16DEV)
    p._cfg = cfg
    p.initialize()
    start = perturbed_start(p, 5)
    p.set(po.N, start[0]); p.set(po.RHO, start[1]); p.set(po.U, start[2])
    p.step(130)
    with gpu_solve(capi, cfg, None, start, 130) as s:   # a graph chunk and single steps
        v = s.variant()
        assert 0 <= v < capi.tune_variants()
        compare(s, p, None, "tuned")
    lines = [l.split() for l in cache.read_text().splitlines()]
    assert lines and lines[-1][0] == "plb-tune-v2" and int(lines[-1][-1]) == v
    # the same class again takes the recorded choice
    with gpu_solve(capi, cfg, None, start, 2) as s2:
        assert s2.variant() == v


def _ref_solve(capi, cfg, mask, start):
    s = capi.Solve.create(**cfg, semantics=capi.SEMANTICS_NATIVE, storage=capi.STORAGE_FP32,
                          arith=capi.ARITH_REFERENCE)
    s.set_mask(mask)
    s.initialize()
    s.set(0, start[0]); s.set(2, start[1]); s.set(3, start[2])
    return s


def _ref_oracle(cfg, mask, seed):
    p = po.Port(**cfg, mode=po.MODE_NATIVE, mask=mask, arith=po.ARITH_AVX2)
    p._cfg = cfg
    p.initialize()
    start = perturbed_start(p, seed)
    p.set(po.N, start[0]); p.set(po.RHO, start[1]); p.set(po.U, start[2])
    return p, start


def _cache_lines(path):
    return [l.split() for l in path.read_text().splitlines()] if path.exists() else []


def test_choice_by_trials_is_timed_again(tmp_path, monkeypatch):
    """A choice made by trials is timed once more after 256 fused steps (a
    second table line for the same key); the march stays bit-exact across
    the switch of kernels and graphs."""
    from plbpd_gb300 import capi
    cache = tmp_path / "tune.txt"
    monkeypatch.setenv("PLB_TUNE_CACHE", str(cache))
    monkeypatch.delenv("PLB_TUNE", raising=False)
    # masked D3Q19 with plbpd's arithmetic, a size class no other test uses
    cfg = dict(NATIVE_CASES["obstacles_d3q19"], nx=64, ny=48, nz=44)
    mask = mask_for("obstacles_d3q19", cfg)
    p, start = _ref_oracle(cfg, mask, 7)
    p.step(300)
    with _ref_solve(capi, cfg, mask, start) as s:
        s.step(300)   # the raw collision, four graph chunks, the second trial, 43 single steps
        compare(s, p, mask, "re-tuned")
        v = s.variant()
    lines = _cache_lines(cache)
    assert len(lines) == 2 and lines[0][:-1] == lines[1][:-1]
    assert int(lines[-1][-1]) == v


def test_explicit_tune_replaces_the_second_trial(tmp_path, monkeypatch):
    from plbpd_gb300 import capi
    cache = tmp_path / "tune.txt"
    monkeypatch.setenv("PLB_TUNE_CACHE", str(cache))
    monkeypatch.delenv("PLB_TUNE", raising=False)
    cfg = dict(NATIVE_CASES["obstacles_d3q19"], nx=40, ny=32, nz=28)
    mask = mask_for("obstacles_d3q19", cfg)
    p, start = _ref_oracle(cfg, mask, 9)
    p.step(303)
    with _ref_solve(capi, cfg, mask, start) as s:
        s.step(3)                       # the first fused steps choose by trials
        assert len(_cache_lines(cache)) == 1
        v = s.tune()
        assert 0 <= v < capi.tune_variants()
        s.step(300)                     # no further trial
        assert s.variant() == v
        compare(s, p, mask, "tuned explicitly")
    lines = _cache_lines(cache)
    assert len(lines) == 2 and int(lines[-1][-1]) == v
