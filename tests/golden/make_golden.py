"""Generates the golden fixtures in tests/golden/ from the reference itself.

Run here, where the reference sources were compiled into oracle/_ref
(``make -C oracle ref``):

    python tests/golden/make_golden.py

Outputs
  * ``ref_<case>.npz``  states of the reference's own PLBPD / LBDynamics /
    Boundary / CalcMoments (AVX2 collision kernel, -ffp-contract=off) on small
    domains: after initialize, after 1, 2, 5 and 20 time steps, and through one
    time step operator by operator.
  * ``golden.json``  the known answers of the reference's unit tests
    (src/utest/TestEqlbDist.cpp:22-26, TestField.cpp:106-107, TestLBModel.cpp)
    as recomputed by the reference, plus SHA-256 digests of the reference's
    final state on the 128x64 D2Q9 channel after 10,000 steps and on the four
    Flow presets (src/Flow.cpp:20-106) after their full step counts.
  * ``ref_sourcemap_<case>.npz``  the integer-encoded source map: n holds
    idx+1 and ntmp -(idx+1), wall velocities are zero, and one push, no-slip
    and periodic copy run; each output slot shows which slot it came from.
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import pyoracle as po  # noqa: E402

from cases import CASES, CHANNEL, PRESETS, SOURCEMAP_CASES  # noqa: E402


def fields(sim):
    return {"n": sim.get(po.N), "ntmp": sim.get(po.NTMP), "rho": sim.get(po.RHO), "u": sim.get(po.U)}


def run_case(name, cfg):
    sim = po.RefSim(**cfg, variant="avx2")
    sim.initialize()
    out = {}
    for k, v in fields(sim).items():
        out[f"init_{k}"] = v
    done = 0
    for target in (1, 2, 5, 20):
        sim.step(target - done)
        done = target
        for k, v in fields(sim).items():
            out[f"step{target}_{k}"] = v
    # one more time step, operator by operator
    sim.collide()
    out["op_collide_n"] = sim.get(po.N)
    sim.stream()
    out["op_stream_n"] = sim.get(po.N)
    out["op_stream_ntmp"] = sim.get(po.NTMP)
    sim.noslip()
    out["op_noslip_n"] = sim.get(po.N)
    sim.periodic()
    out["op_periodic_n"] = sim.get(po.N)
    sim.moments()
    out["op_moments_rho"] = sim.get(po.RHO)
    out["op_moments_u"] = sim.get(po.U)
    sim.reset()
    out["op_reset_rho"] = sim.get(po.RHO)
    out["op_reset_u"] = sim.get(po.U)
    np.savez_compressed(os.path.join(HERE, f"ref_{name}.npz"), **out)


def run_sourcemap(name, cfg):
    sim = po.RefSim(**cfg, variant="avx2")
    sim.initialize()
    shape = sim.shape(po.N)
    idx = np.arange(1, np.prod(shape) + 1, dtype=np.float64)
    assert idx[-1] < 2 ** 24
    sim.set(po.N, idx.astype(np.float32).reshape(shape))
    sim.set(po.NTMP, (-idx).astype(np.float32).reshape(shape))
    sim.stream()
    sim.noslip()
    sim.periodic()
    np.savez_compressed(os.path.join(HERE, f"ref_sourcemap_{name}.npz"), n=sim.get(po.N), ntmp=sim.get(po.NTMP))


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.float32).tobytes()).hexdigest()


def main():
    if not po.ref_available("avx2"):
        raise SystemExit("oracle/_ref/libplbpd_ref_avx2.so is missing: run `make -C oracle ref` first")
    for name, cfg in CASES.items():
        run_case(name, cfg)
    for name, cfg in SOURCEMAP_CASES.items():
        run_sourcemap(name, cfg)
    g = {}
    lib = po.ref_lib("avx2")
    import ctypes as C
    # reference unit-test known answers, recomputed by the reference
    out = (C.c_float * 9)()
    lib.refh_eqlb(b"D2Q9", 1.0, (C.c_float * 3)(0.5, 0.5, -0.5), out)
    g["eqlb_d2q9_rho1_u_05_05_m05"] = [float(v) for v in out]
    for model in ("D2Q9", "D3Q19", "D3Q27"):
        q = po.Q_OF[model]
        c = (C.c_int * (3 * q))()
        w = (C.c_float * q)()
        rev = (C.c_uint * q)()
        cs2 = C.c_float()
        lib.refh_model_tables(model.encode(), c, w, rev, C.byref(cs2))
        g[f"tables_{model}"] = {"c": [int(v) for v in c], "w_bits": [int(np.float32(v).view(np.uint32)) for v in w],
                                "rev": [int(v) for v in rev], "cs2_bits": int(np.float32(cs2.value).view(np.uint32))}
    # the 128x64 channel, 10,000 steps, by the reference's own march
    sim = po.RefSim(**CHANNEL, variant="avx2")
    sim.initialize()
    sim.step(10000)
    g["channel_10000"] = {k: digest(v) for k, v in fields(sim).items()}
    g["channel_10000"]["u_max"] = float(sim.get(po.U)[1:-1, 1, 1:-1, 0].max())
    # plbpd's Flow presets, full step counts, by the reference's own march
    for name, (cfg, steps) in PRESETS.items():
        sim = po.RefSim(**cfg, variant="avx2")
        sim.initialize()
        sim.step(steps)
        g[f"preset_{name}"] = {k: digest(v) for k, v in fields(sim).items()}
        g[f"preset_{name}"]["steps"] = steps
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(g, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
