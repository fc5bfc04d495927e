"""The FP32 evaluation of plbpd's double-precision collision tail
(plbpd_gb300/csrc/tail_exact.h, used by every kernel under REFERENCE
arithmetic) against that tail as the reference writes it
(src/CollisionSRT.cpp:144-147), bit for bit, on the host: lattice-like
nodes, random exponents (tiny, huge and subnormal operands), special values
and nodes at rest.  The same header compiles into the CUDA kernels, where the
GPU parity tests check the result end to end.  Compiled with g++; no GPU."""
import os
import re
import shutil
import subprocess

import pytest

from conftest import ROOT

SRC = os.path.join(ROOT, "tests", "cpp", "test_tail_exact.cpp")


@pytest.mark.skipif(shutil.which("g++") is None, reason="g++ not available")
@pytest.mark.parametrize("seed", [20261203, 7])
def test_tail_matches_double_sequence(tmp_path, seed):
    exe = os.path.join(str(tmp_path), "test_tail_exact")
    # -ffp-contract=off: every float operation rounds on its own, as on the GPU
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-Wall", "-Werror", SRC, "-o", exe]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    r = subprocess.run([exe, "8000000", str(seed)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    m = re.search(r"mismatches (\d+) fp64_mismatches (\d+) fp64_evals (\d+) near_boundary_decided (\d+)", r.stdout)
    assert m, r.stdout
    mismatches, fp64_mismatches, fp64_evals, near = map(int, m.groups())
    assert mismatches == 0 and fp64_mismatches == 0
    # the rounding test decided evaluations that lay close to a rounding
    # boundary (the cases a loose error bound would get wrong) ...
    assert near > 100
    # ... and the FP64 form stays rare: special values and random exponents
    # (a quarter of the samples) take it often, lattice-like nodes about once
    # in 10^4
    assert fp64_evals < 0.3 * 8000000
