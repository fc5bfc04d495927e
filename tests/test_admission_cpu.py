"""The solve server's admission policy (plbpd_gb300/csrc/admission.h) as a
host-only unit: smallest work first, the age bound, FIFO order, the
device-memory budget and the running-cells cap.  Compiled with g++; no GPU."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

SRC = os.path.join(ROOT, "tests", "cpp", "test_admission.cpp")


@pytest.mark.skipif(shutil.which("g++") is None, reason="g++ not available")
def test_admission_policy(tmp_path):
    exe = os.path.join(str(tmp_path), "test_admission")
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Werror", "-I", os.path.join(ROOT, "plbpd_gb300", "csrc"), SRC,
           "-o", exe]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip() == "ok"
