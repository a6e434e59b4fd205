"""The solver's per-node arithmetic (csrc/rr_node.cuh) compiled for the host
and checked against the oracle's restatement of the reference collision,
moments and wall closure (tests/node_check.cu).  No GPU needed."""
import os
import subprocess

import pytest

from conftest import ROOT


def test_node_arithmetic_matches_oracle(tmp_path):
    exe = str(tmp_path / "node_check")
    oracle = os.path.join(ROOT, "oracle")
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-x", "c++",
           "-I", os.path.join(ROOT, "recursively-regularized-lbm_gb300", "csrc"), "-I", oracle,
           os.path.join(ROOT, "tests", "node_check.cu"), "-L", oracle, "-loracle",
           f"-Wl,-rpath={oracle}", "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        pytest.fail("compile failed:\n" + r.stderr[-3000:])
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout
