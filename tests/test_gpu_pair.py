"""The packed FP32-pair node arithmetic against the scalar FP32 arithmetic on
the GPU, bit for bit (tests/pair_check.cu, built here with the library's
nvcc flags): the tile and staged steps compute interior node pairs in the
packed form and the wall nodes one at a time, and every result of the
library assumes the two give the same bits."""
import os
import subprocess
import sys

import pytest

from conftest import PKG, ROOT

pytestmark = pytest.mark.gpu


def test_pair_arithmetic_equals_scalar(tmp_path):
    sys.path.insert(0, PKG)
    from rrlbm import build as b

    exe = str(tmp_path / "pair_check")
    cmd = [b.NVCC] + b.ARCH + b.FLAGS + ["-I", b.CSRC, os.path.join(ROOT, "tests", "pair_check.cu"), "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
