"""Configuration-size turbulence statistics: the 384 x 192 x 128 WALE channel
(Re_tau = 180, laminar parabola + 10 % noise start) for 200,000 steps with
the per-plane profile of output_profile (RR27V33_code_DNS_LES/output.cu:
142-225) accumulated in FP64 every 1,000 steps over the last 100,000
(profile.f90:24-86 averages the same profiles offline), in FP16 storage with
FP32 arithmetic, against the FP64 run of tests/golden/channel_stats_f64.npz
(made by tests/golden/make_channel_stats.py on a GB300).

Bars: the mean streamwise profile <u>(y) within 1 % of the FP64 run's
centreline value (the stated accuracy target); the rms profiles and <u'v'>
within 5 % of the FP64 run's largest value of that profile (statistics of a
finite window; the FP16 and FP64 runs do not share an instantaneous state)."""
import os
import sys

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

FIXTURE = os.path.join(GOLDEN, "channel_stats_f64.npz")


def _compare(prof, ref):
    """relative differences: <u>, rms u, v, w, <u'v'>"""
    u, u0 = prof[:, 2], ref[:, 2]
    out = {"u": float(np.abs(u - u0).max() / np.abs(u0).max())}
    for name, k in (("urms", 5), ("vrms", 6), ("wrms", 7)):
        a, b = np.sqrt(np.maximum(prof[:, k], 0)), np.sqrt(np.maximum(ref[:, k], 0))
        out[name] = float(np.abs(a - b).max() / max(b.max(), 1e-300))
    a, b = prof[:, 8], ref[:, 8]
    out["uv"] = float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))
    return out


@pytest.mark.skipif(not os.path.exists(FIXTURE), reason="FP64 statistics fixture not generated")
def test_channel_statistics_fp16_vs_fp64():
    sys.path.insert(0, GOLDEN)
    from make_channel_stats import run

    ref = np.load(FIXTURE)
    prof, taut, n, ustar = run("f16")
    assert n == int(ref["samples"])
    err = _compare(prof, ref["profile"])
    print("FP16 vs FP64 channel statistics:", err)
    assert err["u"] < 0.01, err
    for k in ("urms", "vrms", "wrms", "uv"):
        assert err[k] < 0.05, err
