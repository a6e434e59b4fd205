"""Turbulence statistics of the 384 x 192 x 128 WALE channel (Re_tau = 180,
laminar parabola + 10 % noise start): the FP64 run whose profiles the FP16
and FP32 runs are held to (tests/test_gpu_channel_stats.py).

The reference averages output_profile's per-plane statistics over time
offline (RR27V33_code_DNS_LES/output.cu:142-225, profile.f90:24-86); here the
solver's FP64 accumulators (rr_accumulate) add the same per-plane profile
every EVERY steps over the second half of the run.  The run needs a GPU and
the built library:

    python tests/golden/make_channel_stats.py [storage] [out.npz]

(storage f64 by default; the committed fixture channel_stats_f64.npz is the
FP64 run).
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "recursively-regularized-lbm_gb300"))

STEPS = 200_000     # the run
AVG_FROM = 100_000  # averaging window: steps (AVG_FROM, STEPS]
EVERY = 1_000       # one profile sample every EVERY steps


def run(storage, steps=STEPS, avg_from=AVG_FROM, every=EVERY, log=None):
    """the channel in `storage`; returns the time-averaged per-plane profile
    (ly x 11: y + 0.5, (y + 0.5) / y*, <u>, <v>, <w>, <u'u'>, <v'v'>, <w'w'>,
    <u'v'>, <u'w'>, <v'w'>), <tau_t> (ly), the sample count and u*"""
    import rrlbm
    from rrlbm import presets

    p, st = presets.channel(storage=storage, les=True, variant="config")
    with rrlbm.Solver(p) as s:
        s.init_state(st["rho"], st["ux"], st["uy"], st["uz"])
        t0 = time.perf_counter()
        s.step(avg_from)
        s.sync()
        if log:
            log(f"{storage}: {avg_from} steps in {time.perf_counter() - t0:.1f} s")
        for k in range((steps - avg_from) // every):
            s.step(every)
            s.accumulate()
        prof, taut, n = s.get_accum()
        if log:
            log(f"{storage}: {steps} steps, {n} samples in {time.perf_counter() - t0:.1f} s")
    return prof / n, taut / n, n, p.ustar


def main():
    storage = sys.argv[1] if len(sys.argv) > 1 else "f64"
    out = sys.argv[2] if len(sys.argv) > 2 else os.path.join(HERE, f"channel_stats_{storage}.npz")
    prof, taut, n, ustar = run(storage, log=print)
    np.savez(out, profile=prof, taut=taut, samples=n, ustar=ustar, steps=STEPS, avg_from=AVG_FROM, every=EVERY,
             storage=storage)
    print("wrote", out)


if __name__ == "__main__":
    main()
