"""The continuous-batching server on the GPU: every served solve must equal
the same solve run alone, bit for bit (stated tolerance: zero), also when the
HBM budget forces domains to wait and to join a running batch."""
import numpy as np
import pytest

from rrlbm import serve, workloads

pytestmark = pytest.mark.gpu


def _small_stream():
    reqs = workloads.request_stream(7, rate=400.0, seed=12, sizes=(10, 22), steps=(20, 150))
    kinds = [d.kind for d in reqs]
    assert len(set(kinds)) == 3, kinds
    return reqs


@pytest.mark.parametrize("budget_domains", [None, 2])
def test_served_equals_alone(budget_domains):
    reqs = _small_stream()
    be = serve.GpuBackend()
    budget = 10 ** 12 if budget_domains is None else budget_domains * max(be.bytes_for(d) for d in reqs)
    srv = serve.Server(be, budget, max_chunk=40, on_result=lambda s: s.get_f())
    recs = srv.run(reqs)
    be.close()
    assert srv.peak_bytes <= budget
    if budget_domains is not None:
        assert any(r.queued > 0 for r in recs)
    for d, r in zip(reqs, recs):
        assert not r.error, r.error
        s = workloads.solve_alone(d)
        alone = s.get_f()
        s.close()
        assert np.array_equal(r.result, alone), (d, np.abs(r.result - alone).max())
    st = serve.summarize(recs)
    assert st["completed"] == len(reqs)


def test_served_error_vs_fp64_rerun():
    # the FP16 / FP32 solve against its FP64 rerun, velocity error relative to its scale
    for kind in ("tg", "cavity", "channel"):
        d = workloads.Domain(kind, 24, 300, "f16", tau=0.6, Ma=0.05, Re=300, seed=3)
        lo, hi = workloads.solve_alone(d), workloads.solve_alone(d, "f64")
        a, b = lo.macro(), hi.macro()
        lo.close()
        hi.close()
        err = max(np.abs(a[k] - b[k]).max() for k in ("ux", "uy", "uz")) / workloads.velocity_scale(d)
        assert err < 2e-2, (kind, err)
