"""The staged DNS step (rr_set_stage RR_DNS_STAGED: face rows in one launch,
interior rows through a shared-memory pipeline of bulk copies) against the
tile step: the same populations bit for bit (stated tolerance: zero), and
against the oracle in FP64.  On the 64-wide grids the tile step computes its
interior rows as packed FP32 node pairs and the staged step one node per
thread, so these cases also hold the two arithmetic forms to the same bits."""
import numpy as np
import pytest

import rrlbm
from rrlbm import presets
from helpers import load_state, oracle_for

pytestmark = pytest.mark.gpu


def _cases():
    return [
        presets.cavity(n=24, Re=300, storage="f16"),
        presets.cavity(n=24, Re=300, storage="bf16"),
        presets.cavity(n=24, Re=300, storage="f32"),
        presets.cavity(n=16, Re=100, storage="f64"),
        presets.taylor_green(L=32, nz=8, tau=0.6, Ma=0.05, storage="f16"),
        presets.taylor_green(L=20, nz=6, tau=0.55, Ma=0.05, q=19, storage="f32"),
        presets.channel(nx=48, ny=18, nz=10, Re_tau=36, les=False, storage="f16", variant="config", amp=0.2),
        presets.cavity(n=8, Re=50, storage="f16", variant="reference"),  # 8 x 8 x 2: no interior row
        # rows wide enough for the tile step's packed node pairs (the staged
        # step computes one node per thread): the two forms agree bit for bit
        presets.cavity(n=64, Re=400, storage="f16"),
        presets.cavity(n=64, Re=400, storage="f32"),
        presets.channel(nx=64, ny=18, nz=10, Re_tau=36, les=False, storage="bf16", variant="config", amp=0.2),
    ]


@pytest.mark.parametrize("k", range(11))
@pytest.mark.parametrize("rows,stages", [(None, None), (1, 2), (3, 4)])
def test_staged_equals_tile(k, rows, stages):
    p, st = _cases()[k]
    out = []
    for method in (0, 1):
        with rrlbm.Solver(p) as s:
            if method == 1:
                if p.lz < 3:
                    with pytest.raises(rrlbm.RRError):
                        s.set_stage(1)
                    return
                r = None if rows is None else min(rows, p.ly - 2)
                s.set_stage(1, r, stages)
                assert s.stage()[0] == 1
            s.init_state(st["rho"], st["ux"], st["uy"], st["uz"], f=st.get("f"))
            s.step(5)
            s.step(66)  # graphs of 32 steps plus single launches
            s.sync()
            out.append(s.get_f())
    assert np.array_equal(out[0], out[1]), np.abs(out[0] - out[1]).max()


def test_staged_fp64_vs_oracle():
    p, st = presets.cavity(n=16, Re=100, storage="f64")
    o = oracle_for(p)
    load_state(o, st)
    with rrlbm.Solver(p) as s:
        s.set_stage(1, 3, 3)
        s.init_state(st["rho"], st["ux"], st["uy"], st["uz"])
        s.step(40)
        o.run(40)
        m = s.macro()
        assert np.abs(m["ux"] - o.ux).max() / 0.1 < 1e-12
        assert np.abs(m["rho"] - o.rho).max() < 1e-13


def test_staged_rejections():
    p, st = presets.cavity(n=20, storage="f16")  # 20 x 2 B rows: not a multiple of 16 bytes
    with rrlbm.Solver(p) as s:
        with pytest.raises(rrlbm.RRError):
            s.set_stage(1)
    p, st = presets.cavity(n=24, storage="f64")
    with rrlbm.Solver(p) as s:
        with pytest.raises(rrlbm.RRError):
            s.set_stage(1, 22, 4)  # 4 stages x 22 rows x 24 x 27 x 8 B > 227 KB
        with pytest.raises(rrlbm.RRError):
            s.set_stage(1, 1, 5)


@pytest.mark.parametrize("k", [4, 0])  # periodic box; six-wall cavity (the x-wall gather path)
def test_staged_wait_timeout_reports_and_recovers(k):
    """Every pipeline wait of the staged step is bounded.  With a limit of 0
    polls every wait gives up at once: the step returns (no hang), rr_sync
    reports the pipeline timeout, and after the default limit is restored and
    the state set again the solver steps exactly as the tile step does."""
    p, st = _cases()[k]
    with rrlbm.Solver(p) as s:
        s.set_stage(1, 2, 2)
        assert s.wait_limit == 1 << 24
        s.set_wait_limit(0)
        assert s.wait_limit == 0
        s.init_state(st["rho"], st["ux"], st["uy"], st["uz"], f=st.get("f"))
        s.step(3)
        with pytest.raises(rrlbm.RRError) as e:
            s.sync()
        assert e.value.code == 5 and "pipeline timed out" in str(e.value)
        s.set_wait_limit(-1)
        assert s.wait_limit == 1 << 24
        s.init_state(st["rho"], st["ux"], st["uy"], st["uz"], f=st.get("f"))
        s.step(70)
        s.sync()
        got = s.get_f()
    with rrlbm.Solver(p) as t:
        t.set_stage(0)
        t.init_state(st["rho"], st["ux"], st["uy"], st["uz"], f=st.get("f"))
        t.step(70)
        want = t.get_f()
    assert np.array_equal(got, want)
