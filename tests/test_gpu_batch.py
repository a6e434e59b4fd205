"""Batches (rr_batch_*) and the autotuner (rr_tune, rr_batch_tune).

A batch advances its members with one persistent launch per step and class;
each member's nodes get the arithmetic and the rounding stream of the
member's own rr_step, so the populations after N steps must be bit-identical
alone and in a mix (the stated tolerance is exactly zero).  The autotuner's
launch shapes must not change any result either."""
import numpy as np
import pytest

import rrlbm
from rrlbm import presets

pytestmark = pytest.mark.gpu


def _domains():
    """A mix of kinds, sizes, lattices, storages and step kinds."""
    out = []
    out.append(presets.taylor_green(L=24, nz=24, tau=0.6, Ma=0.05, storage="f16"))
    out.append(presets.taylor_green(L=20, nz=8, tau=0.55, Ma=0.08, q=19, storage="f32"))
    out.append(presets.cavity(n=20, Re=400, storage="f16"))
    out.append(presets.cavity(n=18, Re=200, storage="bf16"))
    out.append(presets.cavity(n=12, Re=100, storage="f64"))
    out.append(presets.channel(nx=40, ny=18, nz=10, Re_tau=36, les=False, storage="f16", variant="config", amp=0.1))
    out.append(presets.channel(nx=24, ny=16, nz=12, Re_tau=32, les=True, storage="f16", variant="config", amp=0.1))
    out.append(presets.channel(nx=36, ny=14, nz=6, Re_tau=28, les=False, storage="f64", variant="config", amp=0.1))
    return out


def _solver(p, st):
    s = rrlbm.Solver(p)
    s.init_state(st["rho"], st["ux"], st["uy"], st["uz"], f=st.get("f"))
    return s


@pytest.mark.parametrize("mode", [0, 1])
def test_alone_vs_mix_bit_identical(mode):
    doms = _domains()
    late = presets.cavity(n=16, Re=300, storage="f16")  # joins on the other buffer parity
    steps_early, steps = 3, 70  # 70 >= 64: the graph path plus single launches
    alone = []
    for p, st in doms:
        with _solver(p, st) as s:
            s.step(steps_early + steps)
            alone.append(s.get_f())
    with _solver(*late) as s:
        s.step(steps)
        alone_late = s.get_f()
    solvers = [_solver(p, st) for p, st in doms]
    with rrlbm.Batch() as b:
        b.set_mode(mode, 4)
        for s in solvers:
            b.add(s)
        b.step(steps_early)
        s_late = _solver(*late)
        b.add(s_late)
        b.step(steps)
        b.sync()
        for k, s in enumerate(solvers):
            assert s.istep == steps_early + steps
            got = s.get_f()
            assert np.array_equal(got, alone[k]), (k, np.abs(got - alone[k]).max())
        assert np.array_equal(s_late.get_f(), alone_late)
        # readouts of members work and removal hands the solver back
        b.remove(solvers[0])
        solvers[0].step(2)
        solvers[0].sync()
    for s in solvers + [s_late]:
        s.close()


def test_member_state_calls_refused():
    p, st = presets.cavity(n=10)
    with _solver(p, st) as s, rrlbm.Batch() as b:
        b.add(s)
        for call in (lambda: s.step(1), lambda: s.init_state(st["rho"], st["ux"], st["uy"], st["uz"])):
            with pytest.raises(rrlbm.RRError) as e:
                call()
            assert e.value.code == 7
        with pytest.raises(rrlbm.RRError):
            b.add(s)  # already a member
        b.step(2)
        m = s.macro()
        assert np.isfinite(m["ux"]).all()


def test_batch_watchdog_names_member():
    good = presets.cavity(n=10)
    bad = presets.taylor_green(L=16, nz=2, tau=0.5000001, Ma=1.5)
    sg, sb = _solver(*good), _solver(*bad)
    with rrlbm.Batch() as b:
        b.add(sg)
        b.add(sb)
        b.step(400)
        with pytest.raises(rrlbm.RRError) as e:
            b.sync()
        assert e.value.code == 5 and "member 1" in str(e.value)
    sg.sync()
    sg.close()
    sb.close()


@pytest.mark.parametrize("block,cps,order,group,mode", [(64, 0, 0, 0, 0), (128, 1, 1, 1 << 20, 0),
                                                        (256, 2, 0, 8 << 20, 0), (256, 0, 1, 64 << 20, 0),
                                                        (256, 0, 0, 0, 1)])
def test_launch_shapes_change_nothing(block, cps, order, group, mode):
    doms = _domains()[:4]
    ref = []
    for p, st in doms:
        with _solver(p, st) as s:
            s.step(9)
            ref.append(s.get_f())
    solvers = [_solver(p, st) for p, st in doms]
    for s in solvers:
        s.set_launch(64 if block == 64 else 32)
    with rrlbm.Batch() as b:
        b.set_launch(block, cps, order)
        b.grouping = group
        b.set_mode(mode, 3)
        assert b.launch() == (block, cps, order) and b.grouping == group and b.mode() == (mode, 3)
        for s in solvers:
            b.add(s)
        b.step(2)
        b.step(7)  # odd parity at the start of a grouped run
        for k, s in enumerate(solvers):
            assert np.array_equal(s.get_f(), ref[k])
    for s in solvers:
        s.close()


def test_autotuners_keep_results():
    doms = _domains()
    solvers = [_solver(p, st) for p, st in doms]
    with rrlbm.Batch() as b:
        for s in solvers:
            b.add(s)
        run = b.tune(trial_steps=3)
        assert run >= 4
        b.step(5)
        b.sync()
        got = [s.get_f() for s in solvers]
        for s in solvers:
            assert s.istep == run + 5
    for k, (p, st) in enumerate(doms):
        with _solver(p, st) as s:
            s.step(run + 5)
            assert np.array_equal(s.get_f(), got[k]), k
    for s in solvers:
        s.close()
    # single-solver tuner: tile step and WALE step
    for p, st in (doms[2], doms[6]):
        with _solver(p, st) as s, _solver(p, st) as r:
            run = s.tune(trial_steps=2)
            s.step(3)
            r.step(run + 3)
            assert np.array_equal(s.get_f(), r.get_f())
            rg, method, tile = s.launch()
            assert rg % 32 == 0 and method in (0, 1) and tile[0] * tile[1] <= 256
            # the size class remembers the shape for later solvers
            with rrlbm.Solver(p) as t:
                assert t.launch() == s.launch()
