"""GPU parity of the finite-difference wall closure (RR_FACE_FDBC; the
reference's FDBC, BC.cu:129-309) through the C ABI.

The oracle restates FDBC with every wall velocity extrapolated before any
closure reads its neighbours' and is pinned bit for bit to the reference's
kernel run that way (tests/test_oracle.py).  FP64 storage agrees with it to
roundoff: 1e-12 of the velocity scale on u, 1e-13 absolute on rho and f.
FP32 / FP16 / BF16 storage: mean profile against the FP64 run (bars below).
Batches: bit-identical alone and in a mix (tolerance zero).
"""
import sys

import numpy as np
import pytest

import rrlbm
from rrlbm import presets
from conftest import GOLDEN
from helpers import load_state, oracle_for

sys.path.insert(0, GOLDEN)
from make_golden import fdbc_start  # noqa: E402

pytestmark = pytest.mark.gpu

TOL_U = 1e-12
TOL_RHO = 1e-13


def _fdbc(p, lo=True, hi=True):
    if lo:
        p.face[2] = rrlbm.FACE_FDBC
    if hi:
        p.face[3] = rrlbm.FACE_FDBC
    return p


def _fixture_params(les, storage="f64"):
    g = np.load(f"{GOLDEN}/channel_fdbc_ref_16x12x8_les{les}.npz")
    p, _ = presets.channel(nx=16, ny=12, nz=8, les=bool(les), variant="reference", storage=storage)
    p.tau = float(g["tau"])
    p.force[0] = float(g["fx"])
    p.ustar = float(g["ustar"])
    p.ystar = float(g["ystar"])
    p.cw = 0.5
    return _fdbc(p), g


def _loglaw_start(p, seed):
    """the oracle's log-law start perturbed as the fixtures' (fdbc_start)"""
    o = oracle_for(p)
    o.init_channel_loglaw(p.ustar, p.ystar)
    fdbc_start(o, seed)
    return o


def _solver_from(p, o):
    s = rrlbm.Solver(p)
    s.init_state(o.rho.copy(), o.ux.copy(), o.uy.copy(), o.uz.copy(), f=o.f.copy())
    return s


def _compare(s, o, uscale, n, les):
    m = s.macro(taut=bool(les))
    assert np.abs(m["rho"] - o.rho).max() < TOL_RHO, n
    for k in ("ux", "uy", "uz"):
        err = np.abs(m[k] - getattr(o, k)).max() / uscale
        assert err < TOL_U, (n, k, err)
    f = s.get_f()
    assert np.abs(f - o.f).max() < TOL_RHO, n
    if les:
        ot = o.wale()
        assert np.abs(m["taut"] - ot).max() < 1e-12 * max(1e-30, np.abs(ot).max()) + 1e-18, n
    return m, f


@pytest.mark.parametrize("les", [0, 1])
def test_fdbc_fixture_and_oracle_fp64(les):
    """Against the reference kernels' committed output at step 20 and the
    oracle at steps 1, 20 and 100."""
    p, g = _fixture_params(les)
    o = _loglaw_start(p, int(g["seed"]))
    uscale = p.ustar * 20
    with _solver_from(p, o) as s:
        done = 0
        for n in (1, 20, 100):
            s.step(n - done)
            o.run(n - done)
            done = n
            m, f = _compare(s, o, uscale, n, les)
            if n == 20:
                for k in ("ux", "uy", "uz"):
                    assert np.abs(m[k] - g[k]).max() / uscale < TOL_U, k
                assert np.abs(m["rho"] - g["rho"]).max() < TOL_RHO
                assert np.abs(f[:, :, [0, 11], :] - g["f_wall"]).max() < TOL_RHO
                assert np.abs(f.sum(axis=0) - g["f_sum"]).max() < 1e-12


@pytest.mark.parametrize("method", ["tile", "staged"])
def test_fdbc_dns_step_methods(method):
    p, g = _fixture_params(0)
    o = _loglaw_start(p, 5)
    with _solver_from(p, o) as s:
        if method == "staged":
            s.set_stage(1)
            assert s.stage()[0] == 1
        s.step(70)  # past 64 steps: the captured-graph path too
        o.run(70)
        _compare(s, o, p.ustar * 20, 70, 0)


@pytest.mark.parametrize("dims,les", [((37, 5, 5), False), ((37, 5, 5), True), ((2, 6, 3), False),
                                      ((40, 4, 9), False), ((33, 7, 11), True)])
def test_fdbc_odd_grids(dims, les):
    """Partial 32 x 8 tiles in x and z, the thin-grid step (nx < 3), the
    smallest height (ny = 4), a force on every axis."""
    nx, ny, nz = dims
    p, st = presets.channel(nx=nx, ny=ny, nz=nz, Re_tau=1.7 * ny, les=les, variant="config", amp=0.3)
    _fdbc(p)
    p.force[1] = 2e-6
    p.force[2] = -1e-6
    o = oracle_for(p)
    load_state(o, st)
    with rrlbm.Solver(p) as s:
        s.init_state(st["rho"], st["ux"], st["uy"], st["uz"])
        done = 0
        for n in (1, 9):
            s.step(n - done)
            o.run(n - done)
            done = n
            _compare(s, o, st["uc"], n, les)


@pytest.mark.parametrize("other", [rrlbm.FACE_WALL, rrlbm.FACE_WALL_BB])
def test_fdbc_one_face(other):
    """FDBC on y-lo, another closure on y-hi."""
    p, st = presets.channel(nx=20, ny=10, nz=6, Re_tau=17, les=False, variant="config", amp=0.2)
    _fdbc(p, hi=False)
    p.face[3] = other
    o = oracle_for(p)
    load_state(o, st)
    with rrlbm.Solver(p) as s:
        s.init_state(st["rho"], st["ux"], st["uy"], st["uz"])
        s.step(30)
        o.run(30)
        _compare(s, o, st["uc"], 30, False)


@pytest.mark.parametrize("les", [False, True])
def test_fdbc_trip_forcing(les):
    """The start-up trip forcing (per-node force fields) with the FDBC walls."""
    p, st = presets.channel(nx=16, ny=12, nz=8, les=les, variant="reference")
    _fdbc(p)
    p.trip_steps = 4050
    o = oracle_for(p)
    load_state(o, st)
    o.enable_trip(4050)
    with rrlbm.Solver(p) as s:
        s.init_state(st["rho"], st["ux"], st["uy"], st["uz"], f=st.get("f"))
        done = 0
        for n in (1, 50, 200):
            s.step(n - done)
            o.run(n - done)
            done = n
            _compare(s, o, st["ustar"] * 20, n, les)


def _mean_u(storage, les):
    p, st = presets.channel(nx=48, ny=24, nz=16, Re_tau=40, les=les, variant="config", amp=0.2,
                            storage=storage)
    _fdbc(p)
    with rrlbm.Solver(p) as s:
        s.init_state(st["rho"], st["ux"], st["uy"], st["uz"])
        s.step(400)
        m = s.macro()
    return m["ux"].mean(axis=(0, 2)), st["uc"]


@pytest.mark.parametrize("les", [False, True])
def test_fdbc_low_precision_storage(les):
    """FP32 / FP16 / BF16 storage (FP32 arithmetic) against FP64 storage:
    mean profile <u>(y) after 400 steps, relative to the centreline velocity
    (bars: 1e-4 for FP32, 1e-2 for FP16 and BF16)."""
    ref, uc = _mean_u("f64", les)
    for storage, bar in (("f32", 1e-4), ("f16", 1e-2), ("bf16", 1e-2)):
        got, _ = _mean_u(storage, les)
        err = np.abs(got - ref).max() / uc
        print(f"\nFDBC channel 48x24x16 400 steps les={les} {storage}: max |<u> - <u>64| / U_c = {err:.2e}")
        assert err < bar, (storage, err)


@pytest.mark.parametrize("mode", [0, 1])
def test_fdbc_alone_vs_batch_bit_identical(mode):
    """FDBC members (which step through their own launches) beside tile-step
    members; one WALE member joins on the other buffer parity, so its wall
    tau_t slots are relabelled with its buffers."""
    doms = [presets.channel(nx=40, ny=18, nz=10, Re_tau=36, les=False, storage="f16", variant="config", amp=0.1),
            presets.channel(nx=24, ny=16, nz=12, Re_tau=32, les=True, storage="f16", variant="config", amp=0.1),
            presets.cavity(n=16, Re=300, storage="f16")]
    _fdbc(doms[0][0])
    _fdbc(doms[1][0])
    late = presets.channel(nx=20, ny=12, nz=8, Re_tau=24, les=True, storage="f32", variant="config", amp=0.1)
    _fdbc(late[0])

    def solver(p, st):
        s = rrlbm.Solver(p)
        s.init_state(st["rho"], st["ux"], st["uy"], st["uz"], f=st.get("f"))
        return s

    early, steps = 3, 70
    alone = []
    for p, st in doms:
        with solver(p, st) as s:
            s.step(early + steps)
            alone.append((s.get_f(), s.macro(taut=bool(p.use_les))))
    with solver(*late) as s:
        s.step(steps)
        alone_late = (s.get_f(), s.macro(taut=True))
    solvers = [solver(p, st) for p, st in doms]
    with rrlbm.Batch() as b:
        b.set_mode(mode, 4)
        for s in solvers:
            b.add(s)
        b.step(early)
        s_late = solver(*late)
        b.add(s_late)
        b.step(steps)
        b.sync()
        for k, s in enumerate(solvers):
            f = s.get_f()
            assert np.array_equal(f, alone[k][0]), (k, np.abs(f - alone[k][0]).max())
        assert np.array_equal(s_late.get_f(), alone_late[0])
        m = s_late.macro(taut=True)
        for key in ("rho", "ux", "uy", "uz", "taut"):
            assert np.array_equal(m[key], alone_late[1][key]), key
    for s in solvers + [s_late]:
        s.close()


def test_fdbc_les_is_two_pass():
    """WALE with FDBC runs the two tile passes with the closure between them;
    the fused WALE method is refused."""
    p, _ = _fixture_params(1)
    with rrlbm.Solver(p) as s:
        assert s.launch()[1] == 1
        with pytest.raises(rrlbm.RRError) as e:
            s.set_launch(s.launch()[0], les_method=0)
        assert e.value.code == 4


@pytest.mark.parametrize("les", [False, True])
def test_fdbc_d3q19(les):
    """D3Q19 (Fortran population order) with the FDBC walls."""
    p, st = presets.channel(nx=20, ny=9, nz=6, Re_tau=15, q=19, les=les, variant="config", amp=0.3)
    _fdbc(p)
    o = oracle_for(p)
    load_state(o, st)
    with rrlbm.Solver(p) as s:
        s.init_state(st["rho"], st["ux"], st["uy"], st["uz"])
        done = 0
        for n in (1, 12):
            s.step(n - done)
            o.run(n - done)
            done = n
            _compare(s, o, st["uc"], n, les)


def test_fdbc_les_save_load_restart(tmp_path):
    """A restart from the reference's files continues the FDBC + WALE run: the
    wall nodes' tau_t is rebuilt from the saved velocities, as the first
    collision after the restart takes it."""
    p, g = _fixture_params(1)
    o = _loglaw_start(p, 3)
    with _solver_from(p, o) as s:
        s.step(9)
        s.save(str(tmp_path))
        s.step(6)
        m1, f1 = s.macro(taut=True), s.get_f()
    with rrlbm.Solver(p) as s:
        s.load(str(tmp_path), 9)
        s.step(6)
        m2, f2 = s.macro(taut=True), s.get_f()
    for k in m1:
        assert np.abs(m1[k] - m2[k]).max() <= 1e-13 * max(1.0, np.abs(m1[k]).max()), k
    assert np.abs(f1 - f2).max() < 1e-14


@pytest.mark.parametrize("les", [False, True])
def test_fdbc_autotuner_keeps_results(les):
    """rr_tune's trial launch shapes (tile rows, staged blocks) leave an FDBC
    solver's populations unchanged, bit for bit."""
    p, st = presets.channel(nx=32, ny=16, nz=12, Re_tau=27, les=les, storage="f16", variant="config", amp=0.1)
    _fdbc(p)

    def solver():
        s = rrlbm.Solver(p)
        s.init_state(st["rho"], st["ux"], st["uy"], st["uz"])
        return s

    with solver() as s, solver() as r:
        run = s.tune(trial_steps=2)
        s.step(3)
        r.step(run + 3)
        assert np.array_equal(s.get_f(), r.get_f())
