"""GPU parity: the fused CUDA step through the C ABI against the oracle.

FP64 storage: the kernel evaluates the same RR step with a different
association of sums (pair-symmetric form), so results agree to roundoff:
tolerance 1e-12 of the velocity scale on u and 1e-13 absolute on rho and f
after up to 200 steps.
"""
import numpy as np
import pytest

import rrlbm
from rrlbm import presets
from helpers import load_state, oracle_for

pytestmark = pytest.mark.gpu

TOL_U = 1e-12   # relative to the velocity scale
TOL_RHO = 1e-13 # absolute on rho and on f


def _run_pair(p, st, steps, les=None, les_method=None):
    o = oracle_for(p, les)
    load_state(o, st)
    with rrlbm.Solver(p) as s:
        if les_method is not None:
            s.set_launch(s.launch()[0], les_method=les_method)
            assert s.launch()[1] == les_method
        s.init_state(st["rho"], st["ux"], st["uy"], st["uz"], f=st.get("f"))
        done = 0
        out = []
        for n in steps:
            s.step(n - done)
            o.run(n - done)
            done = n
            m = s.macro(taut=bool(p.use_les))
            f = s.get_f()
            out.append((n, m, f, o.rho.copy(), o.ux.copy(), o.uy.copy(), o.uz.copy(), o.f.copy(),
                        o.wale() if p.use_les else None))
    return out


def _check(out, uscale):
    for n, m, f, rho, ux, uy, uz, of, ot in out:
        assert np.abs(m["rho"] - rho).max() < TOL_RHO, n
        for k, ref in (("ux", ux), ("uy", uy), ("uz", uz)):
            assert np.abs(m[k] - ref).max() / uscale < TOL_U, (n, k, np.abs(m[k] - ref).max())
        assert np.abs(f - of).max() < TOL_RHO, n
        if ot is not None:
            assert np.abs(m["taut"] - ot).max() < 1e-12 * max(1e-30, np.abs(ot).max()) + 1e-18, n


@pytest.mark.parametrize("q", [27, 19])
def test_taylor_green_fp64(q):
    p, st = presets.taylor_green(L=24, nz=4, tau=0.6, Ma=0.05, q=q)
    _check(_run_pair(p, st, [1, 10, 100]), st["U0"])


def test_taylor_green_reference_start():
    p, st = presets.taylor_green(L=32, nz=2, q=27, variant="reference")
    _check(_run_pair(p, st, [1, 50]), st["U0"])


def test_cavity_reference_quasi2d():
    # Cavity/*.f90 geometry: walls x, y (lid x-hi moving +y), periodic z
    p, st = presets.cavity(n=24, Re=100.0, U=0.1, variant="reference")
    _check(_run_pair(p, st, [1, 10, 200]), 0.1)


def test_cavity_six_walls():
    p, st = presets.cavity(n=16, Re=100.0, U=0.1, variant="config")
    _check(_run_pair(p, st, [1, 10, 200]), 0.1)


@pytest.mark.parametrize("q", [27, 19])
def test_cavity_q(q):
    p, st = presets.cavity(n=12, Re=50.0, U=0.08, q=q, variant="config")
    _check(_run_pair(p, st, [5, 40]), 0.08)


def test_channel_dns_reference_start():
    # the reference channel (walls at y, force F_x) from its log-law start
    p, st = presets.channel(nx=16, ny=12, nz=8, les=False, variant="reference")
    _check(_run_pair(p, st, [1, 20, 100]), st["ustar"] * 20)


LES_METHODS = [0, 1]  # RR_LES_FUSED (z-marching tiles), RR_LES_TWO_PASS (two tile launches)


@pytest.mark.parametrize("method", LES_METHODS)
def test_channel_les_reference_start(method):
    p, st = presets.channel(nx=16, ny=12, nz=8, les=True, variant="reference")
    _check(_run_pair(p, st, [1, 20, 60], les_method=method), st["ustar"] * 20)


@pytest.mark.parametrize("method", LES_METHODS)
def test_channel_les_noise_start(method):
    # a start with all three velocity components and large gradients
    p, st = presets.channel(nx=40, ny=20, nz=12, les=True, variant="config", amp=0.3)
    _check(_run_pair(p, st, [1, 15], les_method=method), st["uc"])


@pytest.mark.parametrize("method", LES_METHODS)
def test_les_partial_tiles_and_forcing_axes(method):
    # grid not a multiple of the tile, force on all axes, walls on x and z
    p, st = presets.channel(nx=37, ny=11, nz=5, les=True, variant="config", amp=0.3)
    p.face[0] = p.face[1] = rrlbm.FACE_WALL
    if method == 1:
        p.face[4] = p.face[5] = rrlbm.FACE_WALL_BB
    p.force[1] = 1e-6
    p.force[2] = -2e-6
    _check(_run_pair(p, st, [1, 12], les_method=method), st["uc"])


@pytest.mark.parametrize("dims", [(34, 7, 5), (2, 9, 6), (3, 3, 3), (67, 5, 4)])
def test_odd_grids(dims):
    # x-rows whose interior is a multiple of the warp width, row counts that
    # are not a multiple of the row group, the thin-grid fallback (nx < 3)
    nx, ny, nz = dims
    # Re_tau scaled with ny so that the centreline velocity stays near 0.05
    p, st = presets.channel(nx=nx, ny=ny, nz=nz, Re_tau=1.7 * ny, les=False, variant="config", amp=0.3)
    p.force[1] = 3e-6
    _check(_run_pair(p, st, [1, 9]), st["uc"])


def test_fortran_order_readout():
    p, st = presets.cavity(n=10, Re=50.0, U=0.1, variant="config")
    with rrlbm.Solver(p) as s:
        s.init_state(st["rho"], st["ux"], st["uy"], st["uz"])
        s.step(7)
        fc = s.get_f()
    p.order = rrlbm.ORDER_FORTRAN
    with rrlbm.Solver(p) as s:
        s.init_state(st["rho"], st["ux"], st["uy"], st["uz"])
        s.step(7)
        ff = s.get_f()
    assert np.array_equal(ff, fc[presets.FORTRAN_TO_CUDA_27])


def test_graph_path_matches_single_launches():
    p, st = presets.cavity(n=16, Re=100.0, U=0.1, storage="f32")
    with rrlbm.Solver(p) as a, rrlbm.Solver(p) as b:
        for s in (a, b):
            s.init_state(st["rho"], st["ux"], st["uy"], st["uz"])
        a.step(131)  # graphs + remainder
        for _ in range(131):
            b.step(1)
        ma, mb = a.macro(), b.macro()
    for k in ma:
        assert np.array_equal(ma[k], mb[k]), k


def test_diag_profile_accumulators():
    p, st = presets.channel(nx=16, ny=12, nz=8, les=True, variant="config", amp=0.2)
    with rrlbm.Solver(p) as s:
        s.init_state(st["rho"], st["ux"], st["uy"], st["uz"])
        s.step(5)
        m = s.macro(taut=True)
        d = s.diag()
        prof, tmean = s.profile()
        s.accumulate()
        s.step(1)
        s.accumulate()
        acc, tacc, ns = s.get_accum()
    # diag_flow: plain means (output.cu:26-35)
    assert np.allclose(d, [m["ux"].mean(), m["uy"].mean(), m["uz"].mean(), m["rho"].mean()],
                       rtol=1e-13, atol=1e-17)
    # output_profile: per-plane means and second moments about them
    mu = m["ux"].mean(axis=(0, 2))
    mv = m["uy"].mean(axis=(0, 2))
    ur = m["ux"] - mu[None, :, None]
    vr = m["uy"] - mv[None, :, None]
    assert np.allclose(prof[:, 2], mu, rtol=1e-13, atol=1e-18)
    assert np.allclose(prof[:, 8], (ur * vr).mean(axis=(0, 2)), rtol=1e-10, atol=1e-20)
    assert np.allclose(tmean, m["taut"].mean(axis=(0, 2)), rtol=1e-12, atol=1e-20)
    assert ns == 2 and np.all(np.isfinite(acc))


def test_save_load_roundtrip(tmp_path):
    p, st = presets.cavity(n=12, Re=100.0, U=0.1)
    with rrlbm.Solver(p) as s:
        s.init_state(st["rho"], st["ux"], st["uy"], st["uz"])
        s.step(9)
        s.save(str(tmp_path))
        s.step(5)
        m1 = s.macro()
    with rrlbm.Solver(p) as s:
        s.load(str(tmp_path), 9)
        assert s.istep == 9
        s.step(5)
        m2 = s.macro()
    for k in m1:
        assert np.abs(m1[k] - m2[k]).max() < 1e-14, k
    # the reference's restart files: 4 N then 27 N doubles
    n = p.n
    assert (tmp_path / "000000009.dat").stat().st_size == 4 * n * 8
    assert (tmp_path / "f000000009.dat").stat().st_size == 27 * n * 8


def test_watchdog_reports_blow_up():
    # far beyond the stable range: the density watchdog must trip, the
    # context must stay usable
    p, st = presets.taylor_green(L=16, nz=2, tau=0.5000001, Ma=1.5)
    with rrlbm.Solver(p) as s:
        s.init_state(st["rho"], st["ux"], st["uy"], st["uz"], f=st["f"])
        s.step(400)
        with pytest.raises(rrlbm.RRError) as e:
            s.sync()
        assert e.value.code == 5
    p2, st2 = presets.cavity(n=8)
    with rrlbm.Solver(p2) as s:
        s.init_state(st2["rho"], st2["ux"], st2["uy"], st2["uz"])
        s.step(3)
        s.sync()


def test_state_errors():
    p, st = presets.cavity(n=8)
    with rrlbm.Solver(p) as s:
        with pytest.raises(rrlbm.RRError) as e:
            s.step(1)
        assert e.value.code == 7
        s.init_state(st["rho"], st["ux"], st["uy"], st["uz"])
        with pytest.raises(rrlbm.RRError):
            s.macro()


def test_laminar_channel_golden():
    """The FP64 kernel against the reference's own output of the laminar
    channel (Laminar/output/uy*.dat, mid-y line over x) and against the
    oracle; same bar as the oracle's golden test."""
    import os
    from conftest import GOLDEN

    p, st = presets.laminar()
    o = oracle_for(p)
    load_state(o, st)
    with rrlbm.Solver(p) as s:
        s.init_state(st["rho"], st["ux"], st["uy"], st["uz"], f=st["f"])
        done = 0
        for step in (5000, 10000, 60000):
            s.step(step - done)
            o.run(step - done)
            done = step
            m = s.macro()
            ref = np.loadtxt(os.path.join(GOLDEN, f"laminar_uy{step}.txt"))
            got = m["uy"][0, 10, :]
            err = np.abs(got - ref).max() / np.abs(ref).max()
            print(f"\nlaminar step {step}: GPU max |uy - ref| / max uy = {err:.2e}")
            assert err < 1e-8, (step, err)
            assert np.abs(m["uy"] - o.uy).max() / np.abs(ref).max() < 1e-11


@pytest.mark.parametrize("les", [False, True])
def test_trip_forcing(les):
    """The channel program's start-up trip forcing (forcing_GP with the rand()
    phase) against the oracle, which is pinned bit for bit to the reference's
    kernels.  The flow to step 400 (later steps of this small forced channel
    amplify roundoff by about 10 per 300 steps, trip or not); the force field
    itself, which the solver reads out, across the phase draws at steps 2000
    and 4000 and the switch to the uniform force at step 4050."""
    import ctypes
    from oracle import oracle as O

    p, st = presets.channel(nx=16, ny=12, nz=8, les=les, variant="reference")
    p.trip_steps = 4050
    o = oracle_for(p)
    load_state(o, st)
    o.enable_trip(4050)
    ref_rand = O.Trip()
    O.lib().orc_srand(ctypes.byref(ref_rand), 12345)
    phase = 0.0
    want = np.empty((3,) + o.shape)
    with rrlbm.Solver(p) as s:
        s.init_state(st["rho"], st["ux"], st["uy"], st["uz"], f=st.get("f"))
        done = 0
        for n in (1, 100, 400, 1999, 2000, 2001, 4000, 4049, 4050, 4051):
            s.step(n - done)
            if n <= 400:
                o.run(n - done)
                m = s.macro()
                scale = st["ustar"] * 20
                for k, ref in (("ux", o.ux), ("uy", o.uy), ("uz", o.uz)):
                    err = np.abs(m[k] - ref).max() / scale
                    assert err < 1e-12, (n, k, err)
                assert np.abs(m["rho"] - o.rho).max() < 1e-13, n
            # the oracle's field of step n (phases drawn at steps 2000, 4000)
            for k in range(done + 1, n + 1):
                if k % 2000 == 0 and k < 4050:
                    phase = O.lib().orc_rand(ctypes.byref(ref_rand)) / 2147483647.0
            done = n
            if n < 4050:
                P = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
                O.lib().orc_trip_force(ctypes.byref(o.P), n, phase, P(want[0]), P(want[1]), P(want[2]))
            else:
                want[0], want[1], want[2] = p.force[0], 0.0, 0.0
            got = s.get_force()
            assert np.abs(got - want).max() <= 1e-13 * np.abs(want).max(), n


@pytest.mark.parametrize("case", ["channel", "tg"])
def test_bgk_collision(case):
    """The BGK program's collision (incompressible velocity, bounce-back walls)
    against the oracle, which is pinned bit for bit to that program's kernels."""
    if case == "channel":
        p, st = presets.channel(nx=16, ny=12, nz=8, Re_tau=20, les=False, variant="config", amp=0.2)
        p.face[2] = p.face[3] = rrlbm.FACE_WALL_BB
        scale = st["uc"]
    else:
        p, st = presets.taylor_green(L=24, nz=6, tau=0.7, Ma=0.08)
        st["f"] = None
        scale = st["U0"]
    p.collision = rrlbm.COLL_BGK
    _check(_run_pair(p, st, [1, 20, 100]), scale)


def test_bgk_rejects_regularized_walls():
    p, st = presets.cavity(n=8)
    p.collision = rrlbm.COLL_BGK
    with pytest.raises(rrlbm.RRError) as e:
        rrlbm.Solver(p)
    assert e.value.code == 4
