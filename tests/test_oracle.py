"""The oracle, pinned to the reference's own numbers (no GPU).

* lattice tables: the moment identities the RR scheme relies on;
* Taylor-Green D3Q27: the reference's shipped midline after 20,000 steps
  (Taylor_Green/RRBMa0.01L100.txt), reproduced to its printed 10 decimals;
* channel DNS and WALE-LES: the reference's CUDA kernels compiled for the
  host (oracle/_ref), bit for bit, live and through committed fixtures.
"""
import ctypes
import itertools
import os
import sys

import numpy as np
import pytest

from conftest import GOLDEN, ROOT
from oracle import oracle as O

sys.path.insert(0, GOLDEN)
from make_golden import fdbc_start  # noqa: E402


@pytest.mark.parametrize("q,order", [(27, O.ORDER_CUDA), (27, O.ORDER_FORTRAN), (19, O.ORDER_FORTRAN)])
def test_lattice_identities(q, order):
    L = O.lattice(q, order)
    c = np.array([[L.cx[i], L.cy[i], L.cz[i]] for i in range(q)], dtype=float)
    w = np.array(L.w[:q])
    assert abs(w.sum() - 1.0) < 1e-15
    assert np.allclose(np.einsum("i,ia,ib->ab", w, c, c), np.eye(3) / 3.0, atol=1e-15)
    assert np.allclose(np.einsum("i,ia->a", w, c), 0.0, atol=1e-15)
    for i in range(q):
        assert np.array_equal(c[L.opp[i]], -c[i])
    # second-order Hermite orthogonality: sum_i w H2_ab H2_cd = d_ac d_bd + d_ad d_bc
    H2 = {"200": L.H200, "020": L.H020, "002": L.H002, "110": L.H110, "101": L.H101, "011": L.H011}
    idx = {"200": (0, 0), "020": (1, 1), "002": (2, 2), "110": (0, 1), "101": (0, 2), "011": (1, 2)}
    for a, b in itertools.product(H2, H2):
        s = sum(w[i] * H2[a][i] * H2[b][i] for i in range(q))
        (p, r), (s1, t) = idx[a], idx[b]
        expect = float(p == s1 and r == t) + float(p == t and r == s1)
        assert abs(s - expect) < 1e-13, (a, b, s, expect)
    # the projected equilibrium carries rho, rho u and rho (cs^2 I + u u)
    rho, u = 1.03, np.array([0.021, -0.013, 0.007])
    feq = np.array([O.lib().orc_feq(ctypes.byref(L), i, rho, *u) for i in range(q)])
    assert abs(feq.sum() - rho) < 1e-14
    assert np.allclose(c.T @ feq, rho * u, atol=1e-15)
    assert np.allclose(np.einsum("i,ia,ib->ab", feq, c, c), rho * (np.eye(3) / 3 + np.outer(u, u)), atol=1e-15)


@pytest.mark.slow
def test_taylor_green_golden_midline():
    """Taylor_Green/D3Q27RR.f90 at L=100, LZ=2, tau=0.505, 20,000 steps.

    The program keeps its Hermite tables and intermediates in default REAL
    (D3Q27RR.f90:45-61); the oracle's tg_real4 mode follows that, and then
    matches every printed digit of the shipped midline.
    """
    gold = np.loadtxt(os.path.join(GOLDEN, "tg27_L100_midline.txt"))
    U0, visc, tau = O.tg_reference_params(100)
    assert tau == 0.505
    s = O.Sim(100, 100, 2, q=27, order=O.ORDER_FORTRAN, cs_mode=O.CS_INV_SQRT3, tau=tau)
    s.P.tg_real4 = 1
    s.init_tg_reference(U0)
    s.run(20000)
    jj1, jj2 = 49, 50  # L/2 and L/2+1, 1-based
    vnum = 0.5 * (s.uy[0, jj1, :] + s.uy[0, jj2, :])
    p = (s.rho[0] - 1.0) * (1.0 / 3.0)
    pnum = 0.5 * (p[jj1, :] + p[jj2, :])
    # printed with 10 decimals: half a unit of the last digit plus roundoff
    assert np.abs(vnum - gold[:, 1]).max() < 6e-11
    assert np.abs(pnum - gold[:, 3]).max() < 6e-11
    # the analytic column is the decayed vortex exp(-2 k^2 nu t), k = 2 pi / L
    x = np.arange(1, 101) - 0.5
    vtheo = -U0 * np.sin(2 * np.pi * x / 100) * np.exp(-2.0 * 4 * np.pi**2 * visc * 20000 / 100**2)
    assert np.abs(vtheo - gold[:, 2]).max() < 6e-11


def _ref_lib(les):
    path = os.path.join(ROOT, "oracle", "_ref", f"libref_16x12x8_les{les}.so")
    if not os.path.exists(path):
        pytest.skip("reference kernels not built here (oracle/ref_build.sh needs the reference sources)")
    R = ctypes.CDLL(path)
    for n in ["ref_tau", "ref_force_in_x", "ref_ustar", "ref_ystar"]:
        getattr(R, n).restype = ctypes.c_double
    R.ref_init_constants()
    return R


def _channel_sim(les, tau, fx):
    return O.Sim(16, 12, 8, q=27, order=O.ORDER_CUDA, cs_mode=O.CS_SQRT_RT, tau=tau,
                 force=(fx, 0.0, 0.0), les=bool(les), cw=0.5, faces=(0, 0, 1, 1, 0, 0))


@pytest.mark.parametrize("les", [0, 1])
def test_channel_matches_reference_fixture(les):
    g = np.load(os.path.join(GOLDEN, f"channel_ref_16x12x8_les{les}.npz"))
    s = _channel_sim(les, float(g["tau"]), float(g["fx"]))
    s.init_channel_loglaw(float(g["ustar"]), float(g["ystar"]))
    s.run(int(g["steps"]))
    for k in ("rho", "ux", "uy", "uz"):
        assert np.array_equal(getattr(s, k), g[k]), k
    assert np.array_equal(s.f.sum(axis=0), g["f_sum"])
    if les:
        assert np.array_equal(s.taut, g["taut"])


@pytest.mark.parametrize("les", [0, 1])
def test_channel_matches_reference_live(les):
    R = _ref_lib(les)
    s = _channel_sim(les, R.ref_tau(), R.ref_force_in_x())
    s.init_channel_loglaw(R.ref_ustar(), R.ref_ystar())
    # perturb the start so that every population and all three velocity
    # components are exercised, then hand the same state to both
    rng = np.random.default_rng(7)
    s.f *= 1.0 + 1e-3 * rng.standard_normal(s.f.shape)
    s.uy += 1e-3 * rng.standard_normal(s.uy.shape)
    s.uz += 1e-3 * rng.standard_normal(s.uz.shape)
    f, rho, ux, uy, uz = (a.copy() for a in (s.f, s.rho, s.ux, s.uy, s.uz))
    ft, fx, fy, fz, taut = (np.zeros_like(a) for a in (f, rho, rho, rho, rho))
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    R.ref_run(7, P(f), P(ft), P(rho), P(ux), P(uy), P(uz), P(fx), P(fy), P(fz), P(taut))
    s.run(7)
    assert np.array_equal(s.f, f)
    for k, a in (("rho", rho), ("ux", ux), ("uy", uy), ("uz", uz)):
        assert np.array_equal(getattr(s, k), a), k


@pytest.mark.parametrize("les", [0, 1])
def test_fdbc_matches_reference_fixture(les):
    """FDBC channel: the oracle against the reference's kernels' committed
    output (tests/golden/make_golden.py channel_fdbc), bit for bit."""
    g = np.load(os.path.join(GOLDEN, f"channel_fdbc_ref_16x12x8_les{les}.npz"))
    s = O.Sim(16, 12, 8, q=27, order=O.ORDER_CUDA, cs_mode=O.CS_SQRT_RT, tau=float(g["tau"]),
              force=(float(g["fx"]), 0.0, 0.0), les=bool(les), cw=0.5,
              faces=(0, 0, O.FACE_FDBC, O.FACE_FDBC, 0, 0))
    s.init_channel_loglaw(float(g["ustar"]), float(g["ystar"]))
    fdbc_start(s, int(g["seed"]))
    s.run(int(g["steps"]))
    for k in ("rho", "ux", "uy", "uz"):
        assert np.array_equal(getattr(s, k), g[k]), k
    assert np.array_equal(s.f.sum(axis=0), g["f_sum"])
    assert np.array_equal(s.f[:, :, [0, 11], :], g["f_wall"])
    if les:
        assert np.array_equal(s.taut, g["taut"])


@pytest.mark.parametrize("les", [0, 1])
def test_fdbc_matches_reference_live(les):
    """The finite-difference wall closure (FDBC, BC.cu:129-309, in place of RRBC)
    of the oracle against the reference's own FDBC kernel, bit for bit, with
    every wall neighbour extrapolated before the closure reads it."""
    R = _ref_lib(les)
    s = O.Sim(16, 12, 8, q=27, order=O.ORDER_CUDA, cs_mode=O.CS_SQRT_RT, tau=R.ref_tau(),
              force=(R.ref_force_in_x(), 0.0, 0.0), les=bool(les), cw=0.5,
              faces=(0, 0, O.FACE_FDBC, O.FACE_FDBC, 0, 0))
    s.init_channel_loglaw(R.ref_ustar(), R.ref_ystar())
    rng = np.random.default_rng(11)
    s.f *= 1.0 + 1e-3 * rng.standard_normal(s.f.shape)
    s.uy += 1e-3 * rng.standard_normal(s.uy.shape)
    s.uz += 1e-3 * rng.standard_normal(s.uz.shape)
    f, rho, ux, uy, uz = (a.copy() for a in (s.f, s.rho, s.ux, s.uy, s.uz))
    ft, fx, fy, fz, taut = (np.zeros_like(a) for a in (f, rho, rho, rho, rho))
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    R.ref_run_fdbc(5, P(f), P(ft), P(rho), P(ux), P(uy), P(uz), P(fx), P(fy), P(fz), P(taut))
    s.run(5)
    assert np.array_equal(s.f, f)
    for k, a in (("rho", rho), ("ux", ux), ("uy", uy), ("uz", uz)):
        assert np.array_equal(getattr(s, k), a), k
    # one more step from this state with RRBC instead: the two closures
    # differ on the wall rows only
    w = _channel_sim(les, R.ref_tau(), R.ref_force_in_x())
    w.f, w.rho, w.ux, w.uy, w.uz, w.taut = (a.copy() for a in (s.f, s.rho, s.ux, s.uy, s.uz, s.taut))
    s.run(1)
    w.run(1)
    assert np.array_equal(s.f[:, :, 1:-1, :], w.f[:, :, 1:-1, :])
    for y in (0, -1):
        assert np.abs(s.f[:, :, y, :] - w.f[:, :, y, :]).max() > 1e-9


def _laminar_golden(step):
    return np.loadtxt(os.path.join(GOLDEN, f"laminar_uy{step}.txt"))


@pytest.mark.slow
def test_laminar_channel_golden():
    """The oracle against the reference's own FP64 output of the laminar
    channel (Laminar/output/uy{5000,10000,60000}.dat, mid-y line over x).
    The reference's wall closure takes its force term from the last node of
    the collision sweep; in this flow (invariant in y and z, symmetric in x)
    that term equals the local one, so agreement is to roundoff."""
    from rrlbm import presets
    from helpers import load_state, oracle_for

    p, st = presets.laminar()
    o = oracle_for(p)
    load_state(o, st)
    done = 0
    for step in (5000, 10000, 60000):
        o.run(step - done)
        done = step
        ref = _laminar_golden(step)
        got = o.uy[0, 10, :]
        err = np.abs(got - ref).max() / np.abs(ref).max()
        print(f"laminar step {step}: max |uy - ref| / max uy = {err:.2e}")
        assert err < 1e-8, (step, err)


def test_rand_restatement_matches_c_library():
    """orc_rand (the C library's additive-feedback rand(), restated) against
    the C library itself after srand(12345), the reference's seed"""
    libc = ctypes.CDLL(None)
    libc.srand(12345)
    want = [libc.rand() for _ in range(5000)]
    T = O.Trip()
    O.lib().orc_srand(ctypes.byref(T), 12345)
    got = [O.lib().orc_rand(ctypes.byref(T)) for _ in range(5000)]
    assert got == want


@pytest.mark.parametrize("les", [0, 1])
def test_trip_forcing_matches_reference_live(les):
    """The start-up trip forcing (forcing_GP with the rand() phase, main.cu:29-46)
    of the oracle against the reference's own kernels, bit for bit, across two
    phase draws (steps 2000 and 4000) and the switch to the uniform force."""
    R = _ref_lib(les)
    R.ref_run_trip.argtypes = [ctypes.c_int, ctypes.c_longlong, ctypes.c_int] + [ctypes.c_void_p] * 10
    npforcing, steps = 4050, 4100
    s = _channel_sim(les, R.ref_tau(), R.ref_force_in_x())
    s.init_channel_loglaw(R.ref_ustar(), R.ref_ystar())
    s.enable_trip(npforcing)
    f, rho, ux, uy, uz = (a.copy() for a in (s.f, s.rho, s.ux, s.uy, s.uz))
    ft, fx, fy, fz, taut = (np.zeros_like(a) for a in (f, rho, rho, rho, rho))
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    R.ref_run_trip(steps, 0, npforcing, P(f), P(ft), P(rho), P(ux), P(uy), P(uz), P(fx), P(fy), P(fz), P(taut))
    s.run(steps)
    assert s.trip.istep == steps
    assert np.array_equal(s.f, f)
    for k, a in (("rho", rho), ("ux", ux), ("uy", uy), ("uz", uz)):
        assert np.array_equal(getattr(s, k), a), k


@pytest.mark.parametrize("les", [0, 1])
def test_fdbc_trip_forcing_matches_reference_live(les):
    """FDBC walls with the start-up trip forcing (per-node force fields read
    by the closure), bit for bit against the reference's kernels, across the
    phase draw at step 2000 and the switch to the uniform force."""
    R = _ref_lib(les)
    R.ref_run_trip_fdbc.argtypes = [ctypes.c_int, ctypes.c_longlong, ctypes.c_int] + [ctypes.c_void_p] * 10
    npforcing, steps = 2050, 2100
    s = O.Sim(16, 12, 8, q=27, order=O.ORDER_CUDA, cs_mode=O.CS_SQRT_RT, tau=R.ref_tau(),
              force=(R.ref_force_in_x(), 0.0, 0.0), les=bool(les), cw=0.5,
              faces=(0, 0, O.FACE_FDBC, O.FACE_FDBC, 0, 0))
    s.init_channel_loglaw(R.ref_ustar(), R.ref_ystar())
    s.enable_trip(npforcing)
    f, rho, ux, uy, uz = (a.copy() for a in (s.f, s.rho, s.ux, s.uy, s.uz))
    ft, fx, fy, fz, taut = (np.zeros_like(a) for a in (f, rho, rho, rho, rho))
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    R.ref_run_trip_fdbc(steps, 0, npforcing, P(f), P(ft), P(rho), P(ux), P(uy), P(uz), P(fx), P(fy), P(fz),
                        P(taut))
    s.run(steps)
    assert np.array_equal(s.f, f)
    for k, a in (("rho", rho), ("ux", ux), ("uy", uy), ("uz", uz)):
        assert np.array_equal(getattr(s, k), a), k


def test_bgk_matches_reference_live():
    """The oracle's BGK collision (BGK/collision.cu) and incompressible
    moments (BGK/macrovar.cu) with half-way bounce-back at y walls against the
    BGK program's own kernels built for the host, bit for bit."""
    path = os.path.join(ROOT, "oracle", "_ref", "libref_bgk_16x12x8.so")
    if not os.path.exists(path):
        pytest.skip("reference kernels not built here (oracle/ref_build.sh needs the reference sources)")
    R = ctypes.CDLL(path)
    for n in ("bgk_tau", "bgk_force_in_x"):
        getattr(R, n).restype = ctypes.c_double
    R.bgk_init_constants()
    tau, fx0 = R.bgk_tau(), R.bgk_force_in_x()
    s = O.Sim(16, 12, 8, q=27, order=O.ORDER_CUDA, cs_mode=O.CS_SQRT_RT, tau=tau, force=(fx0, 0.0, 0.0),
              faces=(0, 0, 2, 2, 0, 0), bgk=True)
    rng = np.random.default_rng(3)
    s.ux[...] = 0.02 * rng.standard_normal(s.shape)
    s.uy[...] = 0.01 * rng.standard_normal(s.shape)
    s.uz[...] = 0.01 * rng.standard_normal(s.shape)
    s.rho[...] = 1.0 + 1e-3 * rng.standard_normal(s.shape)
    s.init_equilibrium2()
    s.f *= 1.0 + 1e-3 * rng.standard_normal(s.f.shape)
    f, rho, ux, uy, uz = (a.copy() for a in (s.f, s.rho, s.ux, s.uy, s.uz))
    ft, fx, fy, fz = (np.zeros_like(a) for a in (f, rho, rho, rho))
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    R.bgk_run(25, P(f), P(ft), P(rho), P(ux), P(uy), P(uz), P(fx), P(fy), P(fz))
    s.run(25)
    assert np.array_equal(s.f, f)
    for k, a in (("rho", rho), ("ux", ux), ("uy", uy), ("uz", uz)):
        assert np.array_equal(getattr(s, k), a), k


def _out_lib():
    path = os.path.join(ROOT, "oracle", "_ref", "libref_out_16x12x8_les1.so")
    if not os.path.exists(path):
        pytest.skip("reference output routines not built here (oracle/ref_build.sh needs the reference sources)")
    R = ctypes.CDLL(path)
    R.ref_out_ustar.restype = ctypes.c_double
    R.ref_out_ystar.restype = ctypes.c_double
    dp = ctypes.POINTER(ctypes.c_double)
    R.ref_out_bind.argtypes = [dp] * 6
    for n in ("ref_out_diag", "ref_out_flow", "ref_out_profile", "ref_out_f"):
        getattr(R, n).argtypes = [ctypes.c_int]
    return R


def compare_output_dirs(a, b, istep, profile_first_column=True):
    """the reference's four files in directories a and b: byte for byte;
    Profiles.txt without its first column when profile_first_column is False
    (the reference prints an unspecified integer there)"""
    for name in ("statistics.dat", f"{istep:09d}.dat", f"f{istep:09d}.dat"):
        with open(os.path.join(a, name), "rb") as fa, open(os.path.join(b, name), "rb") as fb:
            assert fa.read() == fb.read(), name
    la = open(os.path.join(a, "Profiles.txt")).read().splitlines()
    lb = open(os.path.join(b, "Profiles.txt")).read().splitlines()
    assert len(la) == len(lb) and la[0] == lb[0] == str(istep)
    for x, y in zip(la[1:], lb[1:]):
        if profile_first_column:
            assert x == y
        else:
            assert x.split(",", 1)[1] == y.split(",", 1)[1]


def test_output_writers_match_reference(tmp_path, monkeypatch, capfd):
    """The oracle's restatement of the reference's writers against the
    reference's output.cu compiled for the host, on the same FP64 fields of a
    noisy 16 x 12 x 8 WALE channel after 7 steps: statistics.dat, the flow and
    population restart files byte for byte, Profiles.txt byte for byte but
    for its first column, and the same console line."""
    R = _out_lib()
    ustar, ystar = R.ref_out_ustar(), R.ref_out_ystar()
    from helpers import load_state, oracle_for
    from rrlbm import presets
    p, st = presets.channel(nx=16, ny=12, nz=8, les=True, variant="config", amp=0.2)
    assert (p.ustar, p.ystar) == (ustar, ystar)
    o = oracle_for(p)
    load_state(o, st)
    o.run(7)
    taut = o.wale()
    fields = [np.ascontiguousarray(v) for v in (o.rho, o.ux, o.uy, o.uz, taut, o.f)]
    a = tmp_path / "oracle"
    a.mkdir()
    O.write_outputs(a, 7, *fields[:5], fields[5], ustar, ystar)
    line_a = capfd.readouterr().out
    b = tmp_path / "ref"
    (b / "data").mkdir(parents=True)
    monkeypatch.chdir(b)
    R.ref_out_bind(*[v.ctypes.data_as(ctypes.POINTER(ctypes.c_double)) for v in fields])
    for fn in (R.ref_out_diag, R.ref_out_flow, R.ref_out_profile, R.ref_out_f):
        fn(7)
    line_b = capfd.readouterr().out
    assert line_a == line_b and line_a.startswith("Step 7 ")
    compare_output_dirs(str(a), str(b / "data"), 7, profile_first_column=False)
