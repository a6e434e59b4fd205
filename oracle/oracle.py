"""ctypes front end of the CPU oracle (liboracle.so).

TEST INFRASTRUCTURE ONLY.  The checker that the parity tests, the smoke check
and the benchmark's CPU-baseline leg use; the product (the CUDA library
behind include/rr_api.h and its Python mirror) never imports this module.

Presets reproduce the reference programs:
  * ``tg_reference``  Taylor_Green/D3Q27RR.f90 (and D3Q19RR.f90): periodic,
    Fortran velocity order, cs = 1/sqrt(3), analytic start.
  * ``cavity_reference``  Cavity/*.f90: walls at x=1, x=lx (lid, +y) and
    y=1, y=ly, periodic z, Fortran order, cs = sqrt(1/3).
  * ``channel_reference``  RR27V33_code_DNS_LES/*.cu: walls at y=0, y=LY-1,
    periodic x/z, uniform F_x, CUDA order.
"""
import ctypes
import os
import math

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

ORDER_CUDA, ORDER_FORTRAN = 0, 1
CS_SQRT_RT, CS_INV_SQRT3 = 0, 1
FACE_PERIODIC, FACE_WALL, FACE_WALL_BB, FACE_FDBC = 0, 1, 2, 3


class Lattice(ctypes.Structure):
    _fields_ = [("q", ctypes.c_int), ("ord", ctypes.c_int),
                ("cx", ctypes.c_int * 27), ("cy", ctypes.c_int * 27), ("cz", ctypes.c_int * 27),
                ("opp", ctypes.c_int * 27), ("w", ctypes.c_double * 27),
                ("rt", ctypes.c_double), ("cs", ctypes.c_double), ("cs3", ctypes.c_double)] + [
        (n, ctypes.c_double * 27) for n in
        ["H100", "H010", "H001", "H110", "H101", "H011", "H200", "H020", "H002",
         "H210", "H201", "H021", "H120", "H102", "H012", "H111",
         "Hp1", "Hm1", "Hp2", "Hm2", "Hp3", "Hm3"]]


class Params(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
                ("lat", Lattice), ("tau", ctypes.c_double), ("force", ctypes.c_double * 3),
                ("les", ctypes.c_int), ("cw", ctypes.c_double), ("face", ctypes.c_int * 6),
                ("uwall", (ctypes.c_double * 3) * 6), ("tg_real4", ctypes.c_int),
                ("ffield", ctypes.POINTER(ctypes.c_double)), ("bgk", ctypes.c_int)]


class Trip(ctypes.Structure):
    """orc_trip: the reference channel's start-up trip forcing"""
    _fields_ = [("trip_steps", ctypes.c_int), ("istep", ctypes.c_longlong), ("phase", ctypes.c_double),
                ("r", ctypes.c_int32 * 34), ("k", ctypes.c_int),
                ("fx", ctypes.POINTER(ctypes.c_double)), ("fy", ctypes.POINTER(ctypes.c_double)),
                ("fz", ctypes.POINTER(ctypes.c_double))]


class _State(ctypes.Structure):
    _fields_ = [(n, ctypes.POINTER(ctypes.c_double)) for n in
                ["f", "ftmp", "rho", "ux", "uy", "uz", "taut"]]


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "liboracle.so")
        if not os.path.exists(path):
            raise RuntimeError("oracle not built: run make -C oracle")
        L = ctypes.CDLL(path)
        dp = ctypes.POINTER(ctypes.c_double)
        L.orc_lattice_init.argtypes = [ctypes.POINTER(Lattice), ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.orc_step.argtypes = [ctypes.POINTER(Params), ctypes.POINTER(_State)]
        L.orc_run.argtypes = [ctypes.POINTER(Params), ctypes.POINTER(_State), ctypes.c_int]
        L.orc_wale.argtypes = [ctypes.POINTER(Params), dp, dp, dp, dp]
        L.orc_stream_walls.argtypes = [ctypes.POINTER(Params), dp, dp]
        L.orc_moments_all.argtypes = [ctypes.POINTER(Params), dp, dp, dp, dp, dp]
        L.orc_collide_all.argtypes = [ctypes.POINTER(Params), dp, dp, dp, dp, dp, dp]
        L.orc_init_tg_reference.argtypes = [ctypes.POINTER(Params), ctypes.c_double, dp, dp, dp, dp, dp]
        L.orc_init_tg_config.argtypes = [ctypes.POINTER(Params), ctypes.c_double, dp, dp, dp, dp, dp]
        L.orc_init_equilibrium2.argtypes = [ctypes.POINTER(Params), dp, dp, dp, dp, dp]
        L.orc_init_channel_loglaw.argtypes = [ctypes.POINTER(Params), ctypes.c_double, ctypes.c_double,
                                              dp, dp, dp, dp, dp]
        L.orc_init_channel_config.argtypes = [ctypes.POINTER(Params), ctypes.c_double, ctypes.c_double,
                                              ctypes.c_uint64, dp, dp, dp, dp, dp]
        L.orc_uniform_pm1.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64]
        L.orc_uniform_pm1.restype = ctypes.c_double
        L.orc_feq.argtypes = [ctypes.POINTER(Lattice), ctypes.c_int] + [ctypes.c_double] * 4
        L.orc_feq.restype = ctypes.c_double
        L.orc_set_threads.argtypes = [ctypes.c_int]
        L.orc_srand.argtypes = [ctypes.POINTER(Trip), ctypes.c_uint]
        L.orc_rand.argtypes = [ctypes.POINTER(Trip)]
        L.orc_rand.restype = ctypes.c_int
        L.orc_trip_force.argtypes = [ctypes.POINTER(Params), ctypes.c_longlong, ctypes.c_double, dp, dp, dp]
        L.orc_run_trip.argtypes = [ctypes.POINTER(Params), ctypes.POINTER(_State), ctypes.POINTER(Trip),
                                   ctypes.c_int]
        cp, li = ctypes.c_char_p, ctypes.c_long
        L.orc_out_diag.argtypes = [cp, ctypes.c_int, li, dp, dp, dp, dp, ctypes.c_double]
        L.orc_out_flow.argtypes = [cp, ctypes.c_int, li, dp, dp, dp, dp]
        L.orc_out_profile.argtypes = [cp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, dp, dp, dp, dp,
                                      ctypes.c_double]
        L.orc_out_f.argtypes = [cp, ctypes.c_int, ctypes.c_int, li, dp]
        _LIB = L
    return _LIB


def _p(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def lattice(q=27, order=ORDER_CUDA, cs_mode=CS_SQRT_RT):
    L = Lattice()
    if lib().orc_lattice_init(ctypes.byref(L), q, order, cs_mode) != 0:
        raise ValueError("bad lattice")
    return L


class Sim:
    """A grid in the reference's own state form (post-stream f + macros)."""

    def __init__(self, nx, ny, nz, q=27, order=ORDER_CUDA, cs_mode=CS_SQRT_RT, tau=0.6,
                 force=(0.0, 0.0, 0.0), les=False, cw=0.5, faces=(0,) * 6, uwall=None, bgk=False):
        P = Params()
        P.nx, P.ny, P.nz = nx, ny, nz
        P.lat = lattice(q, order, cs_mode)
        P.tau = tau
        for i in range(3):
            P.force[i] = force[i]
        P.les = int(bool(les))
        P.bgk = int(bool(bgk))
        P.cw = cw
        for i in range(6):
            P.face[i] = faces[i]
            for a in range(3):
                P.uwall[i][a] = 0.0 if uwall is None else uwall[i][a]
        self.P = P
        self.q = q
        self.shape = (nz, ny, nx)
        n = nx * ny * nz
        self.f = np.zeros((q, nz, ny, nx))
        self.ftmp = np.zeros_like(self.f)
        self.rho = np.ones((nz, ny, nx))
        self.ux = np.zeros((nz, ny, nx))
        self.uy = np.zeros_like(self.ux)
        self.uz = np.zeros_like(self.ux)
        self.taut = np.zeros_like(self.ux)
        self.n = n
        self.trip = None

    def enable_trip(self, trip_steps=50000, istep=0, seed=12345):
        """the channel program's trip forcing for steps < trip_steps, the run
        starting after step istep (the rand() sequence restarts with the run)"""
        T = Trip()
        T.trip_steps = int(trip_steps)
        T.istep = int(istep)
        T.phase = 0.0
        lib().orc_srand(ctypes.byref(T), int(seed))
        self.ffield = np.zeros((3,) + self.shape)
        T.fx, T.fy, T.fz = _p(self.ffield[0]), _p(self.ffield[1]), _p(self.ffield[2])
        self.trip = T

    # -- initial states -------------------------------------------------
    def init_tg_reference(self, U0):
        lib().orc_init_tg_reference(ctypes.byref(self.P), U0, _p(self.f), _p(self.rho), _p(self.ux),
                                    _p(self.uy), _p(self.uz))

    def init_tg_config(self, U0):
        lib().orc_init_tg_config(ctypes.byref(self.P), U0, _p(self.f), _p(self.rho), _p(self.ux),
                                 _p(self.uy), _p(self.uz))

    def init_equilibrium2(self):
        lib().orc_init_equilibrium2(ctypes.byref(self.P), _p(self.f), _p(self.rho), _p(self.ux),
                                    _p(self.uy), _p(self.uz))

    def init_channel_loglaw(self, ustar, ystar):
        lib().orc_init_channel_loglaw(ctypes.byref(self.P), ustar, ystar, _p(self.f), _p(self.rho),
                                      _p(self.ux), _p(self.uy), _p(self.uz))

    def init_channel_config(self, uc, amp, seed):
        lib().orc_init_channel_config(ctypes.byref(self.P), uc, amp, seed, _p(self.f), _p(self.rho),
                                      _p(self.ux), _p(self.uy), _p(self.uz))

    # -- stepping ---------------------------------------------------------
    def _state(self):
        s = _State()
        s.f, s.ftmp, s.rho, s.ux, s.uy, s.uz, s.taut = (
            _p(self.f), _p(self.ftmp), _p(self.rho), _p(self.ux), _p(self.uy), _p(self.uz), _p(self.taut))
        return s

    def run(self, nsteps):
        s = self._state()
        if self.trip is not None:
            lib().orc_run_trip(ctypes.byref(self.P), ctypes.byref(s), ctypes.byref(self.trip), int(nsteps))
        else:
            lib().orc_run(ctypes.byref(self.P), ctypes.byref(s), int(nsteps))
        # the C side swaps f/ftmp each step; follow its pointers
        if ctypes.addressof(s.f.contents) != self.f.ctypes.data:
            self.f, self.ftmp = self.ftmp, self.f

    def collided(self):
        """Post-collision populations of the next step (the product's state)."""
        g = self.f.copy()
        lib().orc_collide_all(ctypes.byref(self.P), _p(g), _p(self.rho), _p(self.ux), _p(self.uy),
                              _p(self.uz), _p(self.taut))
        return g

    def wale(self):
        t = np.zeros_like(self.ux)
        lib().orc_wale(ctypes.byref(self.P), _p(self.ux), _p(self.uy), _p(self.uz), _p(t))
        return t

    def stream_walls(self, fin):
        fout = np.zeros_like(fin)
        lib().orc_stream_walls(ctypes.byref(self.P), _p(np.ascontiguousarray(fin)), _p(fout))
        return fout


def set_threads(n):
    lib().orc_set_threads(int(n))


def tg_reference_params(L=100, q=27):
    """Parameters of Taylor_Green/D3Q27RR.f90:78-87 (U0 = cs/100, Re0 = 200/cs)."""
    cs = 1.0 / math.sqrt(3.0)
    Re0 = 200.0 / cs
    U0 = 1.0 * cs / 100.0
    visc = U0 * L / Re0
    tau = visc / (1.0 / 3.0) + 0.5
    return U0, visc, tau


def write_outputs(directory, istep, rho, ux, uy, uz, taut, f, ustar, ystar):
    """The reference's four writers (output.cu, restated in the oracle) on
    FP64 fields of shape (nz, ny, nx) and f of shape (q, nz, ny, nx), into
    directory; the console line of diag_flow goes to stdout."""
    L = lib()
    d = str(directory).encode()
    nz, ny, nx = rho.shape
    n = rho.size
    a = [np.ascontiguousarray(v, dtype=np.float64) for v in (rho, ux, uy, uz, taut)]
    fa = np.ascontiguousarray(f, dtype=np.float64)
    ok = (L.orc_out_diag(d, int(istep), n, _p(a[0]), _p(a[1]), _p(a[2]), _p(a[3]), float(ustar)) == 0
          and L.orc_out_flow(d, int(istep), n, _p(a[0]), _p(a[1]), _p(a[2]), _p(a[3])) == 0
          and L.orc_out_profile(d, int(istep), nx, ny, nz, _p(a[1]), _p(a[2]), _p(a[3]), _p(a[4]),
                                float(ystar)) == 0
          and L.orc_out_f(d, int(istep), fa.shape[0], n, _p(fa)) == 0)
    if not ok:
        raise OSError(f"cannot write the outputs into {directory}")
