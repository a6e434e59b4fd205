"""rrlbm -- Python front end of librrlbm.so (include/rr_api.h).

Mirrors the reference's host interface: the knobs of
RR27V33_code_DNS_LES/parameters.h and globals.cu live in :class:`Params`; a
:class:`Solver` is the state of ``initialize()`` (initial.cu:4-266); ``step``
is one pass of the time loop body (main.cu:360-409); ``output`` writes the
reference's files (output.cu).  Every call goes through the C ABI; there is no
CPU fallback: without the built library or a CUDA device the calls raise.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(_HERE, "librrlbm.so")

STORE_F64, STORE_F32, STORE_F16, STORE_BF16 = 0, 1, 2, 3
STORAGE = {"f64": STORE_F64, "f32": STORE_F32, "f16": STORE_F16, "bf16": STORE_BF16}
FACE_PERIODIC, FACE_WALL, FACE_WALL_BB, FACE_FDBC = 0, 1, 2, 3
COLL_RR, COLL_BGK = 0, 1
ROUND_NEAREST, ROUND_STOCHASTIC = 0, 1
ORDER_CUDA, ORDER_FORTRAN = 0, 1
HOST, DEVICE = 0, 1
OUT_DIAG, OUT_FLOW, OUT_PROFILE, OUT_F = 1, 2, 4, 8

STATUS = {0: "RR_OK", 1: "RR_ERR_INVALID", 2: "RR_ERR_CUDA", 3: "RR_ERR_NOMEM",
          4: "RR_ERR_UNSUPPORTED", 5: "RR_ERR_WATCHDOG", 6: "RR_ERR_IO", 7: "RR_ERR_STATE"}


class RRError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


class Params(ctypes.Structure):
    """rr_params: run-time counterpart of parameters.h:1-25 / globals.cu:18-40."""
    _fields_ = [("lx", ctypes.c_int), ("ly", ctypes.c_int), ("lz", ctypes.c_int),
                ("q", ctypes.c_int), ("use_les", ctypes.c_int), ("tau", ctypes.c_double),
                ("cw", ctypes.c_double), ("force", ctypes.c_double * 3),
                ("face", ctypes.c_int * 6), ("uwall", (ctypes.c_double * 3) * 6),
                ("storage", ctypes.c_int), ("order", ctypes.c_int), ("device", ctypes.c_int),
                ("ustar", ctypes.c_double), ("ystar", ctypes.c_double), ("rounding", ctypes.c_int), ("trip_steps", ctypes.c_int), ("collision", ctypes.c_int)]

    @property
    def n(self):
        return self.lx * self.ly * self.lz

    @property
    def shape(self):
        return (self.lz, self.ly, self.lx)


_LIB = None


def lib():
    """The loaded C library (raises if it was not built)."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIBPATH):
            raise RuntimeError(f"{LIBPATH} missing: build it with rrlbm/build.py (nvcc, sm_103a)")
        L = ctypes.CDLL(LIBPATH)
        vp, dp, P = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(Params)
        sig = {
            "rr_params_default": ([P], ctypes.c_int),
            "rr_create": ([P, ctypes.POINTER(vp)], ctypes.c_int),
            "rr_destroy": ([vp], ctypes.c_int),
            "rr_init_state": ([vp, vp, vp, vp, vp, vp, ctypes.c_int], ctypes.c_int),
            "rr_step": ([vp, ctypes.c_int], ctypes.c_int),
            "rr_sync": ([vp], ctypes.c_int),
            "rr_query": ([vp, ctypes.POINTER(ctypes.c_int)], ctypes.c_int),
            "rr_get_istep": ([vp], ctypes.c_longlong),
            "rr_get_stream": ([vp], ctypes.c_void_p),
            "rr_macro": ([vp, vp, vp, vp, vp, vp, ctypes.c_int], ctypes.c_int),
            "rr_get_f": ([vp, vp, ctypes.c_int], ctypes.c_int),
            "rr_diag": ([vp, dp], ctypes.c_int),
            "rr_diag_fields_noalloc": ([vp, vp, vp, vp, ctypes.c_size_t, vp, vp], ctypes.c_int),
            "rr_profile": ([vp, dp], ctypes.c_int),
            "rr_accumulate": ([vp], ctypes.c_int),
            "rr_get_accum": ([vp, dp, ctypes.POINTER(ctypes.c_longlong)], ctypes.c_int),
            "rr_output": ([vp, ctypes.c_uint, ctypes.c_char_p], ctypes.c_int),
            "rr_save": ([vp, ctypes.c_char_p], ctypes.c_int),
            "rr_get_force": ([vp, vp, ctypes.c_int], ctypes.c_int),
            "rr_load": ([vp, ctypes.c_char_p, ctypes.c_longlong], ctypes.c_int),
            "rr_device_bytes": ([vp], ctypes.c_size_t),
            "rr_bytes_for": ([P], ctypes.c_size_t),
            "rr_last_error": ([], ctypes.c_char_p),
            "rr_batch_create": ([ctypes.c_int, ctypes.POINTER(vp)], ctypes.c_int),
            "rr_batch_destroy": ([vp], ctypes.c_int),
            "rr_batch_add": ([vp, vp], ctypes.c_int),
            "rr_batch_remove": ([vp, vp], ctypes.c_int),
            "rr_batch_size": ([vp], ctypes.c_int),
            "rr_batch_step": ([vp, ctypes.c_int], ctypes.c_int),
            "rr_batch_sync": ([vp], ctypes.c_int),
            "rr_batch_get_stream": ([vp], ctypes.c_void_p),
            "rr_batch_set_launch": ([vp, ctypes.c_int, ctypes.c_int, ctypes.c_int], ctypes.c_int),
            "rr_batch_get_launch": ([vp, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                     ctypes.POINTER(ctypes.c_int)], ctypes.c_int),
            "rr_batch_set_grouping": ([vp, ctypes.c_size_t], ctypes.c_int),
            "rr_batch_set_mode": ([vp, ctypes.c_int, ctypes.c_int], ctypes.c_int),
            "rr_batch_get_mode": ([vp, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)], ctypes.c_int),
            "rr_batch_get_grouping": ([vp], ctypes.c_size_t),
            "rr_tune": ([vp, ctypes.c_int, ctypes.POINTER(ctypes.c_longlong)], ctypes.c_int),
            "rr_set_stage": ([vp, ctypes.c_int, ctypes.c_int, ctypes.c_int], ctypes.c_int),
            "rr_get_stage": ([vp, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                              ctypes.POINTER(ctypes.c_int)], ctypes.c_int),
            "rr_batch_tune": ([vp, ctypes.c_int, ctypes.POINTER(ctypes.c_longlong)], ctypes.c_int),
            "rr_set_wait_limit": ([vp, ctypes.c_longlong], ctypes.c_int),
            "rr_get_wait_limit": ([vp], ctypes.c_longlong),
            "rr_get_launch": ([vp, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                               ctypes.POINTER(ctypes.c_int)], ctypes.c_int),
            "rr_set_launch": ([vp, ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)],
                              ctypes.c_int),
        }
        for name, (args, res) in sig.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _LIB = L
    return _LIB


def _check(code):
    if code != 0:
        raise RRError(code, lib().rr_last_error().decode())


def params_default():
    """parameters.h + globals.cu defaults (64^3 Re_tau=180 channel, DNS, FP64)."""
    p = Params()
    _check(lib().rr_params_default(ctypes.byref(p)))
    return p


def params_host_default():
    """The same defaults as rr_params_default, filled in on the host without
    loading the CUDA library (the presets use it, so that CPU-only callers
    of the workload definitions never map librrlbm.so): parameters.h:9-11
    (64^3) and globals.cu:33-38 (Re_tau = 180, nu = 0.000622,
    u* = 2 Re_tau nu / LY, tau = 3 nu + 0.5, F_x = 2 u*^2 / LY), walls at
    y = 0 and y = LY-1, D3Q27, FP64, CUDA order, stochastic rounding."""
    p = Params()
    p.lx = p.ly = p.lz = 64
    p.q = 27
    p.use_les = 0
    Re, visc = 180.0, 0.000622
    u0 = 2.0 * Re * visc / p.ly
    p.tau = 3.0 * visc + 0.5
    p.cw = 0.5
    p.force[0] = 2.0 * u0 * u0 / p.ly
    p.face[2] = p.face[3] = FACE_WALL
    p.storage = STORE_F64
    p.order = ORDER_CUDA
    p.device = 0
    p.ustar = u0
    p.ystar = visc / u0
    p.rounding = ROUND_STOCHASTIC
    return p


def bytes_for(p):
    return lib().rr_bytes_for(ctypes.byref(p))


def _ptr(a):
    """(pointer, where) of a numpy array or a CUDA tensor (torch / __cuda_array_interface__)."""
    if a is None:
        return None, HOST
    if isinstance(a, np.ndarray):
        if a.dtype != np.float64 or not a.flags.c_contiguous:
            raise ValueError("arrays crossing the API are C-contiguous float64")
        return a.ctypes.data, HOST
    cai = getattr(a, "__cuda_array_interface__", None)
    if cai is not None:
        if cai["typestr"] != "<f8":
            raise ValueError("device arrays crossing the API are float64")
        return cai["data"][0], DEVICE
    raise TypeError(f"unsupported array type {type(a)}")


class Solver:
    """One domain resident in HBM (rr_solver)."""

    def __init__(self, params):
        self.p = params
        h = ctypes.c_void_p()
        _check(lib().rr_create(ctypes.byref(params), ctypes.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            lib().rr_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- state ---------------------------------------------------------------
    def init_state(self, rho, ux, uy, uz, f=None):
        """initialize(): post-stream populations f (q x N, or None for the
        second-order equilibrium) and the macros the first collision uses."""
        ptrs = [_ptr(a) for a in (f, rho, ux, uy, uz)]
        where = ptrs[1][1]
        if any(w != where for p_, w in ptrs if p_ is not None):
            raise ValueError("all arrays on the host or all on the device")
        _check(lib().rr_init_state(self._h, *[p_ for p_, _ in ptrs], where))

    def step(self, n=1):
        _check(lib().rr_step(self._h, int(n)))

    def sync(self):
        _check(lib().rr_sync(self._h))

    def busy(self):
        """work still in flight on the solver's stream (does not wait)"""
        b = ctypes.c_int(0)
        _check(lib().rr_query(self._h, ctypes.byref(b)))
        return bool(b.value)

    @property
    def istep(self):
        return lib().rr_get_istep(self._h)

    @property
    def stream(self):
        """the solver's cudaStream_t as an integer handle"""
        return lib().rr_get_stream(self._h) or 0

    @property
    def device_bytes(self):
        return lib().rr_device_bytes(self._h)

    # -- readouts --------------------------------------------------------------
    def macro(self, taut=False):
        shp = self.p.shape
        out = {k: np.empty(shp) for k in ("rho", "ux", "uy", "uz")}
        if taut:
            out["taut"] = np.empty(shp)
        args = [out[k].ctypes.data if k in out else None for k in ("rho", "ux", "uy", "uz", "taut")]
        _check(lib().rr_macro(self._h, *args, HOST))
        return out

    def macro_into(self, rho, ux, uy, uz, taut=None):
        ptrs = [_ptr(a) for a in (rho, ux, uy, uz, taut)]
        where = ptrs[0][1]
        _check(lib().rr_macro(self._h, *[p_ for p_, _ in ptrs], where))

    def get_force(self):
        """the body force (fx, fy, fz fields) of the step the readouts show"""
        out = np.empty((3,) + self.p.shape)
        _check(lib().rr_get_force(self._h, out.ctypes.data, HOST))
        return out

    def get_f(self):
        f = np.empty((self.p.q,) + self.p.shape)
        _check(lib().rr_get_f(self._h, f.ctypes.data, HOST))
        return f

    def diag(self):
        out = (ctypes.c_double * 4)()
        _check(lib().rr_diag(self._h, out))
        return np.array(out[:])

    def profile(self):
        ly = self.p.ly
        out = np.empty(12 * ly)
        _check(lib().rr_profile(self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        return out[: 11 * ly].reshape(ly, 11), out[11 * ly:]

    def accumulate(self):
        _check(lib().rr_accumulate(self._h))

    def get_accum(self):
        ly = self.p.ly
        out = np.empty(12 * ly)
        n = ctypes.c_longlong()
        _check(lib().rr_get_accum(self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                  ctypes.byref(n)))
        return out[: 11 * ly].reshape(ly, 11), out[11 * ly:], n.value

    # -- files -------------------------------------------------------------------
    def output(self, what, directory="data"):
        _check(lib().rr_output(self._h, int(what), directory.encode()))

    def save(self, directory):
        _check(lib().rr_save(self._h, directory.encode()))

    def load(self, directory, istep):
        _check(lib().rr_load(self._h, directory.encode(), int(istep)))

    # -- launch shapes -------------------------------------------------------------
    def tune(self, trial_steps=8):
        """Autotune the launch shapes on real steps; returns the steps it ran."""
        run = ctypes.c_longlong(0)
        _check(lib().rr_tune(self._h, int(trial_steps), ctypes.byref(run)))
        return run.value

    def launch(self):
        """(rows per work-item group, WALE method (0 fused, 1 two-pass), WALE tile (tx, ty, z chunk))."""
        rg, m, t = ctypes.c_int(0), ctypes.c_int(0), (ctypes.c_int * 3)()
        _check(lib().rr_get_launch(self._h, ctypes.byref(rg), ctypes.byref(m), t))
        return rg.value, m.value, tuple(t)

    def stage(self):
        """(DNS method: 0 tile, 1 staged; rows per staged block; pipeline stages)"""
        m, r, n = ctypes.c_int(0), ctypes.c_int(0), ctypes.c_int(0)
        _check(lib().rr_get_stage(self._h, ctypes.byref(m), ctypes.byref(r), ctypes.byref(n)))
        return m.value, r.value, n.value

    def set_stage(self, method, rows=None, stages=None):
        _, r, n = self.stage()
        _check(lib().rr_set_stage(self._h, int(method), int(rows or r), int(stages or n)))

    def set_wait_limit(self, polls):
        """polls before a wait of the staged step's pipeline gives up (< 0: the default)"""
        _check(lib().rr_set_wait_limit(self._h, int(polls)))

    @property
    def wait_limit(self):
        return lib().rr_get_wait_limit(self._h)

    def set_launch(self, rows_group, les_method=None, les_tile=None):
        m = None if les_method is None else ctypes.byref(ctypes.c_int(int(les_method)))
        t = None if les_tile is None else (ctypes.c_int * 3)(*les_tile)
        _check(lib().rr_set_launch(self._h, int(rows_group), m, t))


class Batch:
    """Many solvers advanced together (rr_batch): one persistent launch per step."""

    def __init__(self, device=0):
        h = ctypes.c_void_p()
        _check(lib().rr_batch_create(int(device), ctypes.byref(h)))
        self._h = h
        self._members = []

    def close(self):
        if self._h:
            lib().rr_batch_destroy(self._h)
            self._h = None
            self._members = []

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __len__(self):
        return lib().rr_batch_size(self._h)

    def add(self, solver):
        _check(lib().rr_batch_add(self._h, solver._h))
        self._members.append(solver)

    def remove(self, solver):
        _check(lib().rr_batch_remove(self._h, solver._h))
        self._members.remove(solver)

    def step(self, n=1):
        _check(lib().rr_batch_step(self._h, int(n)))

    def sync(self):
        _check(lib().rr_batch_sync(self._h))

    @property
    def stream(self):
        return lib().rr_batch_get_stream(self._h) or 0

    def set_launch(self, block, ctas_per_sm=0, order=0):
        """order: 0 strided walk, 1 contiguous chunks"""
        _check(lib().rr_batch_set_launch(self._h, int(block), int(ctas_per_sm), int(order)))

    def launch(self):
        b, c, o = ctypes.c_int(0), ctypes.c_int(0), ctypes.c_int(0)
        _check(lib().rr_batch_get_launch(self._h, ctypes.byref(b), ctypes.byref(c), ctypes.byref(o)))
        return b.value, c.value, o.value

    def tune(self, trial_steps=8):
        run = ctypes.c_longlong(0)
        _check(lib().rr_batch_tune(self._h, int(trial_steps), ctypes.byref(run)))
        return run.value

    def set_mode(self, mode, chains=8):
        """mode: 0 persistent kernel, 1 fan-out of the members' own launches over parallel chains"""
        _check(lib().rr_batch_set_mode(self._h, int(mode), int(chains)))

    def mode(self):
        m, c = ctypes.c_int(0), ctypes.c_int(0)
        _check(lib().rr_batch_get_mode(self._h, ctypes.byref(m), ctypes.byref(c)))
        return m.value, c.value

    @property
    def grouping(self):
        """bytes up to which small members are grouped for L2 reuse (0: off)"""
        return lib().rr_batch_get_grouping(self._h)

    @grouping.setter
    def grouping(self, nbytes):
        _check(lib().rr_batch_set_grouping(self._h, int(nbytes)))


from . import presets  # noqa: E402,F401
