"""Parameter sets and initial states of the reference programs and of the
benchmark workloads (host-side numpy; the solver itself runs on the GPU).

* Taylor-Green vortex: Taylor_Green/D3Q27RR.f90 (and D3Q19RR.f90), start
  134-264: analytic cell-centred fields, f = feq + fneq with the
  non-equilibrium moments from 4th-order finite differences of u, v.
* Lid-driven cavity: Cavity/*.f90 (rest start, Cavity/main.f90:16-21).
* Channel: RR27V33_code_DNS_LES (init_arrays, initial.cu:268-326), and the
  laminar-parabola-plus-noise start of the 384x192x128 workload.
"""
import math

import numpy as np

from . import (FACE_PERIODIC, FACE_WALL, ORDER_CUDA, ORDER_FORTRAN, STORAGE)
from . import params_host_default as params_default

# D3Q27 in the CUDA order (initial.cu:67-69), D3Q19 in the Fortran order
# (Taylor_Green/D3Q19RR.f90:75-77); the solver's internal orders
C27 = np.array([[0, 1, 0, -1, 0, 0, 0, 1, -1, -1, 1, 1, 0, -1, 0, 1, 0, -1, 0, 1, -1, -1, 1, 1, -1, -1, 1],
                [0, 0, 1, 0, -1, 0, 0, 1, 1, -1, -1, 0, 1, 0, -1, 0, 1, 0, -1, 1, 1, -1, -1, 1, 1, -1, -1],
                [0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, 1, 1, -1, -1, -1, -1, 1, 1, 1, 1, -1, -1, -1, -1]]).T
C19 = np.array([[0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1, 0, 0, 0, 0],
                [0, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1],
                [0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1]]).T
# Fortran D3Q27 order (D3Q27RR.f90:69-71): internal (CUDA) index of Fortran population j
FORTRAN_TO_CUDA_27 = [0, 1, 3, 2, 4, 5, 6, 7, 10, 8, 9, 11, 15, 13, 17, 12, 16, 14, 18, 19, 23, 22,
                      26, 20, 24, 21, 25]


def lattice(q):
    c = C27 if q == 27 else C19
    n = np.abs(c).sum(axis=1)
    if q == 27:
        w = np.choose(n, [8 / 27, 2 / 27, 1 / 54, 1 / 216])
    else:
        w = np.choose(n, [1 / 3, 1 / 18, 1 / 36])
    return c.astype(np.float64), w


def hermite(q):
    """Hermite tables H_k(c_i) of initial.cu:92-110 (cs^2 = 1/3)."""
    c, w = lattice(q)
    cs = math.sqrt(1.0 / 3.0)
    x, y, z = c[:, 0], c[:, 1], c[:, 2]
    H = {
        "100": x / cs, "010": y / cs, "001": z / cs,
        "110": 3 * x * y, "101": 3 * x * z, "011": 3 * y * z,
        "200": 3 * x * x - 1, "020": 3 * y * y - 1, "002": 3 * z * z - 1,
        "210": (x * x * y) / cs**3 - y / cs, "201": (x * x * z) / cs**3 - z / cs,
        "021": (y * y * z) / cs**3 - z / cs, "120": (y * y * x) / cs**3 - x / cs,
        "012": (z * z * y) / cs**3 - y / cs, "102": (z * z * x) / cs**3 - x / cs,
        "111": (x * y * z) / cs**3,
    }
    return c, w, H, cs


def _thir(q, H, a):
    """third-order projection; D3Q19 uses the admissible combinations of
    Taylor_Green/D3Q19RR.f90:373-378"""
    if q == 27:
        return (H["210"] * a["210"] + H["201"] * a["201"] + H["021"] * a["021"] + H["120"] * a["120"]
                + H["012"] * a["012"] + H["102"] * a["102"] + 2.0 * H["111"] * a["111"])
    p = lambda k1, k2: (H[k1] + H[k2]) * (a[k1] + a[k2]) + (H[k1] - H[k2]) * (a[k1] - a[k2]) / 3.0
    return p("210", "012") + p("102", "120") + p("021", "201")


def _expand(v):
    return v[None, ...]


def feq_rr(q, rho, ux, uy, uz):
    """3rd-order Hermite equilibrium (collision.cu:41-69), shape (q,) + field shape"""
    c, w, H, cs = hermite(q)
    sh = (q,) + (1,) * rho.ndim
    Hs = {k: v.reshape(sh) for k, v in H.items()}
    uu, vv, ww = _expand(ux / cs), _expand(uy / cs), _expand(uz / cs)
    a = {"110": uu * vv, "101": uu * ww, "011": vv * ww, "200": uu * uu, "020": vv * vv, "002": ww * ww}
    a.update({"210": a["200"] * vv, "201": a["200"] * ww, "120": a["020"] * uu, "021": a["020"] * ww,
              "012": a["002"] * vv, "102": a["002"] * uu, "111": a["110"] * ww})
    fir = Hs["100"] * uu + Hs["010"] * vv + Hs["001"] * ww
    sec = 2.0 * (Hs["110"] * a["110"] + Hs["101"] * a["101"] + Hs["011"] * a["011"]) \
        + Hs["200"] * a["200"] + Hs["020"] * a["020"] + Hs["002"] * a["002"]
    thir = _thir(q, Hs, a)
    return w.reshape(sh) * _expand(rho) * (1.0 + fir + 0.5 * (sec + thir))


def fneq_rr(q, ane2, ux, uy, uz):
    """fneqRR from the six second-order non-equilibrium coefficients with the
    recursive third order (collision.cu:88-115)"""
    c, w, H, cs = hermite(q)
    sh = (q,) + (1,) * ux.ndim
    Hs = {k: v.reshape(sh) for k, v in H.items()}
    uu, vv, ww = ux / cs, uy / cs, uz / cs
    n = dict(ane2)
    n3 = {"210": n["200"] * vv + 2.0 * uu * n["110"], "201": n["200"] * ww + 2.0 * uu * n["101"],
          "120": n["020"] * uu + 2.0 * vv * n["110"], "021": n["020"] * ww + 2.0 * vv * n["011"],
          "102": n["002"] * uu + 2.0 * ww * n["101"], "012": n["002"] * vv + 2.0 * ww * n["011"],
          "111": n["110"] * ww + n["101"] * vv + n["011"] * uu}
    e = {k: _expand(v) for k, v in list(n.items()) + list(n3.items())}
    sec = 2.0 * (Hs["110"] * e["110"] + Hs["101"] * e["101"] + Hs["011"] * e["011"]) \
        + Hs["200"] * e["200"] + Hs["020"] * e["020"] + Hs["002"] * e["002"]
    thir = _thir(q, Hs, e)
    return w.reshape(sh) * (0.5 * (sec + thir))


def _fd4(u, axis):
    """4th-order periodic first derivative of D3Q27RR.f90:198-201"""
    return -(np.roll(u, -2, axis) - 8.0 * np.roll(u, -1, axis) + 8.0 * np.roll(u, 1, axis)
             - np.roll(u, 2, axis)) / 12.0


def tg_state(q, nx, ny, nz, tau, U0, variant):
    """Taylor-Green start: analytic fields + feq + FD-strain fneq."""
    if variant == "reference":
        # D3Q27RR.f90:134-146, k_val = 2, cell centres i - 0.5 (1-based)
        x = np.arange(1, nx + 1) - 0.5
        y = np.arange(1, ny + 1) - 0.5
        X, Y = np.meshgrid(x, y, indexing="xy")
        L, kv = float(nx), 2.0
        u = -U0 * np.cos(kv * math.pi * X / L) * np.sin(kv * math.pi * Y / L)
        v = U0 * np.cos(kv * math.pi * Y / L) * np.sin(kv * math.pi * X / L)
        r = 1.0 - U0 * U0 / 2 * np.cos(kv * math.pi / L * (X - Y)) * np.cos(kv * math.pi / L * (X + Y)) / (1.0 / 3.0)
    else:
        # 2x2 vortices on x = ix + 0.5: u = U0 sin cos, v = -U0 cos sin,
        # rho = 1 + 3 p', p' = -(U0^2/4)(cos 4 pi x/L + cos 4 pi y/L)
        x = np.arange(nx) + 0.5
        y = np.arange(ny) + 0.5
        X, Y = np.meshgrid(x, y, indexing="xy")
        L = float(nx)
        u = U0 * np.sin(2 * math.pi * X / L) * np.cos(2 * math.pi * Y / L)
        v = -U0 * np.cos(2 * math.pi * X / L) * np.sin(2 * math.pi * Y / L)
        r = 1.0 + 3.0 * (-(U0 * U0 / 4.0) * (np.cos(4 * math.pi * X / L) + np.cos(4 * math.pi * Y / L)))
    shp = (nz, ny, nx)
    rho = np.broadcast_to(r, shp).copy()
    ux = np.broadcast_to(u, shp).copy()
    uy = np.broadcast_to(v, shp).copy()
    uz = np.zeros(shp)
    dudx, dudy = _fd4(ux, 2), _fd4(ux, 1)
    dvdx, dvdy = _fd4(uy, 2), _fd4(uy, 1)
    z = np.zeros(shp)
    ane2 = {"110": -tau * rho * (dudy + dvdx), "101": z, "011": z,
            "200": -tau * rho * 2.0 * dudx, "020": -tau * rho * 2.0 * dvdy, "002": z}
    f = feq_rr(q, rho, ux, uy, uz) + fneq_rr(q, ane2, ux, uy, uz)
    return {"f": np.ascontiguousarray(f), "rho": rho, "ux": ux, "uy": uy, "uz": uz}


def taylor_green(L=100, nz=4, tau=0.6, Ma=0.01, q=27, storage="f64", variant="config"):
    """Quasi-2D Taylor-Green vortex, fully periodic.  variant="reference"
    reproduces Taylor_Green/D3Q27RR.f90 (L=100, LZ=2, tau=0.505, U0=cs/100)."""
    p = params_default()
    p.lx, p.ly, p.lz = L, L, nz
    p.q = q
    p.order = ORDER_CUDA if q == 27 else ORDER_FORTRAN
    p.storage = STORAGE[storage]
    for f in range(6):
        p.face[f] = FACE_PERIODIC
    p.force[0] = p.force[1] = p.force[2] = 0.0
    cs = 1.0 / math.sqrt(3.0)
    U0 = Ma * cs
    if variant == "reference":
        Re0 = 200.0 / cs
        U0 = 1.0 * cs / 100.0
        visc = U0 * L / Re0
        tau = visc / (1.0 / 3.0) + 0.5
    p.tau = tau
    st = tg_state(q, L, L, nz, tau, U0, variant)
    st["U0"] = U0
    st["nu"] = (tau - 0.5) / 3.0
    return p, st


def cavity(n=128, Re=1000.0, U=0.1, q=27, storage="f64", variant="config"):
    """Lid-driven cavity.  variant="config": n^3 box, walls on all six faces,
    the lid is the y-hi wall moving in +x.  variant="reference": the
    quasi-2D Cavity/*.f90 box n x n x 2, walls at x=1, x=lx (the lid, moving
    +y), y=1, y=ly, periodic z.  nu = U n / Re, tau = 3 nu + 0.5
    (Cavity/para.f90:114-116)."""
    p = params_default()
    p.q = q
    p.order = ORDER_CUDA if q == 27 else ORDER_FORTRAN
    p.storage = STORAGE[storage]
    p.force[0] = p.force[1] = p.force[2] = 0.0
    visc = U * float(n) / Re
    p.tau = 3.0 * visc + 0.5
    for f in range(6):
        p.face[f] = FACE_WALL
        for a in range(3):
            p.uwall[f][a] = 0.0
    if variant == "reference":
        p.lx, p.ly, p.lz = n, n, 2
        p.face[4] = p.face[5] = FACE_PERIODIC
        p.uwall[1][1] = U
    else:
        p.lx = p.ly = p.lz = n
        p.uwall[3][0] = U
    shp = (p.lz, p.ly, p.lx)
    st = {"f": None, "rho": np.ones(shp), "ux": np.zeros(shp), "uy": np.zeros(shp), "uz": np.zeros(shp),
          "nu": visc, "U": U}
    return p, st


def laminar(storage="f64", q=27):
    """The force-driven laminar channel of Laminar/*.f90: 60 x 20 x 2 nodes,
    walls (bounce-back + regularized closure) at x = 1 and x = lx, periodic y
    and z, body force in +y.  Rstar = 50, ustar = 0.05, nu = ustar nx / Rstar,
    tau = 3 nu + 0.5, F_y = 8 nu ustar / nx^2 (Laminar/para.f90:33-39).  The
    start is the rest equilibrium (initpop with u = 0) with the stored
    velocity of the first macrovar, u_y = F_y / 2 (Laminar/main.f90:38-51),
    which the first collision uses."""
    nx, ny, nz = 60, 20, 2
    Rstar, ustar = 50.0, 0.05
    visc = ustar * nx / Rstar
    p = params_default()
    p.lx, p.ly, p.lz = nx, ny, nz
    p.q = q
    p.order = ORDER_CUDA if q == 27 else ORDER_FORTRAN
    p.storage = STORAGE[storage]
    p.use_les = 0
    p.tau = 3.0 * visc + 0.5
    p.force[0] = p.force[2] = 0.0
    p.force[1] = 8.0 * visc * ustar / nx / nx
    for f in range(6):
        p.face[f] = FACE_PERIODIC
        for a in range(3):
            p.uwall[f][a] = 0.0
    p.face[0] = p.face[1] = FACE_WALL
    shp = (nz, ny, nx)
    _, w = lattice(q)
    f0 = np.ascontiguousarray(np.broadcast_to(w[:, None, None, None], (q,) + shp))
    st = {"f": f0, "rho": np.ones(shp), "ux": np.zeros(shp), "uy": np.full(shp, 0.5 * p.force[1]),
          "uz": np.zeros(shp), "ustar": ustar, "nu": visc}
    return p, st


def splitmix64(x):
    x = (x + np.uint64(0x9E3779B97F4A7C15)) & np.uint64(0xFFFFFFFFFFFFFFFF)
    x = ((x ^ (x >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & np.uint64(0xFFFFFFFFFFFFFFFF)
    x = ((x ^ (x >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & np.uint64(0xFFFFFFFFFFFFFFFF)
    return x ^ (x >> np.uint64(31))


def uniform_pm1(seed, node, comp):
    """counter-based U(-1, 1) keyed by (seed, node, component)"""
    with np.errstate(over="ignore"):
        h = splitmix64(np.uint64(seed) ^ splitmix64(node.astype(np.uint64) * np.uint64(4) + np.uint64(comp)))
    r = (h >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
    return 2.0 * r - 1.0


def channel(nx=384, ny=192, nz=128, Re_tau=180.0, nu=0.000622, les=True, q=27, storage="f64",
            variant="config", amp=0.1, seed=2024):
    """Force-driven channel, walls at y = 0 and y = ny-1, periodic x and z
    (RR27V33_code_DNS_LES).  u* = 2 Re_tau nu / ny, F_x = 2 u*^2 / ny,
    tau = 3 nu + 0.5 (globals.cu:33-38).  variant="config": laminar parabola
    with centreline 1.5 U_b (U_b = 15.7 u*) plus amp * U_c uniform noise on all
    three components, f = second-order equilibrium.  variant="reference":
    the log-law start of init_arrays (initial.cu:268-326)."""
    p = params_default()
    p.lx, p.ly, p.lz = nx, ny, nz
    p.q = q
    p.order = ORDER_CUDA if q == 27 else ORDER_FORTRAN
    p.storage = STORAGE[storage]
    p.use_les = int(bool(les))
    ustar = 2.0 * Re_tau * nu / ny
    p.tau = 3.0 * nu + 0.5
    p.force[0] = 2.0 * ustar * ustar / ny
    p.force[1] = p.force[2] = 0.0
    p.ustar = ustar
    p.ystar = nu / ustar
    shp = (nz, ny, nx)
    if variant == "reference":
        LX, LY, LZ = nx, ny, nz
        pi2 = 2.0 * math.acos(-1.0)
        iz, iy, ix = np.meshgrid(np.arange(LZ), np.arange(LY), np.arange(LX), indexing="ij")
        A9, alpha, beta9, cc = 0.1 * math.sqrt(2.0), 1.0, 1.0, 60.0
        ccc1 = -LX / pi2 / alpha / p.ystar * A9 * ustar / cc / cc
        z9 = pi2 * (iz + 0.5) / LZ
        x9 = pi2 * (ix + 0.5) / LX
        yplus = np.where(iy <= LY // 2, (iy + 0.5) / p.ystar, (LY - iy - 0.5) / p.ystar)
        with np.errstate(divide="ignore"):
            u = np.where(yplus <= 10.8, ustar * yplus, (np.log10(yplus) / 0.41 + 5.0) * ustar)
        ux = u + ccc1 * yplus * np.sin(alpha * x9 + beta9 * z9)
        rho = np.ones(shp)
        c, w = lattice(q)
        feq = w[:, None, None, None] * np.ones((1,) + shp)
        f = feq - 0.5 * p.force[0] * c[:, 0][:, None, None, None] / (1.0 / 3.0) * feq
        st = {"f": np.ascontiguousarray(f), "rho": rho, "ux": ux, "uy": np.zeros(shp), "uz": np.zeros(shp)}
    else:
        Ub = 15.7 * ustar
        uc = 1.5 * Ub
        y = np.arange(ny) + 0.5
        prof = 4.0 * uc * y * (ny - y) / (ny * ny)
        idx = np.arange(nx * ny * nz, dtype=np.uint64).reshape(shp)
        ux = prof[None, :, None] + amp * uc * uniform_pm1(seed, idx, 0)
        uy = amp * uc * uniform_pm1(seed, idx, 1)
        uz = amp * uc * uniform_pm1(seed, idx, 2)
        st = {"f": None, "rho": np.ones(shp), "ux": ux, "uy": uy, "uz": uz, "uc": uc, "Ub": Ub}
    st["ustar"] = ustar
    st["nu"] = nu
    return p, st
