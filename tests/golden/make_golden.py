"""Regenerates the golden fixtures in this directory.

Run in a checkout that has the reference project next to it
(RR_REFERENCE_DIR, default /root/reference) and a built oracle
(``make -C oracle && oracle/ref_build.sh``).  The fixtures are committed, so
the tests never need the reference itself.

* ``tg27_L100_midline.txt`` -- the reference's own Taylor-Green D3Q27 result
  after 20,000 steps (Taylor_Green/RRBMa0.01L100.txt:3-102): position,
  numerical midline v, analytic v, numerical p.
* ``laminar_uy{5000,10000,60000}.txt`` -- the x-profile (mid y, z=1) of the
  reference's force-driven laminar channel (Laminar/output/uy*.dat, Fortran
  unformatted records of 60x20x2 REAL(8), x fastest).
* ``channel_ref_16x12x8_les{0,1}.npz`` -- rho, ux, uy, uz after 20 steps of
  the reference's CUDA channel kernels run on the host (oracle/_ref), from
  the reference's log-law start with its parameters.h physics.
* ``channel_fdbc_ref_16x12x8_les{0,1}.npz`` -- the same channel with the
  reference's finite-difference wall closure FDBC (BC.cu:129-309) in place of
  RRBC, 20 steps from the log-law start perturbed by fdbc_start(), every wall
  neighbour extrapolated before the closure reads it (ref_step_fdbc).
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = os.environ.get("RR_REFERENCE_DIR", "/root/reference")


def tg():
    src = os.path.join(REF, "Taylor_Green", "RRBMa0.01L100.txt")
    rows = np.loadtxt(src, skiprows=2)
    out = rows[:, [0, 1, 2, 3]]
    np.savetxt(os.path.join(HERE, "tg27_L100_midline.txt"), out,
               fmt=["%d", "%.10f", "%.10f", "%.10f"],
               header="i vnum vtheo pnum  (Taylor_Green/RRBMa0.01L100.txt:3-102)")


def laminar():
    for step in (5000, 10000, 60000):
        raw = open(os.path.join(REF, "Laminar", "output", f"uy{step}.dat"), "rb").read()
        n = int.from_bytes(raw[:4], "little")
        data = np.frombuffer(raw[4:4 + n], dtype="<f8").reshape(2, 20, 60)  # (z, y, x)
        np.savetxt(os.path.join(HERE, f"laminar_uy{step}.txt"), data[0, 10, :], fmt="%.17e",
                   header=f"uy(x, y=11, z=1) of Laminar/output/uy{step}.dat")


def channel():
    sys.path.insert(0, ROOT)
    from oracle import oracle as O
    for les in (0, 1):
        path = os.path.join(ROOT, "oracle", "_ref", f"libref_16x12x8_les{les}.so")
        R = ctypes.CDLL(path)
        for n in ["ref_tau", "ref_force_in_x", "ref_ustar", "ref_ystar"]:
            getattr(R, n).restype = ctypes.c_double
        R.ref_init_constants()
        LX, LY, LZ = R.ref_lx(), R.ref_ly(), R.ref_lz()
        s = O.Sim(LX, LY, LZ, tau=R.ref_tau(), force=(R.ref_force_in_x(), 0, 0), les=bool(les),
                  faces=(0, 0, 1, 1, 0, 0))
        s.init_channel_loglaw(R.ref_ustar(), R.ref_ystar())
        f, rho, ux, uy, uz = s.f.copy(), s.rho.copy(), s.ux.copy(), s.uy.copy(), s.uz.copy()
        ft = np.zeros_like(f)
        fx, fy, fz, taut = (np.zeros_like(rho) for _ in range(4))
        P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
        R.ref_run(20, P(f), P(ft), P(rho), P(ux), P(uy), P(uz), P(fx), P(fy), P(fz), P(taut))
        np.savez_compressed(os.path.join(HERE, f"channel_ref_16x12x8_les{les}.npz"), rho=rho,
                            ux=ux, uy=uy, uz=uz, taut=taut, f_sum=f.sum(axis=0),
                            tau=R.ref_tau(), fx=R.ref_force_in_x(), ustar=R.ref_ustar(),
                            ystar=R.ref_ystar(), steps=20)


def fdbc_start(s, seed=11):
    """the perturbed log-law start of the FDBC fixtures (every population and
    all three velocity components exercised)"""
    rng = np.random.default_rng(seed)
    s.f *= 1.0 + 1e-3 * rng.standard_normal(s.f.shape)
    s.uy += 1e-3 * rng.standard_normal(s.uy.shape)
    s.uz += 1e-3 * rng.standard_normal(s.uz.shape)


def channel_fdbc():
    sys.path.insert(0, ROOT)
    from oracle import oracle as O
    for les in (0, 1):
        path = os.path.join(ROOT, "oracle", "_ref", f"libref_16x12x8_les{les}.so")
        R = ctypes.CDLL(path)
        for n in ["ref_tau", "ref_force_in_x", "ref_ustar", "ref_ystar"]:
            getattr(R, n).restype = ctypes.c_double
        R.ref_init_constants()
        LX, LY, LZ = R.ref_lx(), R.ref_ly(), R.ref_lz()
        s = O.Sim(LX, LY, LZ, tau=R.ref_tau(), force=(R.ref_force_in_x(), 0, 0), les=bool(les),
                  faces=(0, 0, O.FACE_FDBC, O.FACE_FDBC, 0, 0))
        s.init_channel_loglaw(R.ref_ustar(), R.ref_ystar())
        fdbc_start(s)
        f, rho, ux, uy, uz = s.f.copy(), s.rho.copy(), s.ux.copy(), s.uy.copy(), s.uz.copy()
        ft = np.zeros_like(f)
        fx, fy, fz, taut = (np.zeros_like(rho) for _ in range(4))
        P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
        R.ref_run_fdbc(20, P(f), P(ft), P(rho), P(ux), P(uy), P(uz), P(fx), P(fy), P(fz), P(taut))
        np.savez_compressed(os.path.join(HERE, f"channel_fdbc_ref_16x12x8_les{les}.npz"), rho=rho,
                            ux=ux, uy=uy, uz=uz, taut=taut, f_sum=f.sum(axis=0),
                            f_wall=f[:, :, [0, LY - 1], :], tau=R.ref_tau(), fx=R.ref_force_in_x(),
                            ustar=R.ref_ustar(), ystar=R.ref_ystar(), steps=20, seed=11)


if __name__ == "__main__":
    tg()
    laminar()
    channel()
    channel_fdbc()
    print("fixtures written to", HERE)
