"""Shared helpers of the test suite: oracle twins of solver parameters."""
import numpy as np

from oracle import oracle as O


def oracle_for(p, les=None):
    """An oracle grid with the same physics as rrlbm Params p (internal order:
    CUDA for D3Q27, Fortran for D3Q19)."""
    order = O.ORDER_CUDA if p.q == 27 else O.ORDER_FORTRAN
    return O.Sim(p.lx, p.ly, p.lz, q=p.q, order=order, cs_mode=O.CS_SQRT_RT, tau=p.tau,
                 force=tuple(p.force), les=bool(p.use_les if les is None else les), cw=p.cw,
                 faces=tuple(p.face), uwall=[list(p.uwall[f]) for f in range(6)], bgk=p.collision == 1)


def load_state(o, st):
    """copy a preset start state into an oracle grid"""
    o.rho[...] = st["rho"]
    o.ux[...] = st["ux"]
    o.uy[...] = st["uy"]
    o.uz[...] = st["uz"]
    if st.get("f") is not None:
        o.f[...] = st["f"]
    else:
        o.init_equilibrium2()


def rel_err(a, b, scale):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / scale)
