"""Seeded synthetic domains of the batched and served forms.

* ensemble(): the multi-domain batch workload -- a seeded mix of fully
  periodic Taylor-Green cubes (32^3-128^3, Ma 0.01-0.1, tau 0.52-0.8) and
  six-wall lid-driven cavities (32^3-96^3, Re 100-1000), FP16 storage.
* request_stream(): the served workload -- Poisson arrivals of Taylor-Green,
  cavity and WALE channel solves, sizes 32^3-192^3 and step counts 1k-20k
  drawn log-uniform, FP16 or FP32 storage.

Initial macroscopic fields are generated on the device (torch), so hundreds
of domains start without host arrays; the solver computes the populations
from them (second-order equilibrium, then the first collision).  The same
fields start a domain's FP64 rerun.
"""
import math
from dataclasses import dataclass, field

import numpy as np

from . import FACE_PERIODIC, FACE_WALL, ORDER_CUDA, STORAGE
from . import params_host_default as params_default

CS = 1.0 / math.sqrt(3.0)
CHANNEL_USTAR = 0.0025  # friction velocity of served channels (centreline ~0.06)
CAVITY_U = 0.1          # lid speed


@dataclass
class Domain:
    kind: str          # "tg", "cavity" or "channel"
    n: int             # cube side
    steps: int
    storage: str = "f16"
    tau: float = 0.6
    Ma: float = 0.0    # Taylor-Green
    Re: float = 0.0    # cavity
    seed: int = 0      # channel noise
    arrival: float = 0.0
    rid: int = 0
    info: dict = field(default_factory=dict)

    @property
    def nodes(self):
        return self.n ** 3


def params_of(d, storage=None):
    """rr_params of a domain (storage overrides the domain's, e.g. for the
    FP64 rerun)."""
    p = params_default()
    p.lx = p.ly = p.lz = d.n
    p.q = 27
    p.order = ORDER_CUDA
    p.storage = STORAGE[storage or d.storage]
    p.force[0] = p.force[1] = p.force[2] = 0.0
    p.use_les = 0
    if d.kind == "tg":
        for f in range(6):
            p.face[f] = FACE_PERIODIC
        p.tau = d.tau
    elif d.kind == "cavity":
        for f in range(6):
            p.face[f] = FACE_WALL
            for a in range(3):
                p.uwall[f][a] = 0.0
        p.uwall[3][0] = CAVITY_U  # lid: the y-hi wall moving in +x
        p.tau = 3.0 * CAVITY_U * d.n / d.Re + 0.5
    elif d.kind == "channel":
        # walls at y = 0, n-1; periodic x, z; WALE; Re_tau = min(180, n)
        for f in range(6):
            p.face[f] = FACE_PERIODIC
        p.face[2] = p.face[3] = FACE_WALL
        for f in (2, 3):
            for a in range(3):
                p.uwall[f][a] = 0.0
        p.use_les = 1
        p.cw = 0.5
        re_tau = min(180.0, float(d.n))
        nu = CHANNEL_USTAR * d.n / (2.0 * re_tau)
        p.tau = 3.0 * nu + 0.5
        p.force[0] = 2.0 * CHANNEL_USTAR ** 2 / d.n
        p.ustar = CHANNEL_USTAR
        p.ystar = nu / CHANNEL_USTAR
    else:
        raise ValueError(d.kind)
    return p


def velocity_scale(d):
    """the velocity an error is quoted against"""
    if d.kind == "tg":
        return d.Ma * CS
    if d.kind == "cavity":
        return CAVITY_U
    return 1.5 * 15.7 * CHANNEL_USTAR


def macros_on_device(d, device="cuda", stream=None):
    """(rho, ux, uy, uz) FP64 tensors of shape (n, n, n) (z, y, x) on the
    device.  With stream (a cudaStream_t handle, e.g. a solver's) that stream
    is made to wait for the fields on the device, and nothing blocks the
    host; without it the fields are complete when this returns.  Either way
    the caller keeps the tensors alive until the stream that reads them has
    passed that point."""
    import torch

    out = _macros(d, device)
    cur = torch.cuda.current_stream(device)
    if stream is None:
        cur.synchronize()
    else:
        torch.cuda.ExternalStream(stream, device=device).wait_stream(cur)
    return out


def _macros(d, device):
    import torch

    n = d.n
    shp = (n, n, n)
    if d.kind == "tg":
        U0 = d.Ma * CS
        x = (torch.arange(n, dtype=torch.float64, device=device) + 0.5) * (2.0 * math.pi / n)
        X = x.view(1, 1, n).expand(shp)
        Y = x.view(1, n, 1).expand(shp)
        ux = (U0 * torch.sin(X) * torch.cos(Y)).contiguous()
        uy = (-U0 * torch.cos(X) * torch.sin(Y)).contiguous()
        uz = torch.zeros(shp, dtype=torch.float64, device=device)
        rho = (1.0 - 0.75 * U0 * U0 * (torch.cos(2.0 * X) + torch.cos(2.0 * Y))).contiguous()
        return rho, ux, uy, uz
    if d.kind == "cavity":
        z = torch.zeros(shp, dtype=torch.float64, device=device)
        return torch.ones(shp, dtype=torch.float64, device=device), z, z.clone(), z.clone()
    # channel: laminar parabola, centreline 1.5 U_b (U_b = 15.7 u*), plus uniform
    # noise of +-10 % of the centreline on all three components
    uc = 1.5 * 15.7 * CHANNEL_USTAR
    y = torch.arange(n, dtype=torch.float64, device=device) + 0.5
    prof = (4.0 * uc * y * (n - y) / (n * n)).view(1, n, 1)
    g = torch.Generator(device=device)
    g.manual_seed(int(d.seed))
    noise = (torch.rand((3,) + shp, generator=g, dtype=torch.float64, device=device) * 2.0 - 1.0) * (0.1 * uc)
    ux = (prof + noise[0]).contiguous()
    uy = noise[1].contiguous()
    uz = noise[2].contiguous()
    return torch.ones(shp, dtype=torch.float64, device=device), ux, uy, uz


def _log_uniform(rng, lo, hi, size=None):
    return np.exp(rng.uniform(math.log(lo), math.log(hi), size))


def ensemble(count=256, seed=4, steps=1000):
    """The multi-domain batch: Taylor-Green cubes and cavities, FP16 storage."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        if rng.random() < 0.5:
            d = Domain("tg", int(round(_log_uniform(rng, 32, 128))), steps, "f16",
                       tau=float(rng.uniform(0.52, 0.8)), Ma=float(_log_uniform(rng, 0.01, 0.1)))
        else:
            d = Domain("cavity", int(round(_log_uniform(rng, 32, 96))), steps, "f16",
                       Re=float(_log_uniform(rng, 100, 1000)))
        d.rid = k
        out.append(d)
    return out


def request_stream(count=64, rate=200.0, seed=5, sizes=(32, 192), steps=(1000, 20000),
                   storages=("f16", "f32"), kinds=("tg", "cavity", "channel")):
    """Poisson arrivals (mean rate req/s) of solves with log-uniform sizes and
    step counts; arrival times in seconds from the start."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for k in range(count):
        t += float(rng.exponential(1.0 / rate))
        kind = kinds[int(rng.integers(len(kinds)))]
        n = int(round(_log_uniform(rng, *sizes)))
        nsteps = int(round(_log_uniform(rng, *steps)))
        storage = storages[int(rng.integers(len(storages)))]
        d = Domain(kind, n, nsteps, storage, arrival=t, rid=k)
        if kind == "tg":
            d.tau = float(rng.uniform(0.52, 0.8))
            d.Ma = float(_log_uniform(rng, 0.01, 0.1))
        elif kind == "cavity":
            d.Re = float(_log_uniform(rng, 100, 1000))
        else:
            d.seed = int(rng.integers(1 << 31))
        out.append(d)
    return out


def solve_alone(d, storage=None, device=0):
    """The domain run by itself (its own rr_step), optionally in another
    storage (the FP64 rerun).  Returns the stepped Solver; the caller closes it."""
    from . import Solver

    s = Solver(params_of(d, storage))
    rho, ux, uy, uz = macros_on_device(d, f"cuda:{device}")
    s.init_state(rho, ux, uy, uz)
    s.sync()  # the upload has read the fields
    s.step(d.steps)
    return s
