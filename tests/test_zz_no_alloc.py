"""rr_diag_fields_noalloc: diag_flow's domain means for callers that may not
allocate device memory at that point (a server whose HBM budget is handed
out to resident domains, a latency-critical loop that cannot take a
cudaMalloc).  Through the C ABI it must give what rr_diag gives for the same
fields, on two calls in a row (the second call reuses the fixed scratch array
the first one left behind).  Collected last on purpose (file name)."""
import ctypes

import numpy as np
import pytest

import rrlbm
from rrlbm import presets

pytestmark = pytest.mark.gpu


def _dptr(t):
    return ctypes.c_void_p(t.data_ptr())


def test_noalloc_diag_matches_rr_diag_twice():
    import torch

    lib = rrlbm.lib()
    p, st = presets.channel(nx=40, ny=20, nz=12, les=False, variant="config", amp=0.2)
    with rrlbm.Solver(p) as s:
        s.init_state(st["rho"], st["ux"], st["uy"], st["uz"])
        for call in range(2):
            s.step(3 + call)
            ref = s.diag()  # the existing entry point
            fields = {k: torch.empty(p.shape, dtype=torch.float64, device="cuda") for k in ("rho", "ux", "uy", "uz")}
            s.macro_into(fields["rho"], fields["ux"], fields["uy"], fields["uz"])
            out = torch.full((4,), float("nan"), dtype=torch.float64, device="cuda")
            rc = lib.rr_diag_fields_noalloc(_dptr(fields["rho"]), _dptr(fields["ux"]), _dptr(fields["uy"]),
                                            _dptr(fields["uz"]), ctypes.c_size_t(p.n), _dptr(out), None)
            assert rc == 0, lib.rr_last_error().decode()
            torch.cuda.synchronize()
            got = out.cpu().numpy()
            assert np.allclose(got, ref, rtol=1e-13, atol=1e-17), (call, got, ref)


def test_noalloc_diag_rejects_bad_sizes():
    import torch

    lib = rrlbm.lib()
    buf = torch.zeros(8, dtype=torch.float64, device="cuda")
    out = torch.zeros(4, dtype=torch.float64, device="cuda")
    for n in (0, 2**31):
        rc = lib.rr_diag_fields_noalloc(_dptr(buf), _dptr(buf), _dptr(buf), _dptr(buf), ctypes.c_size_t(n),
                                        _dptr(out), None)
        assert rc == 1
        assert "2147483647" in lib.rr_last_error().decode()
