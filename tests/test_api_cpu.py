"""The C ABI library without a GPU: it loads, exports every function that
include/rr_api.h declares, validates parameters before touching CUDA, and the
host-side start states match the oracle's."""
import ctypes
import os
import re

import numpy as np
import pytest

import rrlbm
from rrlbm import presets
from conftest import ROOT
from helpers import oracle_for


def _declared():
    src = open(os.path.join(ROOT, "include", "rr_api.h")).read()
    return sorted(set(re.findall(r"^\s*(?:rr_status|size_t|long long|const char \*|void \*)\s*(rr_\w+)\(",
                                 src, re.M)))


def test_library_exports_every_declared_symbol():
    names = _declared()
    assert len(names) >= 19
    L = rrlbm.lib()
    for n in names:
        assert hasattr(L, n), n


def test_defaults_follow_parameters_h():
    p = rrlbm.params_default()
    assert (p.lx, p.ly, p.lz, p.q, p.use_les) == (64, 64, 64, 27, 0)
    visc = 0.000622
    u0 = 2.0 * 180.0 * visc / 64
    assert p.tau == 3.0 * visc + 0.5
    assert p.force[0] == 2.0 * u0 * u0 / 64
    assert list(p.face) == [0, 0, 1, 1, 0, 0]


def test_host_defaults_equal_the_library_defaults():
    """the presets' host-side defaults are rr_params_default byte for byte"""
    a, b = rrlbm.params_default(), rrlbm.params_host_default()
    assert bytes(a) == bytes(b)


@pytest.mark.parametrize("field,value,msg", [
    ("q", 15, "q = 15"), ("tau", 0.5, "tau"), ("lx", 0, "grid"), ("storage", 9, "storage"),
])
def test_invalid_params_rejected_before_cuda(field, value, msg):
    p = rrlbm.params_default()
    setattr(p, field, value)
    with pytest.raises(rrlbm.RRError) as e:
        rrlbm.Solver(p)
    assert e.value.code == 1 and msg in str(e.value)


def test_invalid_faces_rejected():
    p = rrlbm.params_default()
    p.face[0] = rrlbm.FACE_WALL  # x-lo wall with periodic x-hi
    with pytest.raises(rrlbm.RRError) as e:
        rrlbm.Solver(p)
    assert "periodic on both faces" in str(e.value)
    p = rrlbm.params_default()
    p.uwall[0][1] = 0.1  # velocity on a periodic face
    with pytest.raises(rrlbm.RRError):
        rrlbm.Solver(p)
    p = rrlbm.params_default()
    p.q = 19
    p.order = rrlbm.ORDER_CUDA
    with pytest.raises(rrlbm.RRError):
        rrlbm.Solver(p)


def _fdbc_channel(**kw):
    p, _ = presets.channel(nx=16, ny=12, nz=8, les=False, variant="config")
    p.face[2] = p.face[3] = rrlbm.FACE_FDBC
    for k, v in kw.items():
        setattr(p, k, v)
    return p


@pytest.mark.parametrize("change,msg", [
    (lambda p: (p.face.__setitem__(0, rrlbm.FACE_FDBC), p.face.__setitem__(1, rrlbm.FACE_FDBC)), "y faces only"),
    (lambda p: (p.face.__setitem__(0, rrlbm.FACE_WALL), p.face.__setitem__(1, rrlbm.FACE_WALL)), "periodic x and z"),
    (lambda p: p.uwall[3].__setitem__(0, 0.05), "walls at rest"),
    (lambda p: setattr(p, "ly", 3), "ly >= 4"),
    (lambda p: setattr(p, "collision", rrlbm.COLL_BGK), "RR collision"),
    (lambda p: (setattr(p, "use_les", 1), setattr(p, "lx", 2)), "lx >= 3"),
])
def test_fdbc_unsupported_combinations_rejected(change, msg):
    """the finite-difference closure (BC.cu:129-309) is defined for y walls at
    rest with x and z periodic, at least rows 1 and 2 inside"""
    p = _fdbc_channel()
    change(p)
    with pytest.raises(rrlbm.RRError) as e:
        rrlbm.Solver(p)
    assert e.value.code == 4 and msg in str(e.value), str(e.value)
    assert rrlbm.bytes_for(p) == 0


def test_trip_forcing_needs_a_force():
    p, _ = presets.channel(nx=16, ny=12, nz=8, les=False, variant="config")
    p.trip_steps = 100
    p.force[0] = 0.0
    with pytest.raises(rrlbm.RRError) as e:
        rrlbm.Solver(p)
    assert e.value.code == 4 and "force" in str(e.value)


def test_fdbc_face_kind_range():
    p = _fdbc_channel()
    p.face[2] = p.face[3] = 4
    with pytest.raises(rrlbm.RRError) as e:
        rrlbm.Solver(p)
    assert e.value.code == 1 and "unknown" in str(e.value)


def test_fdbc_bytes_for_counts_wall_slots():
    p = _fdbc_channel(use_les=1)
    q = _fdbc_channel(use_les=1)
    q.face[2] = q.face[3] = rrlbm.FACE_WALL
    assert rrlbm.bytes_for(p) - rrlbm.bytes_for(q) == 4 * 16 * 8 * 8
    assert rrlbm.bytes_for(_fdbc_channel()) == rrlbm.bytes_for(_fdbc_channel(face=q.face))


def test_bytes_for():
    p, _ = presets.cavity(n=128, storage="f16")
    b = rrlbm.bytes_for(p)
    n = 128 ** 3
    assert 2 * 27 * n * 2 <= b < 2 * 27 * n * 2 + 2_000_000


def test_tg_start_matches_oracle():
    for variant in ("config", "reference"):
        p, st = presets.taylor_green(L=24, nz=4, variant=variant)
        o = oracle_for(p)
        if variant == "config":
            o.init_tg_config(st["U0"])
        else:
            o.init_tg_reference(st["U0"])
        for k in ("rho", "ux", "uy", "uz"):
            assert np.abs(getattr(o, k) - st[k]).max() < 1e-17, (variant, k)
        assert np.abs(o.f - st["f"]).max() < 2e-16, variant


def test_channel_starts_match_oracle():
    p, st = presets.channel(nx=16, ny=12, nz=8, variant="reference")
    o = oracle_for(p)
    o.init_channel_loglaw(p.ustar, p.ystar)
    for k in ("rho", "ux", "uy", "uz"):
        assert np.abs(getattr(o, k) - st[k]).max() < 1e-17, k
    assert np.array_equal(o.f, st["f"])
    p, st = presets.channel(nx=16, ny=12, nz=8, variant="config", amp=0.1, seed=5)
    o = oracle_for(p)
    o.init_channel_config(st["uc"], 0.1, 5)
    for k in ("ux", "uy", "uz"):
        assert np.abs(getattr(o, k) - st[k]).max() < 1e-18, k


def test_params_layout_matches_the_header(tmp_path):
    """the ctypes mirror of rr_params has the C struct's size and field offsets"""
    import ctypes
    import subprocess

    from conftest import ROOT

    fields = [f[0] for f in rrlbm.Params._fields_]
    src = tmp_path / "layout.c"
    src.write_text('#include <stddef.h>\n#include <stdio.h>\n#include "rr_api.h"\nint main(void) {\n'
                   '    printf("%zu\\n", sizeof(rr_params));\n' +
                   "".join(f'    printf("%zu\\n", offsetof(rr_params, {f}));\n' for f in fields) +
                   "    return 0;\n}\n")
    exe = tmp_path / "layout"
    r = subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True).stdout.split()]
    assert out[0] == ctypes.sizeof(rrlbm.Params)
    assert out[1:] == [getattr(rrlbm.Params, f).offset for f in fields]
