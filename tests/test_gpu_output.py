"""rr_output / rr_save / rr_load against the reference's file formats
(RR27V33_code_DNS_LES/output.cu:3-258, restart reader initial.cu:189-265).

The oracle's restatement of the reference's writers is pinned byte for byte
to output.cu compiled for the host (tests/test_oracle.py).  Here the
library's own writers, fed by the GPU state, are held to that restatement on
the same FP64 fields: the restart files byte for byte, statistics.dat and
Profiles.txt byte for byte, the console line to 1e-13 relative (the library
forms the domain means with a device reduction, the reference with a
sequential loop).  A restart written in the reference's format loads back
through rr_load and continues as the uninterrupted run does (1e-13 on rho and
f, 1e-12 of the velocity scale on u: the upload re-forms the deviations from
FP64 populations)."""
import os
import re

import numpy as np
import pytest

import rrlbm
from rrlbm import presets
from oracle import oracle as O
from test_oracle import compare_output_dirs

pytestmark = pytest.mark.gpu

ALL = rrlbm.OUT_DIAG | rrlbm.OUT_FLOW | rrlbm.OUT_PROFILE | rrlbm.OUT_F


def _console_numbers(line):
    """the four %e numbers of diag_flow's console line"""
    return [float(x) for x in re.findall(r"[-+]?\d\.\d+e[-+]\d+", line)]


@pytest.mark.parametrize("les", [True, False])
def test_outputs_and_restart_in_the_reference_format(tmp_path, capfd, les):
    p, st = presets.channel(nx=16, ny=12, nz=8, les=les, variant="config", amp=0.2)
    lib_dir, orc_dir = tmp_path / "lib", tmp_path / "orc"
    orc_dir.mkdir()
    with rrlbm.Solver(p) as s:
        s.init_state(st["rho"], st["ux"], st["uy"], st["uz"])
        s.step(7)
        capfd.readouterr()
        s.output(ALL, str(lib_dir))
        line_lib = capfd.readouterr().out
        m = s.macro(taut=True)
        f = s.get_f()
        O.write_outputs(orc_dir, 7, m["rho"], m["ux"], m["uy"], m["uz"], m["taut"], f, p.ustar, p.ystar)
        line_orc = capfd.readouterr().out
        # the restart in the reference's format continues the run
        s.step(1)
        cont = s.macro()
        cont_f = s.get_f()
    compare_output_dirs(str(lib_dir), str(orc_dir), 7)
    assert line_lib.startswith("Step 7 ") and line_orc.startswith("Step 7 ")
    a, b = _console_numbers(line_lib), _console_numbers(line_orc)
    assert len(a) == len(b) == 4
    assert np.allclose(a, b, rtol=1e-13, atol=0.0), (a, b)
    # rr_save writes the restart pair of rr_output
    with rrlbm.Solver(p) as r:
        r.load(str(orc_dir), 7)
        assert r.istep == 7
        r.step(1)
        got = r.macro()
        got_f = r.get_f()
        r.save(str(tmp_path / "saved"))
    for name in ("000000008.dat", "f000000008.dat"):
        assert os.path.getsize(tmp_path / "saved" / name) == (4 if name[0] == "0" else p.q) * p.n * 8
    uc = st["uc"]
    assert np.abs(got["rho"] - cont["rho"]).max() < 1e-13
    for k in ("ux", "uy", "uz"):
        assert np.abs(got[k] - cont[k]).max() / uc < 1e-12, k
    assert np.abs(got_f - cont_f).max() < 1e-13
