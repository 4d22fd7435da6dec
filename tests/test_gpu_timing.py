"""The reference's routine timers (timingmod.f90:16-103) on CUDA events.

A CMF2 run and a Cash-Karp run of the small models with the timers on: the
routines each integrator goes through (Calc_MeanField, Calc_h1mode, the grid
SPF derivative, the overlaps, the Lanczos runs for CMF2; CalcDerivs for RK)
report calls and device time, the Gaussian ones none, and the `timing` file
has the reference's layout (write_timings, timingmod.f90:72-103).
"""
import re

import pytest

from macaw_gb300.model import INT_CMF2, INT_RK45, AU2FS, initial_wavefunction
from tests.helpers import small_lvc, small_qvc

pytestmark = pytest.mark.gpu


def test_cmf2_routine_timers_and_timing_file(tmp_path):
    from macaw_gb300.capi import GpuCore
    model = small_qvc(tfinal_fs=0.5)
    A, psi = initial_wavefunction(model)
    core = GpuCore(model)
    core.timing(2)
    core.set_state(A, psi, as_start=True)
    core.propagate_interval(INT_CMF2, 0.2 / AU2FS, 0.0, model.tout * model.eps_int)
    tm = core.timing_read()
    for name in ("Calc_MeanField", "Calc_h1mode", "Calc_Der_SPF_DVR", "normWF/wf_ovl", "Lanczos"):
        assert tm[name]["calls"] > 0 and tm[name]["ms"] > 0.0, (name, tm[name])
    assert tm["Calc_CY"]["calls"] == 0 and tm["Calc_Der_SPF_GWP"]["calls"] == 0
    assert tm["CalcDerivs"]["calls"] == 0          # CMF2 evaluates mean fields, not Calc_Derivs
    path = tmp_path / "timing"
    core.write_timings(str(path), 10.0)
    lines = path.read_text().splitlines()
    assert lines[0] == "Total time:   0 h   0 m   10 s"
    assert lines[3].split() == ["Subroutine", "Calls", "N", "time/N", "[ms]", "time", "[min]", "%time"]
    rows = lines[5:]
    assert len(rows) == 8
    fmt = re.compile(r"^ {0,19}\S+ {4}[ \d]{7} {3}[ \d.]{9} {3}[ \d.]{11} {6}[ \d.]{6}$")
    for name, row in zip(GpuCore.TIMERS, rows):
        assert row[:20].strip() == name and fmt.match(row), row
        assert int(row[24:31]) == tm[name]["calls"]
    core.close()


def test_rk_routine_timers():
    from macaw_gb300.capi import GpuCore
    model = small_lvc(tfinal_fs=0.2)
    A, psi = initial_wavefunction(model)
    core = GpuCore(model)
    core.timing(2)
    core.set_state(A, psi, as_start=True)
    core.propagate_interval(INT_RK45, 0.1 / AU2FS, 0.0, model.tout * model.eps_int)
    tm = core.timing_read()
    assert tm["CalcDerivs"]["calls"] > 0
    assert tm["Calc_MeanField"]["calls"] >= tm["CalcDerivs"]["calls"]
    assert tm["Lanczos"]["calls"] == 0
    core.timing(0)
    n = tm["CalcDerivs"]["calls"]
    core.propagate_interval(INT_RK45, 0.2 / AU2FS, 0.1 / AU2FS, model.tout * model.eps_int)
    assert core.timing_read()["CalcDerivs"]["calls"] == n   # timers off
    core.close()
