"""binary32 form (FP32 element strain/stress/hourglass, Kahan-compensated FP32 nodal sums, FP64
state and fault) against the binary64 oracle.

Budget (the benchmark spec): relative L2 slip-rate error <= 1 % and rupture time within one time step.
The measured errors are printed (pytest -s) and recorded in the design doc.
"""
import tempfile

import numpy as np
import pytest

from conftest import golden_path, nthreads

pytestmark = pytest.mark.gpu


def _errors(cpu, gpu):
    fc, fg = cpu.fric(), gpu.fric()
    peak = np.linalg.norm(fc[:, 75])
    rate = np.linalg.norm(fg[:, [73, 74]] - fc[:, [73, 74]]) / max(np.linalg.norm(fc[:, [73, 74]]), peak)
    slip = np.linalg.norm(fg[:, [70, 71]] - fc[:, [70, 71]]) / np.linalg.norm(fc[:, [70, 71]])
    peak_rate = np.linalg.norm(fg[:, 75] - fc[:, 75]) / peak
    tc, tg = cpu.arrays["fnft"][: cpu.npair], gpu.arrays["fnft"][: gpu.npair]
    both = (tc < 1e4) & (tg < 1e4)
    flips = int(((tc < 1e4) != (tg < 1e4)).sum())
    dtr = np.abs(tc[both] - tg[both]).max() / cpu.scalars.dt if both.any() else 0.0
    return {"slip_rate": rate, "slip": slip, "peak_rate": peak_rate, "rupture_dt_max": dtr,
            "rupture_flips": flips, "ruptured": int((tc < 1e4).sum())}


def _run(case, nsteps):
    from eqdyna_gb300.solver import GpuSolver
    from oracle import Oracle
    cpu, gpu = case.clone(), case.clone()
    Oracle(cpu, nthreads()).step(nsteps)
    with GpuSolver(gpu, precision="fp32") as s:
        s.step(nsteps)
        s.fetch()
    return _errors(cpu, gpu)


def _check(err):
    print(err)
    assert err["slip_rate"] <= 1e-2
    assert err["slip"] <= 1e-2
    assert err["peak_rate"] <= 1e-2
    assert err["rupture_dt_max"] <= 1.0 + 1e-9
    assert err["rupture_flips"] <= max(2, 0.002 * err["ruptured"])


@pytest.mark.parametrize("name,nsteps", [("tpv8", 114), ("tpv104", 80), ("meng2023cb", 100)])
def test_fp32_form_within_budget_on_reference_cases(name, nsteps):
    from eqdyna_gb300.case import Case
    _check(_run(Case.from_fixture(golden_path(name)), nsteps))


def test_fp32_form_within_budget_on_c1_shape():
    """C1 (aging law, 40-layer PML scaled with dx) at dx = 400 m over 300 steps."""
    from eqdyna_gb300.case import Case
    from eqdyna_gb300.configs import config_c1
    case = Case.from_dir(config_c1(tempfile.mkdtemp(prefix="eqd_c1_"), scale=4.0, nsteps=300))
    _check(_run(case, 300))
