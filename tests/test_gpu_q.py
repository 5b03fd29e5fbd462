"""Coarse-grained Q (C_Q = 1: 8 relaxation mechanisms spread over the 2 x 2 x 2 element pattern,
6 memory variables per element, src/calcElemKU.f90:77-132, src/qconstant.f90) on the C0 half-space
at dx = 800 m: the binary64 form against the oracle to relative 1e-9, the binary32 form (Q
constants in the element records, memory variables in binary32) within the accuracy budget, and
the attenuation itself visible (the run differs from the elastic one)."""
import tempfile

import numpy as np
import pytest

from conftest import nthreads

pytestmark = pytest.mark.gpu

NSTEPS = 120


@pytest.fixture(scope="module")
def q_case():
    from eqdyna_gb300.case import Case
    from eqdyna_gb300.configs import config_c0
    from oracle import Oracle
    case = Case.from_dir(config_c0(tempfile.mkdtemp(prefix="eqd_q_"), scale=4.0, nsteps=NSTEPS, C_Q=1))
    assert case.scalars.C_Q == 1
    cpu = case.clone()
    Oracle(cpu, nthreads()).step(NSTEPS)
    return case, cpu


def test_q_fp64_matches_oracle(q_case):
    from eqdyna_gb300.solver import GpuSolver
    from test_gpu_parity import check_parity
    case, cpu = q_case
    gpu = case.clone()
    with GpuSolver(gpu, precision="fp64") as s:
        s.step(NSTEPS)
        s.fetch()
    print(check_parity(cpu, gpu, case.scalars.dt))
    # memory variables (stress rows 7-12 of interior elements)
    et = cpu.arrays["elemTypeArr"]
    base = cpu.arrays["stressCompIndexArr"][et != 2]
    idx = (base[:, None] + 6 + np.arange(6)[None, :]).ravel()
    mc, mg = cpu.arrays["stressArr"][idx], gpu.arrays["stressArr"][idx]
    assert np.abs(mc).max() > 0.0
    assert np.linalg.norm(mg - mc) <= 1e-9 * np.linalg.norm(mc)


def test_q_fp32_within_budget(q_case):
    from eqdyna_gb300.solver import GpuSolver
    from test_gpu_fp32 import _check, _errors
    case, cpu = q_case
    gpu = case.clone()
    with GpuSolver(gpu, precision="fp32") as s:
        s.step(NSTEPS)
        s.fetch()
        info = s.table_info()
    err = _errors(cpu, gpu)
    vc, vg = cpu.arrays["velArr"], gpu.arrays["velArr"]
    err["vel"] = float(np.linalg.norm(vg - vc) / np.linalg.norm(vc))
    print("fp32 with Q", info, err)
    assert info["interior"]["layout"] == "records"
    _check(err)
    assert err["vel"] <= 1e-3


def test_q_changes_the_wavefield(q_case):
    from eqdyna_gb300.case import Case
    from eqdyna_gb300.configs import config_c0
    from eqdyna_gb300.solver import GpuSolver
    case, cpu = q_case
    elastic = Case.from_dir(config_c0(tempfile.mkdtemp(prefix="eqd_q0_"), scale=4.0, nsteps=NSTEPS))
    with GpuSolver(elastic, precision="fp64") as s:
        s.step(NSTEPS)
        s.fetch()
    d = np.linalg.norm(elastic.arrays["velArr"] - cpu.arrays["velArr"]) / np.linalg.norm(cpu.arrays["velArr"])
    print("elastic vs Q relative velocity difference", d)
    assert d > 1e-3


def test_q_streamed_tables_rejected(q_case):
    from eqdyna_gb300 import _native as N
    from eqdyna_gb300.solver import GpuSolver
    case, _ = q_case
    with pytest.raises(N.EqdError) as ei:
        GpuSolver(case.clone(), precision="fp32", table_layout="streamed")
    assert ei.value.code == 5
