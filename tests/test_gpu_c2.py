"""C2: layered medium, Q from Vs (C_Q = 2) together with Drucker-Prager plasticity, von Karman
initial shear stress on a slip-weakening fault; generated at dx = 400 m (240,064 elements) and
advanced 200 steps (3.2 s: the patch nucleates, near-surface cells yield from the first steps).
The binary64 form must match the oracle to relative 1e-9 (slip, tractions, wavefield, stresses,
Q memory variables, plastic strain); the binary32 form must stay within the accuracy budget."""
import tempfile

import numpy as np
import pytest

from conftest import nthreads

pytestmark = pytest.mark.gpu

NSTEPS = 200


@pytest.fixture(scope="module")
def c2():
    from eqdyna_gb300.case import Case
    from eqdyna_gb300.configs import config_c2
    from oracle import Oracle
    case = Case.from_dir(config_c2(tempfile.mkdtemp(prefix="eqd_c2_"), scale=8.0, nsteps=NSTEPS))
    assert case.scalars.C_Q == 2 and case.scalars.C_elastic == 0
    cpu = case.clone()
    Oracle(cpu, nthreads()).step(NSTEPS)
    return case, cpu


def _interior_rows(c, first, n):
    et = c.arrays["elemTypeArr"]
    base = c.arrays["stressCompIndexArr"][et != 2]
    return (base[:, None] + first + np.arange(n)[None, :]).ravel()


def test_c2_fp64_matches_oracle(c2):
    from eqdyna_gb300.solver import GpuSolver
    from test_gpu_parity import check_parity
    case, cpu = c2
    gpu = case.clone()
    with GpuSolver(gpu, precision="fp64") as s:
        s.step(NSTEPS)
        s.fetch()
    print(check_parity(cpu, gpu, case.scalars.dt))
    mem = _interior_rows(cpu, 6, 6)
    mc, mg = cpu.arrays["stressArr"][mem], gpu.arrays["stressArr"][mem]
    pc, pg = cpu.arrays["pstrain"], gpu.arrays["pstrain"]
    print("memory variables", np.linalg.norm(mg - mc) / np.linalg.norm(mc), "plastic strain",
          np.linalg.norm(pg - pc) / np.linalg.norm(pc), "max", pc.max())
    assert np.abs(mc).max() > 0.0 and pc.max() > 0.0
    assert np.linalg.norm(mg - mc) <= 1e-9 * np.linalg.norm(mc)
    assert np.linalg.norm(pg - pc) <= 1e-9 * np.linalg.norm(pc)


def test_c2_fp32_within_budget(c2):
    from eqdyna_gb300.solver import GpuSolver
    from test_gpu_fp32 import _check, _errors
    case, cpu = c2
    gpu = case.clone()
    with GpuSolver(gpu, precision="fp32") as s:
        s.step(NSTEPS)
        s.fetch()
        info = s.table_info()
    err = _errors(cpu, gpu)
    vc, vg = cpu.arrays["velArr"], gpu.arrays["velArr"]
    err["vel"] = float(np.linalg.norm(vg - vc) / np.linalg.norm(vc))
    pc, pg = cpu.arrays["pstrain"], gpu.arrays["pstrain"]
    err["pstrain"] = float(np.linalg.norm(pg - pc) / np.linalg.norm(pc))
    print("fp32 C2", info, err)
    assert err["ruptured"] > 0
    _check(err)
    assert err["vel"] <= 1e-2 and err["pstrain"] <= 1e-2
