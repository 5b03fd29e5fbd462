"""C3: 30-degree dipping reverse fault with degenerated wedge elements, slip law, learned guess.

Generated at dx = 400 m (777,632 elements, 5,000 wedge pairs, 5,151 fault pairs) and advanced 200
steps (3.3 s: the rupture leaves the patch at about 2 s and has broken a fifth of the fault by the
end): the binary64 form against the oracle (relative 1e-9, Newton iteration counts within 0.1 %),
the binary32 form with the learned guess (trained on the binary64 run's own solves) within the
accuracy budget.
"""
import tempfile

import numpy as np
import pytest

from conftest import nthreads

pytestmark = pytest.mark.gpu

NSTEPS = 200


@pytest.fixture(scope="module")
def c3():
    from eqdyna_gb300.case import Case
    from eqdyna_gb300.configs import config_c3
    from oracle import Oracle
    case = Case.from_dir(config_c3(tempfile.mkdtemp(prefix="eqd_c3_"), scale=4.0, nsteps=NSTEPS))
    cpu = case.clone()
    o = Oracle(cpu, nthreads())
    o.step(NSTEPS)
    return case, cpu, o


def test_c3_mesh_has_wedges(c3):
    case, _, _ = c3
    et = case.arrays["elemTypeArr"]
    assert (et == 11).sum() > 0 and (et == 11).sum() == (et == 12).sum() and (et == 13).sum() > 0
    assert case.scalars.friclaw == 4


def test_c3_fp64_matches_oracle(c3):
    from eqdyna_gb300.solver import GpuSolver
    from test_gpu_parity import check_parity
    case, cpu, o = c3
    gpu = case.clone()
    with GpuSolver(gpu, precision="fp64") as s:
        s.step(NSTEPS)
        s.fetch()
        stats = s.stats()
    print(check_parity(cpu, gpu, case.scalars.dt))
    ref = o.stats()["newton_iters"]
    assert abs(stats["newton_iters"] - ref) <= 1e-3 * ref


def test_c3_fp32_learned_within_budget(c3):
    from eqdyna_gb300.solver import GpuSolver
    from test_gpu_fp32 import _check, _errors
    case, cpu, _ = c3
    with GpuSolver(case.clone(), precision="fp64") as plain:
        plain.newton_log(NSTEPS)
        plain.step(NSTEPS)
        hist = plain.train_mlp(epochs=10, batch=1024, lr=2e-3, holdout=0.1, seed=3)
        params, norm = plain.mlp_state()
        counts = (plain.replay(learned=False), plain.replay(learned=True))
    print("loss", hist, "iterations plain / learned", counts)
    gpu = case.clone()
    with GpuSolver(gpu, precision="fp32") as s:
        s.set_mlp(params, norm)
        s.step(NSTEPS)
        s.fetch()
        used = s.newton_counts()["learned"]
    err = _errors(cpu, gpu)
    print("fp32+learned", err)
    assert used == NSTEPS * case.npair
    assert (cpu.arrays["fnft"][: case.npair] < 1e4).sum() > 500  # the rupture is under way
    _check(err)
