"""The metric's accuracy condition over a whole job, past the rupture.

The binary32 form with the learned Newton guess runs a C1 job as bench.py runs it (a plain
warm-up whose Newton solves are logged one step in ten, training on the GPU, then the learned
guess for the rest of the job); the plain binary64 form (itself held to the oracle at 1e-9 in
test_gpu_parity.py and test_gpu_aging_viscous.py) runs the same job.  After 1,500 steps (12 s of
rupture at dx = 200 m, the nucleation ramp is 1 s) the final slip rate, slip and peak slip rate
must agree to 1 % (relative L2), rupture times to one step, with at most 0.2 % of the pairs
ruptured in one run only, and the on- and off-fault station histories to 1 %.
"""
import tempfile

import pytest

pytestmark = pytest.mark.gpu

JOB = 1500
LOG_STEPS, LOG_STRIDE = 70, 10


def test_fp32_learned_job_within_budget_of_plain_fp64_past_the_rupture():
    from bench import compare_fault_results, fault_result
    from eqdyna_gb300.case import Case
    from eqdyna_gb300.configs import config_c1
    from eqdyna_gb300.solver import GpuSolver
    case = Case.from_dir(config_c1(tempfile.mkdtemp(prefix="eqd_c1job_"), scale=2.0, nsteps=JOB))
    run = case.clone()
    with GpuSolver(run, precision="fp32", learned_guess=True) as s:
        s.newton_log(LOG_STEPS, LOG_STRIDE)
        s.step(LOG_STEPS * LOG_STRIDE)
        hist = s.train_mlp(epochs=8, batch=4096, lr=1e-3, holdout=0.05, seed=20261203)
        s.step(JOB - LOG_STEPS * LOG_STRIDE)
        s.fetch()
        counts = s.newton_counts()
    ref = case.clone()
    with GpuSolver(ref, precision="fp64") as r:
        r.step(JOB)
        r.fetch()
    err = compare_fault_results(fault_result(run), fault_result(ref), case.scalars.dt)
    print("C1 dx 200 m,", JOB, "steps, binary32 + learned guess vs plain binary64:", err,
          "training loss", hist["epoch_loss"][0], "->", hist["epoch_loss"][-1], "newton", counts)
    assert counts["learned"] > 0
    assert err["ruptured"] >= 0.1 * case.npair, "the job must run well into the rupture"
    assert err["slip_rate_rel_l2"] <= 1e-2
    assert err["slip_rel_l2"] <= 1e-2
    assert err["peak_rate_rel_l2"] <= 1e-2
    assert err["rupture_dt_max"] <= 1.0 + 1e-9
    assert err["rupture_flips"] <= max(2, 0.002 * err["ruptured"])
    assert err["onfault_stations_rel_l2"] <= 1e-2
    assert err["offfault_stations_rel_l2"] <= 1e-2
