"""Ensembles: scenarios of different mesh sizes and time steps advanced together (one launch per
kernel per step over all members) agree with each member run alone, and every member stays within
the binary32 form's accuracy budget against the binary64 oracle run on that member alone.

Binary32 runs are not bitwise reproducible (the nodal sums end in binary32 L2 reductions from
several CTAs), so members are compared with their solo runs to relative 1e-4.
"""
import tempfile

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SCALES = (4.0, 5.0, 6.0)  # C0 generator at dx = 800, 1000, 1200 m; dt = 0.032, 0.040, 0.048 s
NSTEPS = 60


def _cases():
    from eqdyna_gb300.case import Case
    from eqdyna_gb300.configs import config_c0
    return [Case.from_dir(config_c0(tempfile.mkdtemp(prefix="eqd_c0_"), scale=sc, nsteps=NSTEPS))
            for sc in SCALES]


def _rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def test_ensemble_matches_members_run_alone():
    from eqdyna_gb300.solver import Ensemble, GpuSolver
    cases = _cases()
    assert len({c.sizes["nelem"] for c in cases}) == len(cases)
    solo = []
    for c in cases:
        g = c.clone()
        with GpuSolver(g, precision="fp32", table_layout="records") as s:
            s.step(NSTEPS)
            s.fetch()
        solo.append(g)
    members = [c.clone() for c in cases]
    solvers = [GpuSolver(g, precision="fp32", table_layout="records") for g in members]
    try:
        with Ensemble(solvers) as e:
            e.step(1)    # first step of every member (stored acceleration)
            e.step(40)   # two captured 16-step graphs and a tail
            e.step(NSTEPS - 41)
        for s in solvers:
            s.fetch()
    finally:
        for s in solvers:
            s.close()
    for c, a, b in zip(cases, members, solo):
        fa, fb = a.fric(), b.fric()
        rep = {"slip": _rel(fa[:, 70:73], fb[:, 70:73]), "slip_rate": _rel(fa[:, 73:76], fb[:, 73:76]),
               "vel": _rel(a.arrays["velArr"], b.arrays["velArr"]),
               "disp": _rel(a.arrays["dispArr"], b.arrays["dispArr"])}
        print(c.sizes["nelem"], rep)
        assert all(v <= 1e-4 for v in rep.values()), rep
        ta, tb = a.arrays["fnft"][: a.npair], b.arrays["fnft"][: b.npair]
        assert np.array_equal(ta < 1e4, tb < 1e4)
        both = ta < 1e4
        assert np.all(np.abs(ta[both] - tb[both]) <= c.scalars.dt * 1.000001)
        assert np.abs(fa[:, 75]).max() > 0.0  # the rupture is under way
    # every batched member against the oracle (the binary32 form's budget: 1 % slip rate, slip and
    # peak slip rate, rupture time within one step)
    from conftest import nthreads
    from oracle import Oracle
    from test_gpu_fp32 import _check, _errors
    for c, a in zip(cases, members):
        cpu = c.clone()
        Oracle(cpu, nthreads()).step(NSTEPS)
        err = _errors(cpu, a)
        print("member", c.sizes["nelem"], "vs oracle", err)
        assert err["ruptured"] > 0
        _check(err)


def test_ensemble_rejects_streamed_members():
    from eqdyna_gb300 import _native as N
    from eqdyna_gb300.solver import Ensemble, GpuSolver
    cases = _cases()[:2]
    solvers = [GpuSolver(c.clone(), precision="fp32", table_layout="streamed") for c in cases]
    try:
        with pytest.raises(N.EqdError) as ei:
            Ensemble(solvers)
        assert ei.value.code == 5
    finally:
        for s in solvers:
            s.close()


def test_persistent_launch_matches_batched_launches():
    """eqd_ensemble_mode 1: every step of a call in one persistent cooperative launch (node update,
    element tiles and fault pairs of all members, phases closed by bounded grid barriers).  Each
    member agrees with the batched launches (mode 0) to relative 1e-4 and stays within the binary32
    budget against the oracle; both device times are printed."""
    from conftest import nthreads
    from eqdyna_gb300.solver import Ensemble, GpuSolver
    from oracle import Oracle
    from test_gpu_fp32 import _check, _errors
    cases = _cases()
    runs, times = {}, {}
    for mode in (0, 1):
        members = [c.clone() for c in cases]
        solvers = [GpuSolver(g, precision="fp32", table_layout="records") for g in members]
        try:
            with Ensemble(solvers, persistent=(mode == 1)) as e:
                e.step(1)
                e.step(NSTEPS - 1)
                times[mode] = e.last_step_ms
            for s in solvers:
                s.fetch()
        finally:
            for s in solvers:
                s.close()
        runs[mode] = members
    print("device ms for", NSTEPS - 1, "steps: batched", times[0], "persistent", times[1])
    for c, a, b in zip(cases, runs[1], runs[0]):
        fa, fb = a.fric(), b.fric()
        rep = {"slip": _rel(fa[:, 70:73], fb[:, 70:73]), "slip_rate": _rel(fa[:, 73:76], fb[:, 73:76]),
               "vel": _rel(a.arrays["velArr"], b.arrays["velArr"])}
        assert all(v <= 1e-4 for v in rep.values()), rep
        cpu = c.clone()
        Oracle(cpu, nthreads()).step(NSTEPS)
        err = _errors(cpu, a)
        print("persistent member", c.sizes["nelem"], rep, "vs oracle", err)
        _check(err)


def test_persistent_launch_rejects_rate_and_state_members():
    from eqdyna_gb300 import _native as N
    from eqdyna_gb300.case import Case
    from eqdyna_gb300.configs import config_c1
    from eqdyna_gb300.solver import Ensemble, GpuSolver
    case = Case.from_dir(config_c1(tempfile.mkdtemp(prefix="eqd_c1e_"), scale=8.0, nsteps=10))
    solvers = [GpuSolver(case.clone(), precision="fp32", table_layout="records") for _ in range(2)]
    try:
        with Ensemble(solvers) as e:
            with pytest.raises(N.EqdError) as ei:
                e.set_mode(1)
            assert ei.value.code == 5
            e.step(3)  # the batched launches still run them
    finally:
        for s in solvers:
            s.close()
