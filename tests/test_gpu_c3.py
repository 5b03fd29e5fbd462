"""C3: 30-degree dipping reverse fault with degenerated wedge elements, slip law, learned guess.

Generated at dx = 400 m (777,632 elements, 5,000 wedge pairs, 5,151 fault pairs).  The overstressed
patch slips at the first step, creeps, and at about 1.7 s (step 100) the rupture takes off; by
step 300 it has broken 60 % of the fault.  (The test mesh does not resolve the slip law's process
zone well: around step 500 the oracle itself blows up at this resolution.)  The take-off amplifies
round-off: the oracle itself, with its initial shear perturbed by 1 part in 1e14, differs from the
unperturbed oracle by ~3e-13 at step 90 and by 3e-3 (relative L2 of slip rate) at step 200.  So:
  * up to step 90 the binary64 form must match the oracle to relative 1e-9, and the binary32 form
    with the learned guess must stay within the accuracy budget (1 %);
  * at step 300 the binary64 form must stay within 10x the oracle's own sensitivity to a
    perturbation of 1e-14; the binary32 form's round-off is amplified the same way (to ~1 % on slip
    rate, with either Newton guess), so there the learned guess must keep the binary32 form within
    the spread of the binary32 form with the plain guess.
"""
import tempfile

import numpy as np
import pytest

from conftest import nthreads

pytestmark = pytest.mark.gpu

N_EARLY = 90
N_LATE = 300


def _rel(a, b, scale=None):
    return np.linalg.norm(a - b) / (scale if scale else max(np.linalg.norm(b), 1e-300))


@pytest.fixture(scope="module")
def c3():
    from eqdyna_gb300.case import Case
    from eqdyna_gb300.configs import config_c3
    from oracle import Oracle
    case = Case.from_dir(config_c3(tempfile.mkdtemp(prefix="eqd_c3_"), scale=4.0, nsteps=N_LATE))
    early, late, pert = case.clone(), case.clone(), case.clone()
    pert.arrays["fric"].reshape(-1, 100)[:, 48] *= 1.0 + 1e-14  # fric(49): initial dip shear
    o_early = Oracle(early, nthreads())
    o_early.step(N_EARLY)
    for c in (late, pert):
        Oracle(c, nthreads()).step(N_LATE)
    return case, early, o_early, late, pert


def _fields(c):
    f = c.fric()
    return {"slip": f[:, 70:72], "slip_rate": f[:, 73:75], "peak_rate": f[:, 75], "vel": c.arrays["velArr"]}


def test_c3_mesh_has_wedges(c3):
    case = c3[0]
    et = case.arrays["elemTypeArr"]
    assert (et == 11).sum() > 0 and (et == 11).sum() == (et == 12).sum() and (et == 13).sum() > 0
    assert case.scalars.friclaw == 4


def test_c3_fp64_matches_oracle_before_take_off(c3):
    from eqdyna_gb300.solver import GpuSolver
    from test_gpu_parity import check_parity
    case, early, o_early = c3[:3]
    gpu = case.clone()
    with GpuSolver(gpu, precision="fp64") as s:
        s.step(N_EARLY)
        s.fetch()
        stats = s.stats()
    print(check_parity(early, gpu, case.scalars.dt))
    ref = o_early.stats()["newton_iters"]
    assert abs(stats["newton_iters"] - ref) <= 1e-3 * ref


def test_c3_fp64_within_oracle_sensitivity_after_take_off(c3):
    from eqdyna_gb300.solver import GpuSolver
    case, _, _, late, pert = c3
    gpu = case.clone()
    with GpuSolver(gpu, precision="fp64") as s:
        s.step(N_LATE)
        s.fetch()
    rep = _against_sensitivity(late, pert, gpu)
    print("binary64: gpu vs oracle, oracle perturbed by 1e-14 vs oracle:", rep)
    assert (late.arrays["fnft"][: case.npair] < 1e4).sum() > 500  # the rupture is under way
    for k, (ours, own) in rep.items():
        # pair counts are whole numbers; rupture times are whole steps
        floor = {"ruptured_pairs": 1e-2, "rupture_time_steps": 0.5}.get(k, 1e-9)
        assert ours <= max(floor, 10.0 * own), (k, ours, own)


def _against_sensitivity(ref, pert, gpu):
    fl, fp, fg = _fields(ref), _fields(pert), _fields(gpu)
    scale = max(np.linalg.norm(fl["slip_rate"]), np.linalg.norm(fl["peak_rate"]))
    rep = {}
    for k in fl:
        sc = scale if k == "slip_rate" else None
        rep[k] = (_rel(fg[k], fl[k], sc), _rel(fp[k], fl[k], sc))
    n = ref.npair
    count = lambda c: int((c.arrays["fnft"][:n] < 1e4).sum())
    rep["ruptured_pairs"] = (abs(count(gpu) - count(ref)) / count(ref), abs(count(pert) - count(ref)) / count(ref))
    tr, tp, tg = (c.arrays["fnft"][:n] for c in (ref, pert, gpu))
    both = (tr < 1e4) & (tp < 1e4) & (tg < 1e4)
    dt = ref.scalars.dt
    # mean rupture-time difference in steps, over pairs ruptured in all three runs
    rep["rupture_time_steps"] = (float(np.abs(tg[both] - tr[both]).mean() / dt), float(np.abs(tp[both] - tr[both]).mean() / dt))
    return rep


def test_c3_fp32_learned(c3):
    from eqdyna_gb300.solver import GpuSolver
    from test_gpu_fp32 import _check, _errors
    case, early, _, late, pert = c3
    with GpuSolver(case.clone(), precision="fp64") as plain:
        plain.newton_log(N_LATE // 4, 4)
        plain.step(N_LATE)
        hist = plain.train_mlp(epochs=10, batch=1024, lr=2e-3, holdout=0.1, seed=3)
        params, norm = plain.mlp_state()
        counts = (plain.replay(learned=False), plain.replay(learned=True))
    print("loss", hist, "iterations plain / learned", counts)
    assert counts[1]["records"] == (N_LATE // 4) * case.npair
    gpu = case.clone()
    with GpuSolver(gpu, precision="fp32") as s:
        s.set_mlp(params, norm)
        s.step(N_EARLY)
        s.fetch()
        err = _errors(early, gpu)
        print("fp32+learned before take-off", err)
        _check(err)
        s.step(N_LATE - N_EARLY)
        s.fetch()
        nc = s.newton_counts()
    assert nc["learned"] == N_LATE * case.npair
    plain32 = case.clone()
    with GpuSolver(plain32, precision="fp32") as s:
        s.step(N_LATE)
        s.fetch()
    err, err_plain = _errors(late, gpu), _errors(late, plain32)
    print("after take-off: binary32 + learned", err, "repeated solves", nc["fallbacks"])
    print("after take-off: binary32 + plain guess", err_plain)
    print("after take-off: binary64 oracle perturbed by 1e-14", _against_sensitivity(late, pert, gpu))
    assert (late.arrays["fnft"][: case.npair] < 1e4).mean() > 0.5  # the rupture is under way
    # binary32 round-off amplified by the take-off: ~1 % on slip rate, ~2.5 % on peak slip rate at
    # step 300 with either guess; the learned guess perturbs each solve at round-off level too, so
    # the two binary32 runs are compared as samples of the same spread
    for k in ("slip_rate", "slip", "peak_rate"):
        assert err_plain[k] <= 5e-2, (k, err_plain[k])
        assert err[k] <= max(1e-2, 3.0 * err_plain[k]), (k, err[k], err_plain[k])
    assert err["rupture_flips"] <= max(10, 2 * err_plain["rupture_flips"])


def test_c3_sparse_pml_tiles_are_repacked():
    """C3's PML shell has stretched cells: bins of the median element width merge some and skip
    others, and with the default 4 x 8 x 4 brick about half of the PML slots would stay empty
    (51 %).  The brick order then bins by rank (one bin per cell of a structured layer) and keeps
    the densest candidate order."""
    from eqdyna_gb300.case import Case
    from eqdyna_gb300.configs import config_c3
    from eqdyna_gb300.solver import GpuSolver
    case = Case.from_dir(config_c3(tempfile.mkdtemp(prefix="eqd_c3t_"), scale=4.0, nsteps=10))
    with GpuSolver(case, precision="fp32") as s:
        info = s.table_info()
    for name, grp in info.items():
        live = grp["elements"] / grp["slots"]
        print(name, grp["tiles"], "tiles", round(live, 3), "live")
        assert grp["slots"] == 128 * grp["tiles"]
    assert info["pml"]["elements"] / info["pml"]["slots"] >= 0.65
    assert info["interior"]["elements"] / info["interior"]["slots"] >= 0.7
