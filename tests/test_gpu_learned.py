"""Learned Newton initial guess and the logged-solve machinery.

* the tensor-core training kernel's loss and gradient against the numpy reference (mlp_ref);
* logged solves replay bit for bit, both with the loop the fault kernel runs (loop-invariant law
  terms evaluated once, early stop on a repeated iterate) and with the reference's loop verbatim,
  with the reference's iteration count;
* training on solves logged by the plain method lowers the loss; iteration counts of the plain
  and the learned guess are reported; every solve converges to the same slip rate from either
  guess; the binary32 form with the learned guess stays within the accuracy budget.
"""
import tempfile

import numpy as np
import pytest

from conftest import nthreads
from mlp_ref import BLOCKS, NIN, he_params, loss_grad

pytestmark = pytest.mark.gpu


def test_mlp_gradient_matches_numpy_reference():
    from eqdyna_gb300.solver import mlp_gradient
    rng = np.random.default_rng(7)
    p = he_params(rng)
    x = rng.standard_normal((300, NIN)).astype(np.float32)
    t = rng.standard_normal(300).astype(np.float32)
    loss, g = mlp_gradient(p, x, t)
    lr, gr = loss_grad(p, x, t, rounded=True)
    print("loss", loss, lr)
    assert abs(loss - lr) <= 1e-3 * lr
    for name, sl in BLOCKS.items():
        rel = np.linalg.norm(g[sl] - gr[sl]) / np.linalg.norm(gr[sl])
        print(name, rel)
        assert rel <= 1e-2, name


@pytest.fixture(scope="module")
def c1_logged():
    """C1 at dx = 400 m, plain binary64 method, every other step of the first 160 logged."""
    from eqdyna_gb300.case import Case
    from eqdyna_gb300.configs import config_c1
    from eqdyna_gb300.solver import GpuSolver
    case = Case.from_dir(config_c1(tempfile.mkdtemp(prefix="eqd_c1_"), scale=4.0, nsteps=300))
    s = GpuSolver(case.clone(), precision="fp64")
    s.newton_log(80, stride=2)
    s.step(160)
    yield s, case
    s.close()


def test_logged_solves_replay_bit_for_bit(c1_logged):
    s, case = c1_logged
    rec = s.newton_records()
    assert rec.shape == (80 * case.npair, 16)
    ref, v_ref = s.replay(learned=False, fast=False, values=True)
    fast, v_fast = s.replay(learned=False, fast=True, values=True)
    print("reference loop", ref, "fault-kernel loop", fast)
    assert np.array_equal(v_ref, rec[:, 14])
    assert np.array_equal(v_fast, rec[:, 14])
    assert ref["iterations"] == fast["iterations"] == int(rec[:, 15].sum())
    assert ref["executed"] == ref["iterations"]
    assert fast["executed"] <= ref["executed"]


@pytest.fixture(scope="module")
def c1_trained(c1_logged):
    """The model trained on the logged plain solves (once per module, whichever test asks first)."""
    s, case = c1_logged
    hist = s.train_mlp(epochs=20, batch=1024, lr=2e-3, holdout=0.1, seed=5)
    return s, case, hist


def test_learned_guess_trains_and_converges_to_the_same_solutions(c1_trained):
    s, _, hist = c1_trained
    print("loss", hist)
    assert hist["epoch_loss"][-1] < 0.5 * hist["epoch_loss"][0]
    assert hist["holdout_loss"] < 2.0 * hist["epoch_loss"][-1]
    plain, vp = s.replay(learned=False, values=True)
    learned, vl = s.replay(learned=True, values=True)
    print("plain guess", plain, "learned guess", learned)
    rel = np.abs(vl - vp) / np.abs(vp)
    print("max relative difference of the converged slip rate", rel.max(), "median", np.median(rel))
    assert np.quantile(rel, 0.999) <= 1e-9
    s.enable_mlp(False)


def test_fp32_learned_form_within_budget(c1_trained):
    """The model trained on the plain solves drives the binary32 form over C1 (dx = 400 m, 300
    steps) within the slip-rate budget of the binary64 oracle."""
    from eqdyna_gb300.solver import GpuSolver
    from oracle import Oracle
    from test_gpu_fp32 import _check, _errors
    s, case, _ = c1_trained
    params, norm = s.mlp_state()
    cpu = case.clone()
    Oracle(cpu, nthreads()).step(300)
    gpu = case.clone()
    with GpuSolver(gpu, precision="fp32") as g:
        g.set_mlp(params, norm)
        g.step(300)
        g.fetch()
        counts = g.newton_counts()
    err = _errors(cpu, gpu)
    print("fp32+learned", err, counts)
    assert counts["learned"] == 300 * case.npair
    _check(err)


def test_fast_and_reference_loops_take_the_same_decisions(c1_trained):
    """Per logged solve, the fault kernel's loop (early stop on a fixed point or a 2-cycle) and the
    reference's loop give the same slip rate, the same step ratio of the last evaluation (which
    decides a repeat from the plain guess), the same iteration count, cap and repeat, from the
    plain and from the learned guess; the early stops of both 2-cycle parities occur in the data."""
    s, _, _ = c1_trained
    for learned in (False, True):
        ref = s.replay_records(learned=learned, fast=False)
        fast = s.replay_records(learned=learned, fast=True)
        kinds = np.bincount(fast["exit"], minlength=4)
        print("learned" if learned else "plain", "exits (test/cap, fixed point, 2-cycle last, 2-cycle previous):",
              kinds.tolist(), "repeats", int(fast["fallback"].sum()))
        assert np.array_equal(fast["v"], ref["v"])
        assert np.array_equal(fast["step"], ref["step"])
        for k in ("iters", "capped", "fallback"):
            assert np.array_equal(fast[k], ref[k]), k
        if not learned:
            assert kinds[2] > 0 and kinds[3] > 0


def test_guess_outside_the_training_range_is_the_plain_guess(c1_trained):
    """The learned guess is used only inside the range of each feature over the training data.
    Solves logged later than the training data (here steps 161-280, into the rupture) whose
    features leave that range are solved from the plain guess: the same slip rate and the same
    iteration count as the plain replay.  Solves inside it still use the model."""
    s, _, _ = c1_trained
    params, norm = s.mlp_state()
    lo, hi = norm[18:24].astype(np.float64), norm[26:32].astype(np.float64)
    assert np.all(hi >= lo) and np.any(hi > lo)
    s.newton_log(40, stride=3)
    s.step(120)
    rec = s.newton_records()
    f = np.stack([np.log(np.maximum(rec[:, 13], 1e-30)), np.log(np.maximum(np.abs(rec[:, 7]), 1e-30)),
                  rec[:, 9], rec[:, 10], rec[:, 0], rec[:, 1]], axis=1)
    # the device compares binary32 features; the two logarithms may differ from numpy's in the last
    # place, so those two get a margin on either side of the bound, the others are compared exactly
    f32 = f.astype(np.float32).astype(np.float64)
    margin = np.zeros(6)
    margin[:2] = 1e-5 * np.maximum(np.abs(lo[:2]), np.abs(hi[:2]))
    outside = np.any((f32 < lo - margin) | (f32 > hi + margin), axis=1)
    inside = np.all((f32 >= lo + margin) & (f32 <= hi - margin), axis=1)
    plain = s.replay_records(learned=False)
    learned = s.replay_records(learned=True)
    print("later solves:", len(rec), "outside the training range:", int(outside.sum()), "inside:", int(inside.sum()))
    assert outside.sum() > 0
    assert np.array_equal(learned["v"][outside], plain["v"][outside])
    assert np.array_equal(learned["iters"][outside], plain["iters"][outside])
    # inside the range the model drives the start: some solve takes another path than the plain one
    assert np.any(learned["iters"][inside] != plain["iters"][inside])
