"""Pins the oracle (and the case builder that feeds it) to the reference's own golden outputs.

The goldens are test.reference.results/<case>/frt.txt* of the EQdyna reference (22 columns printed
in E18.7, src/library_output.f90:172-201), produced by a 2x2x1 MPI run; the fixtures were
extracted by tests/golden/make_fixtures.py.  check.test.py:40-52 compares them with an absolute
threshold of 1e-3, which for stresses near 1e8 Pa means print-exact; here every entry must agree
to within 0.75 unit of the 7th printed digit (or 1e-3 absolute).
"""
import numpy as np
import pytest

from conftest import golden_path, nthreads
from frt import FRT_COLUMNS, frt_table, golden_frt, match_rows

WELL_CONDITIONED = ["tpv8", "tpv10", "tpv104", "tpv1053d", "meng2023a", "meng2023cb"]


def _run(name):
    from eqdyna_gb300.case import Case
    from oracle import Oracle
    case = Case.from_fixture(golden_path(name))
    o = Oracle(case, nthreads())
    o.run()
    return case, o


def _unit(gold):
    a = np.abs(gold)
    with np.errstate(divide="ignore"):
        e = np.where(a > 0, np.floor(np.log10(np.where(a > 0, a, 1.0))) + 1, -300)
    return 10.0 ** (e - 7)


@pytest.mark.parametrize("name", WELL_CONDITIONED)
def test_oracle_matches_reference_frt(name):
    case, _ = _run(name)
    ours = frt_table(case)
    gold, dist = match_rows(ours, golden_frt(golden_path(name)))
    assert dist.max() < 1.0, "fault node coordinates do not match the golden grid"
    assert len(np.unique(gold[:, [0, 2]], axis=0)) == len(ours)
    tol = np.maximum(1e-3, 0.75 * _unit(gold))
    bad = np.abs(ours - gold) > tol
    if name == "tpv1053d":
        # fric(23) for friclaw 5 is an uninitialised local of NewtonRaphson in the reference
        # (src/faulting.f90:514, thetaPcTmp is never set when friclaw >= 5): undefined output.
        bad[:, FRT_COLUMNS.index("state_normal")] = False
    # rupture time: print-exact or within one time step
    j = FRT_COLUMNS.index("trup")
    bad[:, j] &= np.abs(ours[:, j] - gold[:, j]) > case.scalars.dt
    msg = {FRT_COLUMNS[k]: int(bad[:, k].sum()) for k in range(bad.shape[1]) if bad[:, k].any()}
    assert not bad.any(), f"{name}: entries outside print tolerance per column: {msg}"


def test_oracle_drv_a6_within_reference_sensitivity():
    """drv.a6 (plastic, fractal fault, RSF slip law) is round-off sensitive in the reference
    itself: before the rupture arrives the dip slip rate is round-off (~1e-19 m/s) and solveRSF
    multiplies its direction by the friction stress (src/faulting.f90:289), so a 1e-14 relative
    change of any input moves the final fields by the amounts bounded below.  The check is
    therefore (a) the on-fault station time series faultst000dp075 print-exact over the first 20
    steps and (b) the final frt fields within twice that self-sensitivity."""
    case, _ = _run("drv.a6")
    d = np.load(golden_path("drv.a6"))
    g = d["faultst_000dp075"]
    an = case.arrays["anonfs"].reshape(-1, 3)
    st = d["st_on_fault"]
    j = [k for k in range(case.sizes["numOnFaultSt"])
         if abs(st[an[k, 1] - 1][0]) < 1e-9 and abs(st[an[k, 1] - 1][1] + 7.5) < 1e-9][0]
    h = case.arrays["onFaultQuantHistSCECForm"].reshape(-1, case.nstep, 12)[j]
    ours = np.column_stack([h[:, 0], h[:, 7] / 1e6, -h[:, 9] / 1e6, h[:, 3]])
    gold = g[:, [0, 3, 7, 8]]
    n = 20
    assert np.all(np.abs(ours[:n] - gold[:n]) <= np.maximum(1e-12, 1.01 * _unit(gold[:n])))
    frt_o = frt_table(case)
    frt_g, _ = match_rows(frt_o, golden_frt(golden_path("drv.a6")))
    bounds = {"slip_s": 2e-2, "tnrm": 2e-3, "tstk": 7e-2, "peak_rate": 1.2e-1}
    for col, b in bounds.items():
        k = FRT_COLUMNS.index(col)
        rel = np.linalg.norm(frt_o[:, k] - frt_g[:, k]) / np.linalg.norm(frt_g[:, k])
        assert rel < b, (col, rel)
    k = FRT_COLUMNS.index("trup")
    n_o, n_g = (frt_o[:, k] < 1e4).sum(), (frt_g[:, k] < 1e4).sum()
    assert abs(n_o - n_g) <= 0.03 * n_g
