"""Failure detection, without faulting the GPU.

The reference stops the process on a NaN velocity (src/driver.f90:147-152) and on a non-positive
Jacobian (src/calcGlobalShapeFunc.f90:52-57).  The library returns a status instead and the
context stays usable:

* a NaN seeded into a host array before upload is reported by the step as EQD_ERR_NAN, in both
  precision forms;
* connectivity with a node id out of range is rejected by eqd_gpu_init (EQD_ERR_INPUT) before any
  device work; an inverted element is reported by the table build on the device;
* the device-side waits are bounded: a wait whose completion never comes (an mbarrier armed for
  bytes no copy delivers, a grid barrier one CTA never reaches) gives up and reports
  EQD_ERR_TIMEOUT, and the device runs the next job normally.
"""
import ctypes as C
import tempfile

import numpy as np
import pytest

from conftest import golden_path

pytestmark = pytest.mark.gpu


def _clean_run_works():
    from eqdyna_gb300.case import Case
    from eqdyna_gb300.solver import GpuSolver
    case = Case.from_fixture(golden_path("tpv8"))
    with GpuSolver(case, precision="fp32") as s:
        s.step(5)
        s.fetch()
    assert np.isfinite(case.arrays["velArr"]).all()


@pytest.mark.parametrize("which,lo_ms,hi_ms", [(0, 50.0, 2000.0), (1, 1000.0, 10000.0)])
def test_bounded_wait_gives_up_and_the_device_stays_usable(which, lo_ms, hi_ms):
    from eqdyna_gb300 import _native as N
    lib = N.gpu_lib()
    status, ms = C.c_int32(-1), C.c_double(0.0)
    assert lib.eqd_gpu_wait_selftest(0, which, C.byref(status), C.byref(ms)) == 0
    print("wait", which, "status", status.value, "after", ms.value, "ms")
    assert status.value == 7  # EQD_ERR_TIMEOUT
    assert lo_ms <= ms.value <= hi_ms
    _clean_run_works()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_nan_velocity_is_reported(precision):
    from eqdyna_gb300 import _native as N
    from eqdyna_gb300.case import Case
    from eqdyna_gb300.solver import GpuSolver
    case = Case.from_fixture(golden_path("tpv8"))
    bad = case.clone()
    # v1 holds the velocity of every equation (src/eqdyna3d.f90:191-212); equation 1 belongs to a
    # 3-DOF node
    bad.arrays["v1"][0] = np.nan
    with GpuSolver(bad, precision=precision) as s:
        with pytest.raises(N.EqdError) as ei:
            s.step(3)
        assert ei.value.code == 4  # EQD_ERR_NAN
        s.fetch()  # the context still answers
    _clean_run_works()


@pytest.mark.parametrize("tables", [True, False])
def test_node_id_out_of_range_is_rejected(tables):
    from eqdyna_gb300 import _native as N
    from eqdyna_gb300.case import Case
    from eqdyna_gb300.configs import config_c0
    from eqdyna_gb300.solver import GpuSolver
    case = Case.from_dir(config_c0(tempfile.mkdtemp(prefix="eqd_bad_"), scale=8.0, nsteps=5), tables=tables)
    conn = case.arrays["nodeElemIdRelation"].copy()
    conn[8 * 17 + 3] = case.sizes["nnode"] + 1
    case.arrays["nodeElemIdRelation"] = conn
    with pytest.raises(N.EqdError) as ei:
        GpuSolver(case, precision="fp32")
    assert ei.value.code == 1  # EQD_ERR_INPUT
    _clean_run_works()


def test_inverted_element_is_reported_by_the_device_table_build():
    """An element with its top and bottom faces exchanged has a negative Jacobian determinant: the
    table build on the device reports it (the host builder stops on it, as the reference does)."""
    from eqdyna_gb300 import _native as N
    from eqdyna_gb300.case import Case
    from eqdyna_gb300.configs import config_c0
    from eqdyna_gb300.solver import GpuSolver
    case = Case.from_dir(config_c0(tempfile.mkdtemp(prefix="eqd_inv_"), scale=8.0, nsteps=5), tables=False)
    conn = case.arrays["nodeElemIdRelation"].copy().reshape(-1, 8)
    e = 123
    conn[e] = np.concatenate([conn[e, 4:], conn[e, :4]])
    case.arrays["nodeElemIdRelation"] = conn.ravel()
    ha = case.host_arrays()
    lib = N.gpu_lib()
    det = np.zeros(case.sizes["nelem"])
    assert lib.eqd_gpu_element_tables(0, C.byref(ha), None, det.ctypes.data_as(N.c_double_p), None, None, None,
                                      None, None) == 1
    with pytest.raises(N.EqdError) as ei:
        GpuSolver(case, precision="fp64")
    assert ei.value.code == 1
    _clean_run_works()
