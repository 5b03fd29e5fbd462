"""Setup on the GPU: the per-element tables and nodal masses built on the device from the mesh.

* eqd_gpu_element_tables gives, bit for bit, the host setup's eleshp, eledet, elemass, ss, phi,
  nodalMassArr and fnms (the restatement of assembleGlobalMass, calcGlobalShapeFunc and
  calcSSPhi4Hrgls, src/assembleGlobalMass.f90:12-38,283-406, src/calcGlobalShapeFunc.f90:1-75) on
  meshes with a stretched PML and an inserted dipping interface (tpv10), wedges on a dipping
  fault (C3) and a rough fault (drv.a6).
* eqd_gpu_init on a mesh-only case (no host tables: it builds them on the device) runs the same
  steps as on the full case, in both precision forms; the tables are the same bits, so the runs
  differ only by the order of the L2 reductions (relative 1e-12 in binary64, 1e-5 in binary32).
"""
import ctypes as C
import tempfile

import numpy as np
import pytest

from conftest import golden_path

pytestmark = pytest.mark.gpu

TABLES = ("eleshp", "eledet", "elemass", "ss", "phi", "nodalMassArr", "fnms")


def _cases():
    from eqdyna_gb300.case import Case
    from eqdyna_gb300.configs import config_c3
    yield "tpv10", Case.from_fixture(golden_path("tpv10"))
    yield "drv.a6", Case.from_fixture(golden_path("drv.a6"))
    yield "C3/4", Case.from_dir(config_c3(tempfile.mkdtemp(prefix="eqd_c3s_"), scale=4.0, nsteps=10))


@pytest.mark.parametrize("idx", [0, 1, 2])
def test_device_tables_equal_host_tables_bit_for_bit(idx):
    from eqdyna_gb300 import _native as N
    name, case = list(_cases())[idx]
    lib = N.gpu_lib()
    a = case.arrays
    out = {k: np.full_like(a[k], np.nan) for k in TABLES}
    ptr = {k: v.ctypes.data_as(N.c_double_p) for k, v in out.items()}
    ha = case.host_arrays()
    rc = lib.eqd_gpu_element_tables(0, C.byref(ha), ptr["eleshp"], ptr["eledet"], ptr["elemass"], ptr["ss"],
                                    ptr["phi"], ptr["nodalMassArr"], ptr["fnms"])
    assert rc == 0
    assert (a["elemTypeArr"] >= 11).any() or name != "C3/4"  # the C3 mesh has wedges
    for k in TABLES:
        assert np.array_equal(out[k].view(np.uint64), a[k].view(np.uint64)), (name, k)


def _rel(x, y):
    return np.linalg.norm(x - y) / max(np.linalg.norm(y), 1e-300)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("fp32", 1e-5)])
def test_init_builds_the_tables_on_the_device(precision, tol):
    """C3 at dx = 400 m (wedges, learned guess off) and C1 at dx = 400 m (aging law, 40-layer PML
    scaled): 60 steps from a mesh-only case against 60 steps from the full case."""
    from eqdyna_gb300.case import Case
    from eqdyna_gb300.configs import config_c1, config_c3
    from eqdyna_gb300.solver import GpuSolver
    for mk in (lambda d: config_c3(d, scale=4.0, nsteps=60), lambda d: config_c1(d, scale=4.0, nsteps=60)):
        d = mk(tempfile.mkdtemp(prefix="eqd_sd_"))
        full, mesh = Case.from_dir(d), Case.from_dir(d, tables=False)
        assert all(mesh.arrays[k] is None for k in TABLES)
        with GpuSolver(full, precision=precision) as s:
            s.step(60)
            s.fetch()
        with GpuSolver(mesh, precision=precision) as s:
            s.step(60)
            s.fetch()
        rep = {k: _rel(mesh.arrays[k], full.arrays[k]) for k in ("velArr", "dispArr", "stressArr")}
        fa, fb = mesh.fric(), full.fric()
        rep["slip_rate"] = _rel(fa[:, 73:76], fb[:, 73:76])
        rep["slip"] = _rel(fa[:, 70:73], fb[:, 70:73])
        print(precision, mesh.sizes["nelem"], rep)
        assert np.abs(fb[:, 75]).max() > 0.0
        assert all(v <= tol for v in rep.values()), rep


def test_element_tables_reject_bad_input():
    from eqdyna_gb300 import _native as N
    lib = N.gpu_lib()
    assert lib.eqd_gpu_element_tables(0, None, None, None, None, None, None, None, None) == 1
