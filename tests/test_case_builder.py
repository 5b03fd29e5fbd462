"""Unit tests of the host case setup against hand-derived values (CPU only)."""
import numpy as np
import pytest

from conftest import golden_path


@pytest.fixture(scope="module")
def tpv8():
    from eqdyna_gb300.case import Case
    return Case.from_fixture(golden_path("tpv8"))


def test_uniform_cube_tables(tpv8):
    """For an undistorted cube of side h the one-point tables are: det = (h/2)^3,
    dN/dx_k = +-1/(4h) (src/calcGlobalShapeFunc.f90), lumped mass rho*h^3/8 per node
    (src/assembleGlobalMass.f90:376-406) and hourglass vectors equal to the +-1 base patterns
    (src/assembleGlobalMass.f90:353-373)."""
    c = tpv8
    et = c.arrays["elemTypeArr"]
    conn = c.arrays["nodeElemIdRelation"].reshape(-1, 8)
    xyz = c.arrays["meshCoor"].reshape(-1, 3)
    h = 500.0
    # pick an interior element well inside the uniform region
    ctr = xyz[conn - 1].mean(axis=1)
    e = int(np.argmin(np.abs(ctr[:, 0] - 250) + np.abs(ctr[:, 1] - 1250) + np.abs(ctr[:, 2] + 5250)))
    assert et[e] == 1
    ext = xyz[conn[e] - 1].max(0) - xyz[conn[e] - 1].min(0)
    assert np.allclose(ext, h)
    assert c.arrays["eledet"][e] == pytest.approx((h / 2) ** 3, rel=1e-12)
    shp = c.arrays["eleshp"].reshape(-1, 8, 3)[e]
    assert np.allclose(np.abs(shp), 1 / (4 * h), rtol=1e-12)
    rho = c.arrays["mat"].reshape(5, -1)[2, e]
    assert np.allclose(c.arrays["elemass"].reshape(-1, 24)[e], rho * h ** 3 / 8, rtol=1e-12)
    phi = c.arrays["phi"].reshape(-1, 4, 8)[e]
    assert np.allclose(np.abs(phi), 1.0, atol=1e-9)
    # hourglass vectors are orthogonal to the linear fields x, y, z and to constants
    X = xyz[conn[e] - 1]
    assert np.allclose(phi @ X, 0.0, atol=1e-6)
    assert np.allclose(phi.sum(axis=1), 0.0, atol=1e-9)


def test_mass_and_equation_bookkeeping(tpv8):
    c = tpv8
    a = c.arrays
    ne = c.sizes["nelem"]
    rho = a["mat"].reshape(5, -1)[2]
    vol = a["eledet"] * 8.0
    total = (rho * vol).sum()
    # every node's fnms sums the element masses (one DOF's worth); totals agree
    assert a["fnms"].sum() == pytest.approx(total, rel=1e-12)
    ndof = a["numOfDofPerNodeArr"]
    assert set(np.unique(ndof)) <= {3, 12}
    assert a["eqNumIndexArr"].size == ndof.sum()
    eqs = a["eqNumIndexArr"]
    assert eqs.max() == c.sizes["neq"]
    assert np.array_equal(np.sort(eqs[eqs > 0]), np.arange(1, c.sizes["neq"] + 1))
    # PML elements take 21 stress slots, the others 12
    et = a["elemTypeArr"]
    assert a["stressArr"].size == 21 * (et == 2).sum() + 12 * (et != 2).sum()
    assert ne == (c.dims["nx"] - 1) * (c.dims["ny"] - 1) * (c.dims["nz"] - 1)


def test_split_nodes(tpv8):
    c = tpv8
    nsmp = c.arrays["nsmp"].reshape(-1, 2)
    xyz = c.arrays["meshCoor"].reshape(-1, 3)
    assert np.array_equal(xyz[nsmp[:, 0] - 1], xyz[nsmp[:, 1] - 1])
    # master nodes are appended after the nx*ny*nz grid nodes (src/meshgen.f90:805)
    ngrid = c.dims["nx"] * c.dims["ny"] * c.dims["nz"]
    assert np.array_equal(nsmp[:, 1], ngrid + np.arange(1, len(nsmp) + 1))
    # elements on the +y side of the fault use master nodes; none uses a slave there
    conn = c.arrays["nodeElemIdRelation"].reshape(-1, 8)
    ctr = xyz[conn - 1].mean(axis=1)
    plus = (ctr[:, 1] > 0) & (ctr[:, 1] < 500)
    uses_master = np.isin(conn[plus], nsmp[:, 1]).any(axis=1)
    p = xyz[conn[plus] - 1]
    on_fault = ((np.abs(p[:, :, 1]) < 1e-9) & (np.abs(p[:, :, 0]) <= 15e3 + 1e-6)
                & (p[:, :, 2] >= -15e3 - 1e-6))
    # The reference rewires an element only when its last-created corner node lies below
    # fxmax + dx (src/meshgen.f90:751-754).  With stretched cells (rat = 1.025) the column just
    # beyond the +x fault edge is 512.5 m wide, so those elements keep the slave nodes.
    reachable = p[:, :, 0].max(axis=1) < 15e3 + 500.0 + 1e-5
    assert np.array_equal(uses_master, on_fault.any(axis=1) & reachable)
    uses_slave = np.isin(conn[plus], nsmp[:, 0]).any(axis=1)
    assert np.array_equal(uses_slave, on_fault.any(axis=1) & ~reachable)
    # fault areas sum to the fault area
    assert c.arrays["arn"].sum() == pytest.approx(30e3 * 15e3, rel=1e-12)


_HASH_SCRIPT = """
import hashlib, sys, tempfile
from eqdyna_gb300 import configs
from eqdyna_gb300.case import Case
d = tempfile.mkdtemp(prefix="eqd_thr_")
configs.CONFIGS[sys.argv[1]](d, scale=float(sys.argv[2]), nsteps=20)
c = Case.from_dir(d)
for k, v in sorted(c.arrays.items()):
    print(k, None if v is None else hashlib.sha1(v.tobytes()).hexdigest())
"""


@pytest.mark.parametrize("config,scale", [("C0", 4.0), ("C3", 8.0)])
def test_tables_independent_of_thread_count(config, scale):
    """The parallel setup (per-element tables, nodal masses assembled plane by plane in element
    order, parallel first touch) gives the same bytes with one host thread as with all of them."""
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    out = []
    for threads in ("1", str(max(os.cpu_count() or 2, 2))):
        env = dict(os.environ, OMP_NUM_THREADS=threads, PYTHONPATH=root)
        r = subprocess.run([sys.executable, "-c", _HASH_SCRIPT, config, str(scale)], env=env,
                           capture_output=True, text=True, timeout=600, cwd=root)
        assert r.returncode == 0, r.stderr
        out.append(r.stdout)
    assert out[0] == out[1] and "nodalMassArr" in out[0]


def test_arrays_outlive_the_case_and_clones_are_private():
    """Case.from_dir hands out views of the builder's arrays without copying: an array kept after
    its case is gone stays valid (the builder is freed with the last view), the views are writable,
    and a clone's state arrays are private copies."""
    import gc
    import tempfile
    from eqdyna_gb300.case import Case
    from eqdyna_gb300.configs import config_c0
    case = Case.from_dir(config_c0(tempfile.mkdtemp(prefix="eqd_view_"), scale=4.0, nsteps=5))
    assert set(case.build_phases_s) >= {"mesh", "element_tables", "views"}
    coor = case.arrays["meshCoor"]
    expect = float(coor.sum())
    twin = case.clone()
    twin.arrays["velArr"][:] = 1.0
    assert not case.arrays["velArr"].any()
    case.arrays["dispArr"][:3] = 2.0  # writable view
    del case, twin
    gc.collect()
    assert float(coor.sum()) == expect


TABLES = ("eleshp", "eledet", "elemass", "ss", "phi", "nodalMassArr", "fnms")


def test_mesh_only_build_has_everything_but_the_tables():
    """Case.from_dir(tables=False) (eqd_case_build_opt with EQD_CASE_MESH_ONLY) leaves the seven
    table arrays out, for eqd_gpu_init to build them on the device, and gives every other array
    byte for byte as the full build does (a C3 mesh: wedges, a dipping fault, a stretched PML)."""
    import tempfile
    from eqdyna_gb300.case import Case
    from eqdyna_gb300.configs import config_c3
    d = config_c3(tempfile.mkdtemp(prefix="eqd_c3m_"), scale=4.0, nsteps=10)
    full, mesh = Case.from_dir(d), Case.from_dir(d, tables=False)
    for k, v in full.arrays.items():
        if k in TABLES:
            assert v is not None and mesh.arrays[k] is None, k
        elif v is None:
            assert mesh.arrays[k] is None, k
        else:
            assert np.array_equal(v, mesh.arrays[k]), k
    assert full.sizes == mesh.sizes
    assert bytes(full.scalars) == bytes(mesh.scalars)
