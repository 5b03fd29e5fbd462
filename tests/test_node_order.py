"""The device node order eqd_gpu_init uses (eqd_host_node_order, host only).

The order is: split nodes of the first fault, the other 3-DOF nodes, padding to a multiple of 32,
PML nodes with equations, fixed PML nodes (every equation -1, src/driver.f90:141-144), padding to
a multiple of 32. The mesh order is kept within each class. The binary32 node update tells a node's
class by its device index, and the padding aligns every component array. These tests check that
every mesh node appears exactly once, the class boundaries, the padding, and the rejected inputs.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import golden_path


def _order(case):
    from eqdyna_gb300 import _native as N
    lib = N.gpu_lib()
    ha = case.host_arrays()
    n, counts = C.c_int64(), (C.c_int32 * 4)()
    assert lib.eqd_host_node_order(C.byref(ha), None, 0, C.byref(n), counts) == 0
    out = np.empty(n.value, dtype=np.int32)
    rc = lib.eqd_host_node_order(C.byref(ha), out.ctypes.data_as(C.POINTER(C.c_int32)), n.value, C.byref(n),
                                 counts)
    assert rc == 0
    return out, list(counts)


def _classes(case):
    """The four classes of mesh nodes (0-based ids, mesh order) from the host arrays."""
    a = case.arrays
    dof = a["numOfDofPerNodeArr"]
    nft = int(a["nftnd"][0]) if case.sizes.get("ntotft", 0) >= 1 else 0
    split = np.zeros(len(dof), dtype=bool)
    split[a["nsmp"][: 2 * nft] - 1] = True
    loc = a["eqNumStartIndexLoc"].astype(np.int64)  # 0-based position of a node's first equation
    eq1 = a["eqNumIndexArr"][loc]
    ids = np.arange(len(dof))
    return (ids[(dof == 3) & split], ids[(dof == 3) & ~split], ids[(dof == 12) & (eq1 > 0)],
            ids[(dof == 12) & (eq1 <= 0)])


@pytest.fixture(scope="module", params=["tpv8", "drv.a6"])
def case(request):
    from eqdyna_gb300.case import Case
    return Case.from_fixture(golden_path(request.param))


def test_every_mesh_node_once_and_ranges_aligned(case):
    out, (n_split, n_int, npml_live, nd) = _order(case)
    nn = case.sizes["nnode"]
    assert nd == len(out) and nd % 32 == 0 and n_int % 32 == 0
    live = out[out >= 0]
    assert len(live) == nn and np.array_equal(np.sort(live), np.arange(nn))
    assert (out < 0).sum() == nd - nn
    assert (out[:n_int] < 0).sum() < 32 and (out[n_int:] < 0).sum() < 32


def test_class_boundaries_follow_the_node_update(case):
    out, (n_split, n_int, npml_live, nd) = _order(case)
    split, other3, pml_live, pml_fixed = _classes(case)
    assert n_split == len(split) > 0
    assert np.array_equal(out[:n_split], split)
    k = n_split + len(other3)
    assert np.array_equal(out[n_split:k], other3)
    assert np.all(out[k:n_int] == -1)
    assert npml_live == len(pml_live)
    assert np.array_equal(out[n_int:n_int + npml_live], pml_live)
    f = n_int + npml_live
    assert np.array_equal(out[f:f + len(pml_fixed)], pml_fixed)
    assert np.all(out[f + len(pml_fixed):] == -1)


def test_rejected_inputs(case):
    from eqdyna_gb300 import _native as N
    lib = N.gpu_lib()
    n, counts = C.c_int64(), (C.c_int32 * 4)()
    out, _ = _order(case)
    small = np.empty(len(out) - 1, dtype=np.int32)
    ha = case.host_arrays()
    assert lib.eqd_host_node_order(C.byref(ha), small.ctypes.data_as(C.POINTER(C.c_int32)), len(small),
                                   C.byref(n), counts) == 1
    bad = case.clone()
    dof = bad.arrays["numOfDofPerNodeArr"].copy()
    dof[7] = 5  # neither 3 nor 12 degrees of freedom
    bad.arrays["numOfDofPerNodeArr"] = dof
    ha = bad.host_arrays()
    assert lib.eqd_host_node_order(C.byref(ha), None, 0, C.byref(n), counts) == 1
    bad = case.clone()
    nsmp = bad.arrays["nsmp"].copy()
    nsmp[3] = case.sizes["nnode"] + 1  # a split node outside the mesh
    bad.arrays["nsmp"] = nsmp
    ha = bad.host_arrays()
    assert lib.eqd_host_node_order(C.byref(ha), None, 0, C.byref(n), counts) == 1
