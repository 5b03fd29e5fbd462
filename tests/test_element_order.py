"""The element order the binary32 tiles are cut from (eqd_host_element_order, host only): every
element exactly once, empty slots only at the end of a tile, the same order for any number of host
threads, and sparse orders repacked (C3's stretched PML cells)."""
import ctypes as C
import os
import subprocess
import sys
import tempfile

import numpy as np
import pytest

from conftest import ROOT

TILE = 128


def _order(case, group, tile_shape=0):
    from eqdyna_gb300 import _native as N
    lib = N.gpu_lib()
    ha = case.host_arrays()
    n, live = C.c_int64(), C.c_double()
    assert lib.eqd_host_element_order(C.byref(ha), group, tile_shape, None, 0, C.byref(n), C.byref(live)) == 0
    out = np.empty(n.value, dtype=np.int32)
    rc = lib.eqd_host_element_order(C.byref(ha), group, tile_shape, out.ctypes.data_as(C.POINTER(C.c_int32)),
                                    n.value, C.byref(n), C.byref(live))
    assert rc == 0
    return out, live.value


@pytest.fixture(scope="module")
def c3_case():
    from eqdyna_gb300.case import Case
    from eqdyna_gb300.configs import config_c3
    return Case.from_dir(config_c3(tempfile.mkdtemp(prefix="eqd_ord_"), scale=4.0, nsteps=10))


def _check_tiles(order, members):
    # the last tile may be partial (the kernels cut ceil(len / TILE) tiles)
    order = np.concatenate([order, np.full(-len(order) % TILE, -1, dtype=order.dtype)])
    live = order[order >= 0]
    assert np.array_equal(np.sort(live), np.sort(members))  # every element exactly once
    t = order.reshape(-1, TILE) >= 0
    # the elements of a tile are its first slots: no element after an empty slot
    assert not (np.diff(t.astype(np.int8), axis=1) > 0).any()
    assert t[:, 0].all()


@pytest.mark.parametrize("group", [0, 1])
def test_every_element_once_and_padding_at_tile_ends(c3_case, group):
    et = c3_case.arrays["elemTypeArr"]
    members = np.flatnonzero((et == 1) | (et > 10)) if group == 0 else np.flatnonzero(et == 2)
    order, live = _order(c3_case, group)
    _check_tiles(order, members)
    slots = -(-len(order) // TILE) * TILE
    assert abs(live - len(members) / slots) < 1e-12


def test_sparse_pml_order_is_repacked(c3_case):
    """With the default 4 x 8 x 4 brick, bins of the median element width leave 49 % of C3's PML
    slots empty; bins by rank leave 28 % (the same figures as the GPU's table_info)."""
    _, live_pml = _order(c3_case, 1)
    _, live_int = _order(c3_case, 0)
    print("live slots: interior", live_int, "pml", live_pml)
    assert live_pml >= 0.7 and live_int >= 0.75


def test_uniform_mesh_keeps_the_tuned_brick():
    """C1 (uniform cells) at dx = 200 m with the tuned 2 x 16 x 4 brick: every element once, empty
    slots only at tile ends, and most slots live (nine in ten at dx = 100 m)."""
    from eqdyna_gb300.case import Case
    from eqdyna_gb300.configs import config_c1
    case = Case.from_dir(config_c1(tempfile.mkdtemp(prefix="eqd_ord1_"), scale=2.0, nsteps=10))
    et = case.arrays["elemTypeArr"]
    order, live = _order(case, 0, 2 | 16 << 8 | 4 << 16)
    _check_tiles(order, np.flatnonzero((et == 1) | (et > 10)))
    assert live > 0.85


_HASH = """
import hashlib, sys, tempfile
sys.path.insert(0, "tests")
import numpy as np
from eqdyna_gb300.case import Case
from eqdyna_gb300.configs import config_c3
from test_element_order import _order
case = Case.from_dir(config_c3(tempfile.mkdtemp(prefix="eqd_ordh_"), scale=8.0, nsteps=10))
for g in (0, 1):
    o, live = _order(case, g)
    print(g, hashlib.sha1(o.tobytes()).hexdigest(), repr(live))
"""


def test_order_independent_of_thread_count():
    out = []
    for threads in ("1", str(max(os.cpu_count() or 2, 2))):
        env = dict(os.environ, OMP_NUM_THREADS=threads, PYTHONPATH=ROOT)
        r = subprocess.run([sys.executable, "-c", _HASH], env=env, capture_output=True, text=True,
                           timeout=600, cwd=ROOT)
        assert r.returncode == 0, r.stderr
        out.append(r.stdout)
    assert out[0] == out[1] and out[0].count("\n") == 2


def test_rejects_bad_arguments(c3_case):
    from eqdyna_gb300 import _native as N
    lib = N.gpu_lib()
    ha = c3_case.host_arrays()
    n, live = C.c_int64(), C.c_double()
    assert lib.eqd_host_element_order(C.byref(ha), 2, 0, None, 0, C.byref(n), C.byref(live)) != 0
    small = np.empty(4, dtype=np.int32)
    rc = lib.eqd_host_element_order(C.byref(ha), 1, 0, small.ctypes.data_as(C.POINTER(C.c_int32)), 4,
                                    C.byref(n), C.byref(live))
    assert rc != 0 and n.value > 4


def test_node_id_out_of_range_is_rejected_before_any_coordinate_is_read(c3_case):
    """The element order reads the coordinates of every element's nodes; a connectivity with a node
    id outside 1 .. nnode (here one past the end, and a 0-based 0) is refused first (EQD_ERR_INPUT)
    rather than read past the caller's coordinate array.  eqd_gpu_init makes the same check
    before anything else."""
    from eqdyna_gb300 import _native as N
    lib = N.gpu_lib()
    for bad_id in (c3_case.sizes["nnode"] + 1, 0):
        case = c3_case.clone()
        conn = case.arrays["nodeElemIdRelation"].copy()
        conn[8 * 5 + 2] = bad_id
        case.arrays["nodeElemIdRelation"] = conn
        ha = case.host_arrays()
        n, live = C.c_int64(), C.c_double()
        assert lib.eqd_host_element_order(C.byref(ha), 0, 0, None, 0, C.byref(n), C.byref(live)) == 1
