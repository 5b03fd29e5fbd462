"""eqd_gpu_elem_forces_noalloc: the element force pass for callers that cannot allocate device
memory (their arrays are already on the GPU, e.g. under OpenACC or CUDA Fortran data management,
or all device memory is planned at start-up).  The entry point keeps its per-node accumulator in
a fixed static device array, so it must give the same forces and stresses as the time step of the
context API (eqd_gpu_init / eqd_gpu_step / eqd_gpu_fetch), on two calls in a row: the second call
must not see anything left in the shared accumulator by the first.  The device tables cannot be
checked on the host, so the kernel checks node ids and stress offsets itself: an element with a
bad id is skipped and reported (EQD_ERR_INPUT) without a memory fault, the other elements' forces
are those of the good tables, and the next call with good tables is clean again.

This file is collected last on purpose, and passes both alone in a fresh process and after the
rest of the suite.
"""
import ctypes as C
import tempfile

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-9


class ElemDeviceView(C.Structure):
    _fields_ = [("nnode", C.c_int32), ("nelem", C.c_int32),
                ("nodeElemIdRelation", C.c_void_p), ("elemTypeArr", C.c_void_p),
                ("eleshp", C.c_void_p), ("eledet", C.c_void_p), ("mat", C.c_void_p),
                ("ss", C.c_void_p), ("phi", C.c_void_p), ("stressArr", C.c_void_p),
                ("stressCompIndexArr", C.c_void_p), ("velArr", C.c_void_p),
                ("dispArr", C.c_void_p), ("dt", C.c_double), ("rdampk", C.c_double),
                ("w", C.c_double), ("size_stress", C.c_int64), ("C_elastic", C.c_int32),
                ("C_Q", C.c_int32), ("C_hg", C.c_int32)]


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def test_noalloc_element_forces_match_the_step_on_two_calls():
    torch = pytest.importorskip("torch")
    from eqdyna_gb300 import _native as N
    from eqdyna_gb300.case import Case
    from eqdyna_gb300.configs import config_c0
    from eqdyna_gb300.solver import GpuSolver

    lib = N.gpu_lib()
    lib.eqd_gpu_elem_forces_noalloc.argtypes = [C.POINTER(ElemDeviceView), C.c_void_p, C.c_void_p]
    lib.eqd_gpu_elem_forces_noalloc.restype = C.c_int

    case = Case.from_dir(config_c0(tempfile.mkdtemp(prefix="eqd_noalloc_"), scale=4.0, nsteps=10))
    a = case.arrays
    nn, ne = case.sizes["nnode"], case.sizes["nelem"]
    assert nn <= 524288
    dev = torch.device("cuda:0")
    t = lambda x: torch.from_numpy(np.ascontiguousarray(x)).to(dev)
    d_conn, d_type = t(a["nodeElemIdRelation"]), t(a["elemTypeArr"])
    d_shp, d_det, d_mat = t(a["eleshp"]), t(a["eledet"]), t(a["mat"])
    d_ss, d_phi, d_sidx = t(a["ss"]), t(a["phi"]), t(a["stressCompIndexArr"])
    d_stress = t(a["stressArr"].copy())
    d_force = torch.full((3 * nn,), np.nan, dtype=torch.float64, device=dev)  # garbage in

    # nodes whose force is the interior-element sum alone (no PML element, not a split node)
    et = a["elemTypeArr"]
    conn = a["nodeElemIdRelation"].reshape(-1, 8) - 1
    only = np.ones(nn, dtype=bool)
    only[np.unique(conn[et == 2])] = False
    only[a["nsmp"].reshape(-1, 2)[: case.npair].ravel() - 1] = False
    only &= a["numOfDofPerNodeArr"] == 3
    eq = a["eqNumIndexArr"]
    loc = a["eqNumStartIndexLoc"]
    eq3 = np.stack([eq[loc + k] for k in range(3)], axis=1)  # (nn, 3) 1-based equations
    sel = np.where(only)[0]
    interior_stress = (a["stressCompIndexArr"][et != 2][:, None] + np.arange(6)[None, :]).ravel()

    def make_view(d_conn, d_vel, d_disp, **switches):
        sw = {"C_elastic": 1, "C_Q": 0, "C_hg": 1}
        sw.update(switches)
        return ElemDeviceView(nn, ne, d_conn.data_ptr(), d_type.data_ptr(), d_shp.data_ptr(),
                              d_det.data_ptr(), d_mat.data_ptr(), d_ss.data_ptr(),
                              d_phi.data_ptr(), d_stress.data_ptr(), d_sidx.data_ptr(),
                              d_vel.data_ptr(), d_disp.data_ptr(), case.scalars.dt,
                              case.scalars.rdampk, case.scalars.w, int(a["stressArr"].size),
                              sw["C_elastic"], sw["C_Q"], sw["C_hg"])

    ref = case.clone()
    stream = torch.cuda.current_stream(dev)
    with GpuSolver(ref, use_graph=False) as s:
        # advance until the rupture has set the medium in motion; the next two steps are compared
        s.step(20)
        s.fetch()
        d_stress.copy_(t(ref.arrays["stressArr"]))
        for call in range(2):
            prev_stress = d_stress.cpu().numpy()
            s.step(1)
            s.fetch()
            d_vel, d_disp = t(ref.arrays["velArr"]), t(ref.arrays["dispArr"])
            view = make_view(d_conn, d_vel, d_disp)
            rc = lib.eqd_gpu_elem_forces_noalloc(C.byref(view), C.c_void_p(d_force.data_ptr()),
                                                 C.c_void_p(stream.cuda_stream))
            assert rc == 0
            torch.cuda.synchronize(dev)
            force = d_force.cpu().numpy().reshape(nn, 3)
            stress = d_stress.cpu().numpy()
            assert np.isfinite(force).all()
            assert np.abs(force[sel]).max() > 0 and np.abs(stress[interior_stress]).max() > 0
            # stresses after this step, interior elements
            assert _rel(stress[interior_stress], ref.arrays["stressArr"][interior_stress]) <= TOL
            # forces: the step stores acceleration F/m in nodalForceArr
            acc = ref.arrays["nodalForceArr"][eq3[sel] - 1]
            mass = ref.arrays["nodalMassArr"][eq3[sel] - 1]
            assert _rel(force[sel], acc * mass) <= TOL, f"call {call + 1}"
        good_force = force.copy()
        good_stress = stress.copy()

        # one interior element with a node id above nnode, another with a 0-based id (0): both are
        # skipped on the device, the call reports EQD_ERR_INPUT, nothing faults
        interior = np.where(et != 2)[0]
        bad = [int(interior[len(interior) // 3]), int(interior[2 * len(interior) // 3])]
        conn_bad = a["nodeElemIdRelation"].copy().reshape(-1, 8)
        conn_bad[bad[0], 3] = nn + 5
        conn_bad[bad[1], 0] = 0
        d_conn_bad = t(conn_bad.ravel())
        d_stress.copy_(t(prev_stress))
        view = make_view(d_conn_bad, d_vel, d_disp)
        rc = lib.eqd_gpu_elem_forces_noalloc(C.byref(view), C.c_void_p(d_force.data_ptr()),
                                             C.c_void_p(stream.cuda_stream))
        assert rc == 1, rc
        torch.cuda.synchronize(dev)
        force_bad = d_force.cpu().numpy().reshape(nn, 3)
        stress_bad = d_stress.cpu().numpy()
        # the skipped elements kept their stress; every other element was updated as before
        for e in bad:
            o = a["stressCompIndexArr"][e]
            assert np.array_equal(stress_bad[o:o + 6], prev_stress[o:o + 6])
        keep = np.ones(stress_bad.size, dtype=bool)
        for e in bad:
            o = a["stressCompIndexArr"][e]
            keep[o:o + 6] = False
        assert np.array_equal(stress_bad[keep & np.isin(np.arange(stress_bad.size), interior_stress)],
                              good_stress[keep & np.isin(np.arange(stress_bad.size), interior_stress)])
        # nodes of the skipped elements lost those elements' forces; all others are unchanged
        touched = np.zeros(nn, dtype=bool)
        touched[conn[bad].ravel()] = True
        other = ~touched
        assert np.isfinite(force_bad).all()
        assert _rel(force_bad[other], good_force[other]) <= TOL

        # the next call with good tables is clean: the skip count and accumulator start afresh
        d_stress.copy_(t(prev_stress))
        view = make_view(d_conn, d_vel, d_disp)
        rc = lib.eqd_gpu_elem_forces_noalloc(C.byref(view), C.c_void_p(d_force.data_ptr()),
                                             C.c_void_p(stream.cuda_stream))
        assert rc == 0
        torch.cuda.synchronize(dev)
        assert _rel(d_force.cpu().numpy().reshape(nn, 3)[sel], good_force[sel]) <= TOL

        # switches the pass does not implement are refused before any launch
        for sw in ({"C_hg": 2}, {"C_elastic": 0}, {"C_Q": 1}):
            view = make_view(d_conn, d_vel, d_disp, **sw)
            assert lib.eqd_gpu_elem_forces_noalloc(C.byref(view), C.c_void_p(d_force.data_ptr()),
                                                   C.c_void_p(stream.cuda_stream)) == 5, sw

    # sizes beyond the fixed scratch are refused before any launch
    big = ElemDeviceView(524289, 1, size_stress=0, C_elastic=1, C_Q=0, C_hg=1)
    assert lib.eqd_gpu_elem_forces_noalloc(C.byref(big), C.c_void_p(d_force.data_ptr()), None) == 1
