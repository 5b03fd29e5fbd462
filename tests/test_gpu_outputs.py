"""Output streams captured on the device (output_gm / output_src_evol frames of the steps with
mod(nt, 10) == 1, src/driver.f90:30-33): the frames match the oracle's velocities and fric(47) at
those steps, a full ring keeps the newest frames, and the files are the reference's byte layout."""
import os
import tempfile

import numpy as np
import pytest

from conftest import golden_path, nthreads

pytestmark = pytest.mark.gpu


def _oracle_frames(case, nodes, steps):
    from oracle import Oracle
    cpu = case.clone()
    o = Oracle(cpu, nthreads())
    gm, src, done = [], [], 0
    for nt in steps:
        o.step(nt - done)
        done = nt
        gm.append(cpu.arrays["velArr"].reshape(-1, 3)[nodes - 1].copy())
        src.append(cpu.fric()[:, 46].copy())
    return np.array(gm), np.array(src)


def test_output_frames_match_oracle():
    from eqdyna_gb300.case import Case
    from eqdyna_gb300.outputs import append_frames, surface_nodes
    from eqdyna_gb300.solver import GpuSolver
    case = Case.from_fixture(golden_path("tpv8"))
    nodes = surface_nodes(case)
    assert len(nodes) > 100
    with GpuSolver(case.clone(), precision="fp64") as s:
        s.output_setup(nodes, every=10, ring_frames=8)
        s.step(35)
        first, gm, src = s.output_drain()
        s.step(10)
        first2, gm2, src2 = s.output_drain()
    assert first == 1 and len(gm) == 4 and first2 == 41 and len(gm2) == 1
    ref_gm, ref_src = _oracle_frames(case, nodes, [1, 11, 21, 31, 41])
    gm_all, src_all = np.concatenate([gm, gm2]), np.concatenate([src, src2])
    sg = max(np.abs(ref_gm).max(), 1e-30)
    ss = max(np.abs(ref_src).max(), 1e-30)
    print("frames", gm_all.shape, "max |v|", sg, "max fric(47)", ss)
    assert np.abs(ref_gm).max() > 0.0
    assert np.abs(gm_all - ref_gm).max() <= 1e-9 * sg
    assert np.abs(src_all - ref_src).max() <= 1e-9 * ss
    d = tempfile.mkdtemp(prefix="eqd_out_")
    append_frames(d, gm_all, src_all, suffix="000000")
    raw = np.fromfile(os.path.join(d, "gm000000"), dtype=np.float64)
    assert raw.size == 5 * len(nodes) * 3 and np.array_equal(raw.reshape(5, len(nodes), 3), gm_all)


def test_output_ring_keeps_newest_frames_binary32():
    from eqdyna_gb300.case import Case
    from eqdyna_gb300.outputs import surface_nodes
    from eqdyna_gb300.solver import GpuSolver
    case = Case.from_fixture(golden_path("tpv8"))
    nodes = surface_nodes(case)
    g = case.clone()
    with GpuSolver(g, precision="fp32") as s:
        s.output_setup(nodes, every=10, ring_frames=2)
        s.step(41)          # frames at 1, 11, 21, 31, 41; the ring holds 31 and 41
        first, gm, src = s.output_drain()
        s.fetch()
    assert first == 31 and len(gm) == 2
    # the frame of step 41 is the state the full fetch reads after step 41
    assert np.array_equal(gm[1], g.arrays["velArr"].reshape(-1, 3)[nodes - 1])
    assert np.array_equal(src[1], g.fric()[:, 46])
