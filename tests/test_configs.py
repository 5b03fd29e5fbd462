"""Configuration generators (CPU): the C3 dipping thrust builds wedge pairs along the fault and starts
in equilibrium away from its nucleation patch; C4 members differ in mesh size and stress field."""
import tempfile

import numpy as np

from conftest import nthreads


def test_c3_wedges_and_initial_equilibrium():
    from eqdyna_gb300.case import Case
    from eqdyna_gb300.configs import config_c3
    from oracle import Oracle
    case = Case.from_dir(config_c3(tempfile.mkdtemp(prefix="eqd_c3_"), scale=8.0, nsteps=10))
    et = case.arrays["elemTypeArr"]
    assert (et == 11).sum() > 0 and (et == 11).sum() == (et == 12).sum() and (et == 13).sum() > 0
    assert case.scalars.friclaw == 4
    fr = case.fric()
    # creep along the initial shear (dip direction): fric(26) = 0, fric(27) = Vini
    assert np.all(fr[:, 25] == 0.0) and np.all(fr[:, 26] == fr[:, 45])
    xyz = case.fault_coords()
    sd = np.sin(np.radians(30.0))
    downdip = np.abs(xyz[:, 2]) / sd
    patch = np.hypot(xyz[:, 0], downdip - 10.0e3) <= 2.0e3 + 1.0
    assert patch.sum() >= 1
    o = Oracle(case, nthreads())
    o.step(3)
    fr = case.fric()
    rate = np.hypot(fr[:, 73], fr[:, 74])
    far = np.hypot(xyz[:, 0], downdip - 10.0e3) > 6.0e3
    assert rate[patch].max() > 0.01          # the overstressed patch slips at once
    assert rate[far].max() < 1e-9            # the background stays at its creep rate
    o.close()


def test_c4_members_differ():
    from eqdyna_gb300.case import Case
    from eqdyna_gb300.configs import config_c4
    dx, tau = set(), []
    for m in range(6):
        c = Case.from_dir(config_c4(tempfile.mkdtemp(prefix="eqd_c4_"), m, nsteps=4))
        dx.add(round(c.scalars.dx))
        tau.append(float(c.fric()[:, 7].std()))
    assert len(dx) >= 2
    assert all(t > 0.0 for t in tau) and len({round(t, 3) for t in tau}) == len(tau)


def test_c2_layers_and_switches():
    import pytest
    from eqdyna_gb300.case import Case
    from eqdyna_gb300.configs import c2_layers, config_c2
    rows = c2_layers(50.0)
    assert rows.shape[1] == 4 and rows[-1, 0] == 1.0e6
    assert abs(rows[0, 2] - 1506.25) < 1e-9 and rows[-1, 2] == 3500.0   # Vs at 25 m and below 8 km
    assert np.allclose(rows[:, 1], 1.73 * rows[:, 2])
    assert np.all(np.diff(rows[:, 3]) >= 0.0)
    case = Case.from_dir(config_c2(tempfile.mkdtemp(prefix="eqd_c2_"), scale=8.0, nsteps=4))
    assert case.scalars.C_Q == 2 and case.scalars.C_elastic == 0
    vs = case.arrays["mat"].reshape(5, -1)[1]
    assert vs.min() < 2000.0 and vs.max() == 3500.0
    with pytest.raises(ValueError):
        config_c2(tempfile.mkdtemp(prefix="eqd_c2_"), scale=8.0, nsteps=4, q=1, plastic=True)


def test_surface_nodes_follow_find_surface_node_id_arr():
    from conftest import golden_path
    from eqdyna_gb300.case import Case
    from eqdyna_gb300.outputs import _e18, surface_nodes
    case = Case.from_fixture(golden_path("tpv8"))
    nodes = surface_nodes(case)
    xyz = case.arrays["meshCoor"].reshape(-1, 3)
    assert len(nodes) > 0 and nodes.min() >= 1
    assert np.all(np.abs(xyz[nodes - 1, 2]) < case.scalars.dx / 1000.0)
    top = np.flatnonzero(np.abs(xyz[:, 2]) < case.scalars.dx / 1000.0)
    assert len(top) >= len(nodes)
    assert _e18(-2.5e-3) == "  -0.2500000E-0002" and _e18(1000.0) == "   0.1000000E+0004"
