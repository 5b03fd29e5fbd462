"""Synthetic inputs for the benchmark configurations (no external dataset exists for them).

Each config is written as an ordinary case directory (same files the reference's case.setup
writes, see eqdyna_gb300.case), seeded with 20261203 + config id.

  C0  slip-weakening, homogeneous half-space, box x[-15,15] y[-10,10] z[-15,0] km, dx = 200 m
      (150 x 100 x 75 physical + 6 PML layers = 1,469,664 elements), fault x[-12,12] z[-12,0] km,
      mu_s 0.70 / mu_d 0.50 / Dc 0.3 m, sigma_n -100 MPa, tau0 60 MPa, 3 x 3 km patch at
      (0, -7.5 km) with tau0 72 MPa, strength barrier on the fault edge, dt 0.008 s, 1000 steps,
      20 on-fault + 20 surface stations at seeded uniform positions.
  C1  rate-and-state aging law on the same box at dx = 100 m with a 4 km PML (40 layers,
      380 x 280 x 190 = 20,216,000 elements), a in [0.008, 0.016] rising smoothly outside a
      velocity-weakening core (b = 0.012), L 0.02 m, V0 1e-6 m/s, f0 0.6, initial V 1e-12 m/s,
      241 x 121 fault node pairs, sigma_n -100 MPa, tau0 60 MPa, smooth 25 MPa overstress
      nucleation of radius 3 km at (0, -7.5 km) (TPV104 form), dt 0.004 s,
      4000 steps.
  C4  64 members of the C0 box, each at a seeded dx from {200, 250, 300, 400} m with its own dt,
      von Karman initial shear stress (correlation 1-4 km, Hurst 0.8, 5-15 %), seeded
      hypocentre; advanced as one ensemble, 1500 steps.
  C3  30-degree dipping reverse fault reaching the surface, degenerated wedge elements along
      the fault, slip law, depth-dependent sigma_n (16.2 MPa/km, capped at 120 MPa),
      tau0/sigma_n 0.55 with a 2 km circular patch at 0.75.

``scale`` > 1 coarsens dx by that factor (same shapes, fewer elements) for parity tests.
"""
import math

import numpy as np

from .case import NC_FIELDS, write_case_dir

SEED0 = 20261203

_NC_INDEX = {k: i for i, (_, k) in enumerate(NC_FIELDS)}


def _smooth_box(x, w_flat, w_taper):
    """1 inside |x| <= w_flat, 0 beyond w_flat + w_taper, C-infinity transition in between
    (the boxcar of TPV104/105)."""
    ax = abs(x)
    if ax <= w_flat:
        return 1.0
    if ax >= w_flat + w_taper:
        return 0.0
    return 0.5 * (1.0 + math.tanh(w_taper / (ax - w_flat - w_taper) + w_taper / (ax - w_flat)))


def _base_params():
    return dict(mode=1, C_elastic=1, C_nuclea=0, C_degen=0, insertFaultType=0, friclaw=1,
                ntotft=1, nucfault=1, tpv=0, output_plastic=0, outputGroundMotion=0,
                outputFinalSurfDisp=0, nx=1, ny=1, nz=1, term=1.0, dt=0.008, nmat=1, n2mat=3,
                roumax=2670.0, rhow=1000.0, gamar=0.66, rdampk=0.1, vmaxPML=6000.0,
                xsource=0.0, ysource=0.0, zsource=-7.5e3, nucR=3.0e3, nucRuptVel=-9999.0,
                nucdtau0=0.0, nucT=1.0, str1ToFaultAngle=45.0, devStrToStrVertRatio=0.33,
                bulk=0.75, coheplas=5.0e6, strike=270.0, dip=90.0, slipRateThres=0.001,
                xmin=-15e3, xmax=15e3, ymin=-10e3, ymax=10e3, zmin=-15e3, zmax=0.0,
                nuni_y_minus=5, nuni_y_plus=5, enlarging_ratio=1.0, dx=200.0, dy=200.0, dz=200.0,
                fxmin=-12e3, fxmax=12e3, fymin=0.0, fymax=0.0, fzmin=-12e3, fzmax=0.0)


def _stations(rng, p, n_on=20, n_off=20):
    dx = p["dx"]
    nx = int(round((p["fxmax"] - p["fxmin"]) / dx))
    nz = int(round((p["fzmax"] - p["fzmin"]) / p["dz"]))
    on = set()
    while len(on) < min(n_on, (nx + 1) * (nz + 1)):
        on.add((int(rng.integers(0, nx + 1)), int(rng.integers(0, nz + 1))))
    st_on = np.array([[(p["fxmin"] + i * dx) / 1e3, (p["fzmin"] + k * p["dz"]) / 1e3]
                      for i, k in sorted(on)])
    # surface stations on grid nodes strictly inside the physical box, off the fault plane; the
    # grid lines are aligned with the fault edge (x) and the fault plane (y = 0)
    ilo = int(math.ceil((p["xmin"] - p["fxmin"]) / dx)) + 1
    ihi = int(math.floor((p["xmax"] - p["fxmin"]) / dx)) - 1
    jlo = int(math.ceil(p["ymin"] / p["dy"])) + 1
    jhi = int(math.floor(p["ymax"] / p["dy"])) - 1
    off = set()
    while len(off) < n_off:
        i, j = int(rng.integers(ilo, ihi + 1)), int(rng.integers(jlo, jhi + 1))
        if j != 0:
            off.add((i, j))
    st_off = np.array([[(p["fxmin"] + i * dx) / 1e3, j * p["dy"] / 1e3, 0.0] for i, j in sorted(off)])
    return st_on, st_off


def _fault_grid(p):
    nfx = int(round((p["fxmax"] - p["fxmin"]) / p["dx"])) + 1
    nfz = int(round((p["fzmax"] - p["fzmin"]) / p["dz"])) + 1
    fx = np.linspace(p["fxmin"], p["fxmax"], nfx)
    fz = np.linspace(p["fzmin"], p["fzmax"], nfz)
    return fx, fz


def config_c0(path, scale=1.0, nsteps=1000, **switches):
    """C0 slip-weakening half-space; `switches` are extra bGPU.txt switches (e.g. C_Q=1 for the
    coarse-grained Q model)."""
    p = _base_params()
    dx = 200.0 * scale
    p.update(dx=dx, dy=dx, dz=dx, dt=0.008 * scale, friclaw=1, tpv=0, C_nuclea=0)
    p["term"] = nsteps * p["dt"]
    rng = np.random.default_rng(SEED0 + 0)
    fx, fz = _fault_grid(p)
    ofv = np.zeros((24, len(fz), len(fx)))
    F = _NC_INDEX
    for ix, x in enumerate(fx):
        for iz, z in enumerate(fz):
            edge = abs(abs(x) - p["fxmax"]) < 0.01 or abs(z - p["fzmin"]) < 0.01
            ofv[F[1], iz, ix] = 1000.0 if edge else 0.70
            ofv[F[2], iz, ix] = 0.50
            ofv[F[3], iz, ix] = 0.30
            ofv[F[7], iz, ix] = -100.0e6
            patch = abs(x) <= 1.5e3 + 1e-6 and abs(z + 7.5e3) <= 1.5e3 + 1e-6
            ofv[F[8], iz, ix] = 72.0e6 if patch else 60.0e6
    st_on, st_off = _stations(rng, p)
    write_case_dir(path, p, [[6000.0, 3464.0, 2670.0]], st_on, st_off, ofv,
                   gpu_switches=dict({"nPML": 6, "C_hg": 1, "kapa_hg": 0.1}, **switches))
    return path


def aging_state(a, b, L, V0, f0, tau_over_sigma, V):
    """State theta for which the regularised aging-law friction equals tau/|sigma| at slip rate V
    (mu = a asinh(V/(2 V0) exp((f0 + b ln(V0 theta / L)) / a)), solved for theta)."""
    psi = a * (math.log(2.0 * V0 / V) + _log_sinh(tau_over_sigma / a))
    return L / V0 * math.exp((psi - f0) / b)


def _log_sinh(x):
    return x + math.log1p(-math.exp(-2 * x)) - math.log(2.0) if x > 20 else math.log(math.sinh(x))


def config_c1(path, scale=1.0, nsteps=4000, npml=None):
    p = _base_params()
    dx = 100.0 * scale
    p.update(dx=dx, dy=dx, dz=dx, dt=0.004 * scale, friclaw=3, tpv=104, C_nuclea=1,
             xsource=0.0, ysource=0.0, zsource=-7.5e3, nucR=3.0e3, nucdtau0=25.0e6, nucT=1.0)
    p["term"] = nsteps * p["dt"]
    npml = npml if npml is not None else max(2, int(round(4000.0 / dx)))
    rng = np.random.default_rng(SEED0 + 1)
    fx, fz = _fault_grid(p)
    ofv = np.zeros((24, len(fz), len(fx)))
    F = _NC_INDEX
    a0, da, b, L, V0, f0, Vini, sigma, tau = 0.008, 0.008, 0.012, 0.02, 1e-6, 0.6, 1e-12, -100e6, 60e6
    for ix, x in enumerate(fx):
        for iz, z in enumerate(fz):
            core = _smooth_box(x, 9.0e3, 3.0e3) * _smooth_box(-z - 6.0e3, 3.0e3, 3.0e3)
            a = a0 + da * (1.0 - core)
            ofv[F[9], iz, ix] = a
            ofv[F[10], iz, ix] = b
            ofv[F[11], iz, ix] = L
            ofv[F[12], iz, ix] = V0
            ofv[F[13], iz, ix] = f0
            ofv[F[46], iz, ix] = Vini
            ofv[F[7], iz, ix] = sigma
            ofv[F[8], iz, ix] = tau
            ofv[F[20], iz, ix] = aging_state(a, b, L, V0, f0, tau / abs(sigma), Vini)
            ofv[F[1], iz, ix], ofv[F[2], iz, ix], ofv[F[3], iz, ix] = 0.7, 0.5, 0.3
    st_on, st_off = _stations(rng, p)
    R = {6: 0.01, 10: 0.001, 20: 0.0001}.get(npml, 1e-5 if npml > 20 else 0.001)
    write_case_dir(path, p, [[6000.0, 3464.0, 2670.0]], st_on, st_off, ofv,
                   gpu_switches={"nPML": npml, "R": R, "C_hg": 1})
    return path


def c2_layers(dz):
    """1-D layered medium of C2, one row per cell of thickness dz down to 8 km (as the reference's
    drv.a6 compset builds its profile): Vs from 1500 m/s at the surface to 3500 m/s at 8 km
    (linear in depth at the cell centre), Vp = 1.73 Vs, Gardner density rho = 1741 Vp^0.25
    (kg/m^3, Vp in km/s); rows [depth of the layer bottom, Vp, Vs, rho], the last extended to
    1000 km."""
    rows = []
    i = 0
    while True:
        zc = (i + 0.5) * dz
        vs = 1500.0 + 2000.0 * min(zc / 8.0e3, 1.0)
        vp = 1.73 * vs
        rho = 1741.0 * (vp / 1000.0) ** 0.25
        rows.append([zc + 0.5 * dz, vp, vs, rho])
        i += 1
        if zc > 8.0e3:
            break
    rows[-1][0] = 1.0e6
    return np.array(rows)


def config_c2(path, scale=1.0, nsteps=6000, q=2, plastic=True):
    """C2: the C0 box at dx = 50 m (600 x 400 x 300 = 72 M elements + 6-layer PML) in the layered
    medium of c2_layers; Q with 8 coarse-grained mechanisms, Qs = 50 Vs (km/s), Qp = 2 Qs
    (C_Q = 2, an extension: the reference's Q is Qs = 10 / 50 by depth and stops with plasticity);
    Drucker-Prager plasticity (cohesion 1 MPa, bulk friction 0.75, tv = 2 dz / 3464 = 0.029 s at
    50 m, gravity and the reference's regional stress: principal stress at 45 degrees to the fault,
    deviatoric / vertical 0.33, hydrostatic pore pressure with overpressure 0.66); slip weakening
    (mu_s 0.70, mu_d 0.50, Dc 0.3 m, sigma_n = -100 MPa) with tau0 = 60 MPa (1 + 0.1 f), f a seeded
    von Karman field (correlation length 2 km, Hurst 0.8), and a 3 x 3 km patch at 72 MPa around
    (0, -7.5 km).  q = 1 selects the reference's Q (then plastic must be False), q = 0 no Q."""
    if q == 1 and plastic:
        raise ValueError("the reference's Q (C_Q = 1) does not run with plasticity")
    p = _base_params()
    dx = 50.0 * scale
    layers = c2_layers(dx)
    p.update(dx=dx, dy=dx, dz=dx, dt=0.002 * scale, friclaw=1, tpv=0, C_nuclea=0,
             C_elastic=0 if plastic else 1, nmat=len(layers), n2mat=4, roumax=float(layers[-1, 3]),
             rhow=1000.0, gamar=0.66, bulk=0.75, coheplas=1.0e6, vmaxPML=float(layers[-1, 1]))
    p["term"] = nsteps * p["dt"]
    rng = np.random.default_rng(SEED0 + 2)
    fx, fz = _fault_grid(p)
    field = von_karman_field(rng, len(fz), len(fx), dx, 2.0e3, 0.8)
    ofv = np.zeros((24, len(fz), len(fx)))
    F = _NC_INDEX
    for ix, x in enumerate(fx):
        for iz, z in enumerate(fz):
            edge = abs(abs(x) - p["fxmax"]) < 0.01 or abs(z - p["fzmin"]) < 0.01
            ofv[F[1], iz, ix] = 1000.0 if edge else 0.70
            ofv[F[2], iz, ix] = 0.50
            ofv[F[3], iz, ix] = 0.30
            ofv[F[7], iz, ix] = -100.0e6
            patch = abs(x) <= 1.5e3 + 1e-6 and abs(z + 7.5e3) <= 1.5e3 + 1e-6
            ofv[F[8], iz, ix] = 72.0e6 if patch else 60.0e6 * (1.0 + 0.1 * field[iz, ix])
    st_on, st_off = _stations(rng, p)
    write_case_dir(path, p, layers, st_on, st_off, ofv,
                   gpu_switches={"nPML": 6, "C_hg": 1, "kapa_hg": 0.1, "C_Q": int(q)})
    return path


def config_c3(path, scale=1.0, nsteps=5000, L=0.2, patch_ratio=0.75, patch_radius=2.0e3):
    """30-degree dipping reverse fault reaching the free surface (down-dip width 20 km, 40 km along
    strike), as the reference builds dipping faults (case_input/test.tpv36): cells of dx along
    strike, dx cos(dip) and dx sin(dip) across it, hexahedra along the fault degenerated into wedge
    pairs (C_degen = dip), dt = 0.5 dz / vp (scripts/defaultParameters.py mod4dip).  Slip law with
    strong rate weakening (TPV104 form: a = 0.01 rising by 0.01 and Vw from 0.1 by 0.9 outside a
    smooth core, b 0.014, V0 1e-6, f0 0.6, fw 0.2; L 0.2 m, half TPV104's, because with 0.4 m the
    2 km patch stays below the nucleation size and creeps for tens of seconds), initial slip rate
    1e-12 m/s and the state at steady state for the background stress; sigma_n = 16.2 MPa/km x depth
    capped at 120 MPa (floored at 1 MPa at the surface); dip shear 0.55 sigma_n moving the hanging
    wall (y+) up, 0.75 sigma_n in a 2 km circle at 10 km down dip.  The initial creep rate points
    along the initial shear (bGPU.txt vini_along_shear): the reference always starts it along
    strike, which leaves a dip-loaded rate-and-state fault out of equilibrium at the first step."""
    dip = 30.0
    sd, cd = math.sin(math.radians(dip)), math.cos(math.radians(dip))
    width, length = 20.0e3, 40.0e3
    p = _base_params()
    dx = 100.0 * scale
    dy, dz = dx * cd, dx * sd
    p.update(dx=dx, dy=dy, dz=dz, dt=0.5 * dz / 6000.0, friclaw=4, tpv=0, C_nuclea=0, dip=dip, C_degen=dip,
             insertFaultType=0,
             xmin=-length / 2 - 3.0e3, xmax=length / 2 + 3.0e3, ymin=-4.0e3, ymax=width * cd + 4.0e3,
             zmin=-width * sd - 4.0e3, zmax=0.0,
             fxmin=-length / 2, fxmax=length / 2, fymin=0.0, fymax=width * cd, fzmin=-width * sd, fzmax=0.0,
             nuni_y_minus=5, nuni_y_plus=int(round(width / dx)) + 5, enlarging_ratio=1.025,
             xsource=0.0, ysource=10.0e3 * cd, zsource=-10.0e3 * sd)
    p["term"] = nsteps * p["dt"]
    rng = np.random.default_rng(SEED0 + 3)
    nfx = int(round((p["fxmax"] - p["fxmin"]) / dx)) + 1
    nfz = int(round((p["fzmax"] - p["fzmin"]) / dz)) + 1
    fx = np.linspace(p["fxmin"], p["fxmax"], nfx)
    fz = np.linspace(p["fzmin"], p["fzmax"], nfz)
    ofv = np.zeros((24, nfz, nfx))
    F = _NC_INDEX
    a0, da, b, V0, f0, fw, vw0, dvw, Vini = 0.01, 0.01, 0.014, 1e-6, 0.6, 0.2, 0.1, 0.9, 1e-12
    for ix, x in enumerate(fx):
        for iz, z in enumerate(fz):
            downdip = abs(z) / sd
            core = _smooth_box(x, length / 2 - 3.0e3, 3.0e3) * _smooth_box(downdip - width / 2, width / 2 - 3.0e3, 3.0e3)
            a = a0 + da * (1.0 - core)
            sigma = max(min(16.2e6 * abs(z) / 1e3, 120.0e6), 1.0e6)
            ratio = patch_ratio if math.hypot(x, downdip - 10.0e3) <= patch_radius else 0.55
            tau = ratio * sigma
            ofv[F[9], iz, ix] = a
            ofv[F[10], iz, ix] = b
            ofv[F[11], iz, ix] = L
            ofv[F[12], iz, ix] = V0
            ofv[F[13], iz, ix] = f0
            ofv[F[14], iz, ix] = fw
            ofv[F[15], iz, ix] = vw0 + dvw * (1.0 - core)
            ofv[F[46], iz, ix] = Vini
            ofv[F[7], iz, ix] = -sigma
            ofv[F[8], iz, ix] = 0.0
            ofv[F[49], iz, ix] = tau
            # background steady state (0.55), so the overstressed patch accelerates and nucleates
            ofv[F[20], iz, ix] = a * math.log(2.0 * V0 / Vini * math.sinh(0.55 / a))
            ofv[F[1], iz, ix], ofv[F[2], iz, ix], ofv[F[3], iz, ix] = 0.7, 0.5, 0.3
    st_on = np.array([[0.0, 0.0], [0.0, -2.5], [0.0, -5.0], [10.0, -5.0], [-10.0, -2.5]])
    st_off = np.array([[0.0, -2.0, 0.0], [0.0, 2.0, 0.0], [10.0, 8.0, 0.0], [0.0, 16.0, 0.0]])
    write_case_dir(path, p, [[6000.0, 3464.0, 2670.0]], st_on, st_off, ofv,
                   gpu_switches={"nPML": 6, "C_hg": 1, "kapa_hg": 0.1, "vini_along_shear": 1})
    return path


def von_karman_field(rng, nz, nx, h, corr, hurst):
    """Zero-mean, unit-variance 2-D random field with the von Karman spectrum
    P(k) ~ (1 + (k a)^2)^-(H + 1) (correlation length a, Hurst exponent H) on an nz x nx grid of
    spacing h: seeded white noise filtered in the Fourier domain (periodic)."""
    noise = rng.standard_normal((nz, nx))
    kz = 2.0 * np.pi * np.fft.fftfreq(nz, d=h)
    kx = 2.0 * np.pi * np.fft.fftfreq(nx, d=h)
    k2 = kz[:, None] ** 2 + kx[None, :] ** 2
    amp = (1.0 + k2 * corr * corr) ** (-(hurst + 1.0) / 2.0)
    f = np.real(np.fft.ifft2(np.fft.fft2(noise) * amp))
    f -= f.mean()
    sd = f.std()
    return f / sd if sd > 0 else f


C4_DX = (200.0, 250.0, 300.0, 400.0)


def config_c4(path, member, nsteps=1500):
    """Member `member` (0..63) of the C4 ensemble: the C0 box and slip-weakening fault at a seeded
    dx from {200, 250, 300, 400} m (dt = 0.008 s * dx / 200 m), initial shear stress
    60 MPa * (1 + s f) with f a seeded von Karman field (correlation length 1-4 km, Hurst 0.8,
    s = 5-15 %), and a 3 x 3 km nucleation patch at 72 MPa around a seeded hypocentre."""
    rng = np.random.default_rng(SEED0 + 4 + 1000 * member)
    dx = float(C4_DX[int(rng.integers(0, len(C4_DX)))])
    p = _base_params()
    p.update(dx=dx, dy=dx, dz=dx, dt=0.008 * dx / 200.0, friclaw=1, tpv=0, C_nuclea=0)
    p["term"] = nsteps * p["dt"]
    corr = float(rng.uniform(1.0e3, 4.0e3))
    sd = float(rng.uniform(0.05, 0.15))
    hx = float(rng.uniform(-8.0e3, 8.0e3))
    hz = float(rng.uniform(-10.0e3, -3.0e3))
    fx, fz = _fault_grid(p)
    field = von_karman_field(rng, len(fz), len(fx), dx, corr, 0.8)
    ofv = np.zeros((24, len(fz), len(fx)))
    F = _NC_INDEX
    for ix, x in enumerate(fx):
        for iz, z in enumerate(fz):
            edge = abs(abs(x) - p["fxmax"]) < 0.01 or abs(z - p["fzmin"]) < 0.01
            ofv[F[1], iz, ix] = 1000.0 if edge else 0.70
            ofv[F[2], iz, ix] = 0.50
            ofv[F[3], iz, ix] = 0.30
            ofv[F[7], iz, ix] = -100.0e6
            patch = abs(x - hx) <= 1.5e3 + 1e-6 and abs(z - hz) <= 1.5e3 + 1e-6
            ofv[F[8], iz, ix] = 72.0e6 if patch else 60.0e6 * (1.0 + sd * field[iz, ix])
    st_on, st_off = _stations(rng, p, n_on=4, n_off=4)
    write_case_dir(path, p, [[6000.0, 3464.0, 2670.0]], st_on, st_off, ofv,
                   gpu_switches={"nPML": 6, "C_hg": 1, "kapa_hg": 0.1})
    return path


CONFIGS = {"C2": config_c2, "C0": config_c0, "C1": config_c1, "C3": config_c3}

WORKLOADS = {
    "C0": "slip-weakening half-space, dx 200 m, 1,469,664 elements (6-layer PML)",
    "C2": "layered medium (Vs 1.5-3.5 km/s), Q = 50 Vs with 8 mechanisms, Drucker-Prager plasticity, "
          "von Karman initial shear stress, slip weakening, dx 50 m",
    "C3": "30-degree dipping reverse fault to the surface, wedge elements along the fault, slip law, "
          "dx 100 m along strike and dip, learned Newton guess",
    "C4": "ensemble of 64 slip-weakening scenarios, dx from {200, 250, 300, 400} m, von Karman initial "
          "shear stress, seeded hypocentres, one launch per kernel per step",
    "C1": "rate-and-state aging law, dx 100 m, 20,216,000 elements (40-layer PML), learned Newton guess",
}
