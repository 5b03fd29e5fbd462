"""Output streams of the time loop, fed by the device-side capture of GpuSolver.output_setup.

The reference writes, when mod(nt, 10) == 1 (src/driver.f90:30-33), the velocity of every surface
node as a binary stream (output_gm, src/library_output.f90:267-279, file ``gm<rank>``) and fric(47)
of every fault pair (output_src_evol, :297-312, file ``src_evol<rank>``); the surface nodes and their
coordinates come from find_surfaceNodeIdArr (:246-262, ``surface_coor.txt<rank>``).  Here the
frames are written on the device inside each step and drained in batches; these helpers pick the
same surface nodes and append the same bytes.
"""
import os

import numpy as np


def surface_nodes(case):
    """Fortran (1-based) numbers of the nodes find_surfaceNodeIdArr selects: within 20 km of the
    fault's bounding box in x and y, and |z| < dx / 1000 (the free surface)."""
    xyz = case.arrays["meshCoor"].reshape(-1, 3)
    f = case.fault_coords()
    lo, hi = f.min(axis=0), f.max(axis=0)
    dx = case.scalars.dx
    sel = ((xyz[:, 0] < hi[0] + 20.0e3) & (xyz[:, 0] > lo[0] - 20.0e3) &
           (xyz[:, 1] < hi[1] + 20.0e3) & (xyz[:, 1] > lo[1] - 20.0e3) & (np.abs(xyz[:, 2]) < dx / 1000.0))
    return np.flatnonzero(sel).astype(np.int32) + 1


def write_surface_coor(directory, case, nodes, suffix=""):
    """surface_coor.txt: one line of x y z per surface node (format 1x,3e18.7e4)."""
    xyz = case.arrays["meshCoor"].reshape(-1, 3)[np.asarray(nodes) - 1]
    with open(os.path.join(directory, "surface_coor.txt" + suffix), "a") as fh:
        for x, y, z in xyz:
            fh.write(" %s%s%s\n" % (_e18(x), _e18(y), _e18(z)))


def append_frames(directory, gm, src_evol, suffix=""):
    """Append drained frames to ``gm`` (3 doubles per surface node per frame) and ``src_evol``
    (fric(47) per pair per frame), native byte order, as the reference's stream writes do."""
    if gm is not None and gm.size:
        with open(os.path.join(directory, "gm" + suffix), "ab") as fh:
            np.ascontiguousarray(gm, dtype=np.float64).tofile(fh)
    if src_evol is not None and src_evol.size:
        with open(os.path.join(directory, "src_evol" + suffix), "ab") as fh:
            np.ascontiguousarray(src_evol, dtype=np.float64).tofile(fh)


def _e18(v):
    """Fortran e18.7e4: width 18, 7 digits after the point, 4-digit exponent (0.1234567E+0003)."""
    if v == 0.0:
        mant, exp = 0.0, 0
    else:
        exp = int(np.floor(np.log10(abs(v)))) + 1
        mant = v / 10.0 ** exp
        if abs(round(mant, 7)) >= 1.0:
            mant /= 10.0
            exp += 1
    return ("%.7fE%s%04d" % (mant, "+" if exp >= 0 else "-", abs(exp))).rjust(18)
