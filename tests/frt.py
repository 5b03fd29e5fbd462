"""Helpers shared by the tests: the 22-column frt table (src/library_output.f90:160-205) and
matching of computed fault nodes to golden rows by coordinates."""
import numpy as np
from scipy.spatial import cKDTree

FRT_COLUMNS = ["x", "y", "z", "trup", "slip_s", "slip_d", "slip_n", "rate_s", "rate_d",
               "peak_rate", "final_rate", "tnrm", "tstk", "tdip", "vxm", "vym", "vzm", "vxs",
               "vys", "vzs", "state", "state_normal"]
FRIC_OF_COLUMN = [71, 72, 73, 74, 75, 76, 47, 78, 79, 80, 31, 32, 33, 34, 35, 36, 20, 23]


def frt_table(case):
    """The rows output_frt writes, one per fault pair, from a Case's arrays."""
    fr = case.fric()
    cols = [case.arrays["fnft"][: case.npair]] + [fr[:, k - 1] for k in FRIC_OF_COLUMN]
    return np.column_stack([case.fault_coords()] + cols)


def golden_frt(npz):
    d = np.load(npz)
    return np.vstack([d[k] for k in sorted(d.files) if k.startswith("frt_rank")])


def match_rows(ours, gold):
    """Golden row for each of our rows (nearest (x, z), duplicates from the shared MPI plane
    collapse onto the same coordinates)."""
    dist, idx = cKDTree(gold[:, [0, 2]]).query(ours[:, [0, 2]])
    return gold[idx], dist


def print_rounded(a):
    """Round to the 7 significant digits of the E18.7 format the reference prints."""
    a = np.asarray(a, dtype=np.float64)
    out = np.zeros_like(a)
    nz = a != 0
    e = np.floor(np.log10(np.abs(a[nz]))) + 1
    out[nz] = np.round(a[nz] / 10.0 ** e, 7) * 10.0 ** e
    return out
