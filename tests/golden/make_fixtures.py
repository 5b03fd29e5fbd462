#!/usr/bin/env python3
"""Generate the golden case fixtures under tests/golden/ from the EQdyna reference tree.

This script is the only place that reads the reference tree.  For every case that ships a
golden output in ``test.reference.results/`` it

1. imports the case's own ``case_input/<case>/user_defined_params.py`` (which itself imports the
   reference's ``scripts/defaultParameters.py`` and ``scripts/lib.py``) and records every value
   that ``scripts/case.setup:10-76`` writes into the b-files (bGlobal, bModelGeometry,
   bFaultGeometry, bMaterial, bStations);
2. records the 24 on-fault fields that ``scripts/case.setup:78-185`` writes to
   ``on_fault_vars_input.nc`` (netCDF cannot be written here; the arrays are stored directly, in
   the (dip, strike) order of the netCDF variables);
3. for ``insertFaultType > 0`` runs the reference's own ``scripts/generateFaultInterface``
   (matplotlib replaced by a do-nothing stub, since only its numeric part matters) and reads the
   ``bFault_Rough_Geometry.txt`` it writes back with the same text->double parsing the Fortran
   reader does (``src/readInputFiles.f90:268-312``);
4. parses the golden ``frt.txt<rank>`` files (22 columns, ``src/library_output.f90:160-205``)
   and the one golden on-fault station time series.

Usage:  python tests/golden/make_fixtures.py [--ref /root/reference]
"""
import argparse
import importlib
import json
import os
import sys
import tempfile
import types
import unittest.mock

import numpy as np

CASES = ["test.tpv8", "test.tpv10", "test.tpv104", "test.tpv1053d", "test.drv.a6",
         "test.meng2023a", "test.meng2023cb"]

# netCDF variable order of scripts/case.setup:86-121 mapped to the index of par.on_fault_vars
# that feeds it (scripts/case.setup:153-185).  The Fortran reader (src/netcdf_io.f90:40-63)
# reads the variables in exactly this order.
NC_FIELDS = [("sw_fs", 1), ("sw_fd", 2), ("sw_D0", 3), ("rsf_a", 9), ("rsf_b", 10),
             ("rsf_Dc", 11), ("rsf_v0", 12), ("rsf_r0", 13), ("rsf_fw", 14), ("rsf_vw", 15),
             ("tp_a_hy", 16), ("tp_a_th", 17), ("tp_rouc", 18), ("tp_lambda", 19),
             ("tp_h", 40), ("tp_Tini", 41), ("tp_pini", 42), ("init_slip_rate", 46),
             ("init_strike_shear", 8), ("init_normal_stress", 7), ("init_state", 20),
             ("tw_t0", 5), ("cohesion", 4), ("init_dip_shear", 49)]


def _load_par(ref, case):
    case_dir = os.path.join(ref, "case_input", case)
    scripts = os.path.join(ref, "scripts")
    for name in ("user_defined_params", "defaultParameters", "lib"):
        sys.modules.pop(name, None)
    old_path = list(sys.path)
    sys.path[:0] = [case_dir, scripts]
    try:
        with unittest.mock.patch("builtins.print"):
            mod = importlib.import_module("user_defined_params")
    finally:
        sys.path[:] = old_path
    return mod.par, case_dir, scripts


def _rough_geometry(par, case_dir, scripts):
    """Run the reference generateFaultInterface numeric path; return the parsed text file."""
    fake_plt = unittest.mock.MagicMock()
    fake_mpl = types.ModuleType("matplotlib")
    fake_mpl.pyplot = fake_plt
    saved = {k: sys.modules.get(k) for k in ("matplotlib", "matplotlib.pyplot")}
    sys.modules["matplotlib"] = fake_mpl
    sys.modules["matplotlib.pyplot"] = fake_plt
    src = open(os.path.join(scripts, "generateFaultInterface")).read()
    cwd = os.getcwd()
    with tempfile.TemporaryDirectory() as tmp:
        os.chdir(tmp)
        try:
            sys.modules["user_defined_params"].par = par
            glb = {"__name__": "gfi"}
            with unittest.mock.patch("builtins.print"):
                exec(compile(src, "generateFaultInterface", "exec"), glb)
                glb["_main_func"](None)
            rough = np.loadtxt("bFault_Rough_Geometry.txt", dtype=np.float64)
        finally:
            os.chdir(cwd)
            for k, v in saved.items():
                if v is None:
                    sys.modules.pop(k, None)
                else:
                    sys.modules[k] = v
    return rough


def _params(par):
    g = {}
    for key in ("mode", "C_elastic", "C_nuclea", "C_degen", "insertFaultType", "friclaw",
                "ntotft", "nucfault", "tpv", "output_plastic", "outputGroundMotion",
                "outputFinalSurfDisp", "nx", "ny", "nz", "term", "dt", "nmat", "n2mat",
                "roumax", "rhow", "gamar", "rdampk", "vmaxPML", "xsource", "ysource", "zsource",
                "nucR", "nucRuptVel", "nucdtau0", "nucT", "str1ToFaultAngle",
                "devStrToStrVertRatio", "bulk", "coheplas", "strike", "dip", "slipRateThres",
                "xmin", "xmax", "ymin", "ymax", "zmin", "zmax", "nuni_y_minus", "nuni_y_plus",
                "enlarging_ratio", "dx", "dy", "dz", "fxmin", "fxmax", "fymin", "fymax",
                "fzmin", "fzmax"):
        v = getattr(par, key)
        g[key] = v.item() if isinstance(v, np.generic) else v
    return g


def _material(par):
    if par.nmat == 1:
        return np.array([[par.vp, par.vs, par.rou]], dtype=np.float64)
    return np.asarray(par.mat, dtype=np.float64)[:par.nmat, :par.n2mat].copy()


def _parse_table(path, skip_comments=True):
    rows = []
    with open(path) as f:
        for line in f:
            s = line.strip()
            if not s or (skip_comments and (s.startswith("#") or s[0].isalpha())):
                continue
            rows.append([float(t) for t in s.split()])
    return np.array(rows, dtype=np.float64)


def make_case(ref, case, outdir):
    par, case_dir, scripts = _load_par(ref, case)
    params = _params(par)
    out = {"params_json": np.array(json.dumps(params))}
    out["material"] = _material(par)
    out["st_on_fault"] = np.asarray(par.st_coor_on_fault, dtype=np.float64).reshape(-1, 2)
    out["st_off_fault"] = np.asarray(par.st_coor_off_fault, dtype=np.float64).reshape(-1, 3)
    ofv = np.asarray(par.on_fault_vars, dtype=np.float64)
    out["on_fault_vars"] = np.stack([ofv[:, :, k] for _, k in NC_FIELDS])  # (24, nfz, nfx)
    if par.insertFaultType > 0:
        out["rough_geometry"] = _rough_geometry(par, case_dir, scripts)
    golden_dir = os.path.join(ref, "test.reference.results", case)
    frt = []
    for name in sorted(os.listdir(golden_dir)):
        if name.startswith("frt.txt"):
            tab = _parse_table(os.path.join(golden_dir, name))
            out["frt_rank" + name[len("frt.txt"):]] = tab
            frt.append(tab)
        elif name.startswith("faultst") and name.endswith(".txt"):
            out["faultst_" + name[len("faultst"):-len(".txt")]] = _parse_table(
                os.path.join(golden_dir, name))
    path = os.path.join(outdir, case.replace("test.", "") + ".npz")
    np.savez_compressed(path, **out)
    return path


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default="/root/reference")
    ap.add_argument("--out", default=os.path.dirname(os.path.abspath(__file__)))
    args = ap.parse_args()
    for case in CASES:
        p = make_case(args.ref, case, args.out)
        print(case, "->", p, os.path.getsize(p), "bytes")


if __name__ == "__main__":
    main()
