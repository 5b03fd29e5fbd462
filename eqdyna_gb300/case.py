"""Case directories and the Fortran-layout state built from them.

A case directory holds the reference's input files, written in the exact format of
``scripts/case.setup:10-76`` (bGlobal.txt, bModelGeometry.txt, bFaultGeometry.txt, bMaterial.txt,
bStations.txt), the optional bFault_Rough_Geometry.txt of ``scripts/generateFaultInterface``, and
``on_fault_vars_input.bin`` — the 24 netCDF fields of ``on_fault_vars_input.nc``
(``scripts/case.setup:78-185``) as raw binary64, since netCDF is not part of this stack.
``bGPU.txt`` optionally sets switches that are compile-time constants in the reference.

``Case.from_dir`` runs the native case builder (the reference's setup restated in C++) and keeps
the resulting globalvar arrays as numpy arrays in Fortran order.
"""
import ctypes as C
import json
import os
import tempfile
import time

import numpy as np

from . import _native as N

# netCDF variable order of on_fault_vars_input.nc (src/netcdf_io.f90:40-63) -> on_fault_vars index
NC_FIELDS = [("sw_fs", 1), ("sw_fd", 2), ("sw_D0", 3), ("rsf_a", 9), ("rsf_b", 10),
             ("rsf_Dc", 11), ("rsf_v0", 12), ("rsf_r0", 13), ("rsf_fw", 14), ("rsf_vw", 15),
             ("tp_a_hy", 16), ("tp_a_th", 17), ("tp_rouc", 18), ("tp_lambda", 19),
             ("tp_h", 40), ("tp_Tini", 41), ("tp_pini", 42), ("init_slip_rate", 46),
             ("init_strike_shear", 8), ("init_normal_stress", 7), ("init_state", 20),
             ("tw_t0", 5), ("cohesion", 4), ("init_dip_shear", 49)]

MUTABLE = ("stressArr", "pstrain", "v1", "velArr", "dispArr", "nodalForceArr", "fric", "fnft",
           "onFaultQuantHistSCECForm", "OffFaultStGramSCEC", "onFaultTPHist")


def _s(v):
    """str() exactly as case.setup writes a Python value."""
    return str(v)


def write_case_dir(path, params, material, st_on_fault, st_off_fault, on_fault_vars,
                   rough_geometry=None, gpu_switches=None):
    """Write a case directory.

    params        dict with the attribute names of the reference ``parameters`` class
                  (scripts/defaultParameters.py)
    material      (nmat, n2mat) array
    st_on_fault   (n, 2) km;  st_off_fault (m, 3) km
    on_fault_vars (24, nfz, nfx) in NC_FIELDS order
    """
    p = params
    os.makedirs(path, exist_ok=True)
    with open(os.path.join(path, "bGlobal.txt"), "w") as f:
        for k in ("mode", "C_elastic", "C_nuclea", "C_degen", "insertFaultType", "friclaw",
                  "ntotft", "nucfault", "tpv", "output_plastic", "outputGroundMotion",
                  "outputFinalSurfDisp"):
            f.write(_s(p[k]) + "\n")
        f.write(" \n")
        f.write(f"{_s(p['nx'])} {_s(p['ny'])} {_s(p['nz'])}\n")
        f.write(" \n")
        f.write(_s(p["term"]) + "\n")
        f.write(_s(p["dt"]) + "\n")
        f.write(" \n")
        f.write(f"{_s(p['nmat'])} {_s(p['n2mat'])}\n")
        f.write(f"{_s(p['roumax'])} {_s(p['rhow'])} {_s(p['gamar'])}\n")
        f.write(f"{_s(p['rdampk'])} {_s(p['vmaxPML'])}\n")
        f.write(" \n")
        f.write(f"{_s(p['xsource'])} {_s(p['ysource'])} {_s(p['zsource'])}\n")
        f.write(f"{_s(p['nucR'])} {_s(p['nucRuptVel'])} {_s(p['nucdtau0'])} {_s(p['nucT'])}\n")
        f.write(f"{_s(p['str1ToFaultAngle'])} {_s(p['devStrToStrVertRatio'])}\n")
        f.write(f"{_s(p['bulk'])} {_s(p['coheplas'])}\n")
        f.write(f"{_s(p['strike'])} {_s(p['dip'])}\n")
        f.write(_s(p["slipRateThres"]) + "\n")
    with open(os.path.join(path, "bModelGeometry.txt"), "w") as f:
        f.write(f"{_s(p['xmin'])}  {_s(p['xmax'])}\n")
        f.write(f"{_s(p['ymin'])}  {_s(p['ymax'])}\n")
        f.write(f"{_s(p['zmin'])}  {_s(p['zmax'])}\n")
        f.write(" \n")
        f.write(f"{_s(p['nuni_y_minus'])} {_s(p['nuni_y_plus'])}\n")
        f.write(_s(p["enlarging_ratio"]) + "\n")
        f.write(f"{_s(p['dx'])} {_s(p['dy'])} {_s(p['dz'])}\n")
    with open(os.path.join(path, "bFaultGeometry.txt"), "w") as f:
        f.write("For fault No. 1\n")
        f.write(f"{_s(p['fxmin'])}  {_s(p['fxmax'])}\n")
        f.write(f"{_s(p['fymin'])}  {_s(p['fymax'])}\n")
        f.write(f"{_s(p['fzmin'])}  {_s(p['fzmax'])}\n")
    material = np.atleast_2d(np.asarray(material, dtype=np.float64))
    with open(os.path.join(path, "bMaterial.txt"), "w") as f:
        for row in material:
            f.write(" ".join(_s(float(v)) for v in row) + "\n")
    st_on = np.asarray(st_on_fault, dtype=np.float64).reshape(-1, 2)
    st_off = np.asarray(st_off_fault, dtype=np.float64).reshape(-1, 3)
    with open(os.path.join(path, "bStations.txt"), "w") as f:
        f.write(f"{len(st_off)}\n{len(st_on)}\n \n")
        for r in st_on:
            f.write(f"{_s(float(r[0]))} {_s(float(r[1]))}\n")
        f.write(" \n")
        for r in st_off:
            f.write(f"{_s(float(r[0]))} {_s(float(r[1]))} {_s(float(r[2]))}\n")
    ofv = np.ascontiguousarray(on_fault_vars, dtype=np.float64)
    assert ofv.ndim == 3 and ofv.shape[0] == 24, ofv.shape
    with open(os.path.join(path, "on_fault_vars_input.bin"), "wb") as f:
        np.array([24, ofv.shape[2], ofv.shape[1]], dtype=np.int32).tofile(f)
        ofv.tofile(f)  # (24, nfz, nfx) C order == Fortran (nfx, nfz, 24)
    if rough_geometry is not None:
        # read back by the builder with the same text->double parse the Fortran reader uses
        rough = np.asarray(rough_geometry, dtype=np.float64)
        np.savetxt(os.path.join(path, "bFault_Rough_Geometry.txt"), rough, fmt="%.17g",
                   delimiter="\t")
    gpu_path = os.path.join(path, "bGPU.txt")
    if gpu_switches:
        with open(gpu_path, "w") as f:
            for k, v in gpu_switches.items():
                f.write(f"{k} {_s(v)}\n")
    elif os.path.exists(gpu_path):
        os.remove(gpu_path)
    return path


class _NativeCase:
    """Owns a built case's native arrays; the case is freed when the last array viewing them is
    gone, so that the arrays are handed out without a copy."""

    def __init__(self, lib, handle):
        self.lib, self.handle = lib, handle

    def view(self, ptr, n, dtype):
        ctype = C.c_int32 if dtype == np.int32 else C.c_double
        buf = (ctype * n).from_address(C.cast(ptr, C.c_void_p).value)
        buf._owner = self
        return np.frombuffer(buf, dtype=dtype)

    def __del__(self):
        if self.handle:
            self.lib.eqd_case_free(self.handle)
            self.handle = None


class Case:
    """Fortran-layout state of one case (the globalvar arrays after setup)."""

    def __init__(self, scalars, arrays, sizes, dims, lines, directory=None):
        self.scalars = scalars
        self.arrays = arrays
        self.sizes = sizes
        self.dims = dims
        self.lines = lines
        self.directory = directory
        self.build_phases_s = None

    @classmethod
    def from_dir(cls, path, tables=True):
        """Build the case in directory `path`.  tables=False builds the mesh only: the per-element
        tables and nodal masses (eleshp, eledet, elemass, ss, phi, nodalMassArr, fnms) are None,
        and eqd_gpu_init builds them on the device."""
        lib = N.case_lib()
        h = C.c_void_p()
        t0 = time.perf_counter()
        rc = lib.eqd_case_build_opt(os.fsencode(path), 0 if tables else 1, C.byref(h))
        if rc != 0:
            raise N.EqdError(rc, "eqd_case_build", lib.eqd_case_last_error().decode())
        owner = _NativeCase(lib, h)
        try:
            sc = N.EqdScalars()
            ha = N.EqdHostArrays()
            lib.eqd_case_view(h, C.byref(sc), C.byref(ha))
            arrays = {}
            for name in N.ARRAY_NAMES:
                eb = C.c_int32()
                n = lib.eqd_case_array_len(h, name.encode(), C.byref(eb))
                ptr = getattr(ha, name)
                if n == 0 or not ptr:
                    arrays[name] = None
                    continue
                arrays[name] = owner.view(ptr, n, np.int32 if name in N.INT_ARRAYS else np.float64)
            sizes = {k: getattr(ha, k) for k in ("nnode", "nelem", "neq", "size_eqidx",
                                                  "size_stress", "ntotft", "nftmx",
                                                  "numOnFaultSt", "numOffFaultSt")}
            nx, ny, nz, nst = C.c_int32(), C.c_int32(), C.c_int32(), C.c_int32()
            nph = C.c_int64()
            lib.eqd_case_dims(h, C.byref(nx), C.byref(ny), C.byref(nz), C.byref(nph), C.byref(nst))
            dims = {"nx": nx.value, "ny": ny.value, "nz": nz.value,
                    "n_phys_elem": nph.value, "nstep": nst.value}
            xs, ys, zs = N.c_double_p(), N.c_double_p(), N.c_double_p()
            lib.eqd_case_lines(h, C.byref(xs), C.byref(ys), C.byref(zs))
            lines = (np.ctypeslib.as_array(xs, shape=(nx.value,)).copy(),
                     np.ctypeslib.as_array(ys, shape=(ny.value,)).copy(),
                     np.ctypeslib.as_array(zs, shape=(nz.value,)).copy())
            ph = (C.c_double * 5)()
            lib.eqd_case_phase_seconds(h, ph)
        finally:
            del owner  # the builder's memory lives on in the arrays viewing it
        case = cls(sc, arrays, sizes, dims, lines, directory=path)
        case.build_phases_s = dict(zip(("inputs", "mesh", "fault", "element_tables", "finish"),
                                       (round(v, 3) for v in ph)))
        case.build_phases_s["views"] = round(time.perf_counter() - t0 - sum(ph), 3)
        return case

    @classmethod
    def from_fixture(cls, npz_path, workdir=None, overrides=None, gpu_switches=None):
        """Build a case from a tests/golden/*.npz fixture (optionally overriding parameters)."""
        d = np.load(npz_path)
        params = json.loads(str(d["params_json"]))
        params.update(overrides or {})
        rough = d["rough_geometry"] if "rough_geometry" in d.files else None
        tmp = workdir or tempfile.mkdtemp(prefix="eqd_case_")
        write_case_dir(tmp, params, d["material"], d["st_on_fault"], d["st_off_fault"],
                       d["on_fault_vars"], rough, gpu_switches)
        return cls.from_dir(tmp)

    # ---- state handling ------------------------------------------------------------------------
    @property
    def nstep(self):
        return self.scalars.nstep

    @property
    def npair(self):
        return int(self.arrays["nftnd"][0])

    def clone(self):
        """Copy with private mutable arrays (read-only tables are shared)."""
        arrays = dict(self.arrays)
        for k in MUTABLE:
            if arrays.get(k) is not None:
                arrays[k] = arrays[k].copy()
        sc = N.EqdScalars()
        C.pointer(sc)[0] = self.scalars
        return Case(sc, arrays, dict(self.sizes), dict(self.dims), self.lines, self.directory)

    def host_arrays(self):
        """eqd_host_arrays pointing into this case's numpy arrays (keep the case alive)."""
        ha = N.EqdHostArrays()
        for k, v in self.sizes.items():
            setattr(ha, k, v)
        for name in N.ARRAY_NAMES:
            a = self.arrays.get(name)
            if a is None:
                continue
            assert a.flags["C_CONTIGUOUS"]
            ptype = N.c_int32_p if name in N.INT_ARRAYS else N.c_double_p
            setattr(ha, name, a.ctypes.data_as(ptype))
        return ha

    # ---- convenience views ---------------------------------------------------------------------
    def fric(self):
        """fric as (npair, 100) (row i = pair i, column k-1 = fric(k))."""
        return self.arrays["fric"].reshape(-1, 100)[: self.npair]

    def fault_coords(self):
        """(npair, 3) coordinates of the slave node of each pair (meshCoor(:, nsmp(1,i)))."""
        nsmp = self.arrays["nsmp"].reshape(-1, 2)[: self.npair]
        xyz = self.arrays["meshCoor"].reshape(-1, 3)
        return xyz[nsmp[:, 0] - 1]

    def n_elements(self):
        return self.sizes["nelem"]
