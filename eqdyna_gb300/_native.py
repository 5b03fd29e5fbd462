"""ctypes view of the C ABI declared in include/eqdyna_gb300.h and include/eqdyna_case.h.

The shared libraries are built in-tree by eqdyna_gb300.build.  Loading never falls back to
anything else: a missing library raises NativeLibraryMissing with the path that was expected.
"""
import ctypes as C
import os

from . import build as _build

c_double_p = C.POINTER(C.c_double)
c_int32_p = C.POINTER(C.c_int32)


class NativeLibraryMissing(RuntimeError):
    pass


class EqdScalars(C.Structure):
    _fields_ = [
        ("dt", C.c_double), ("rdampk", C.c_double), ("rdampm", C.c_double),
        ("grav", C.c_double), ("roumax", C.c_double), ("rhow", C.c_double), ("gamar", C.c_double),
        ("w", C.c_double), ("kapa_hg", C.c_double),
        ("xsource", C.c_double), ("ysource", C.c_double), ("zsource", C.c_double),
        ("nucR", C.c_double), ("nucRuptVel", C.c_double), ("nucdtau0", C.c_double),
        ("nucT", C.c_double),
        ("PMLb", C.c_double * 8), ("vmaxPML", C.c_double), ("R", C.c_double),
        ("ccosphi", C.c_double), ("sinphi", C.c_double), ("tv", C.c_double), ("dx", C.c_double),
        ("slipRateThres", C.c_double), ("fric_tp_h", C.c_double), ("time0", C.c_double),
        ("C_elastic", C.c_int32), ("C_Q", C.c_int32), ("C_hg", C.c_int32),
        ("friclaw", C.c_int32), ("TPV", C.c_int32), ("C_nuclea", C.c_int32),
        ("nucfault", C.c_int32), ("insertFaultType", C.c_int32),
        ("nPML", C.c_int32), ("nstep", C.c_int32), ("mode", C.c_int32), ("reserved", C.c_int32),
    ]


# (field name, ctypes pointer type) in declaration order, plus scalar size fields
HOST_ARRAY_FIELDS = [
    ("nodeElemIdRelation", c_int32_p), ("elemTypeArr", c_int32_p), ("eqNumIndexArr", c_int32_p),
    ("eqNumStartIndexLoc", c_int32_p), ("numOfDofPerNodeArr", c_int32_p), ("meshCoor", c_double_p),
    ("eleshp", c_double_p), ("eledet", c_double_p), ("mat", c_double_p), ("elemass", c_double_p),
    ("ss", c_double_p), ("phi", c_double_p), ("stressArr", c_double_p),
    ("stressCompIndexArr", c_int32_p), ("pstrain", c_double_p), ("eleporep", c_double_p),
    ("nodalMassArr", c_double_p), ("fnms", c_double_p), ("v1", c_double_p), ("velArr", c_double_p),
    ("dispArr", c_double_p), ("nodalForceArr", c_double_p),
]
FAULT_FIELDS = [("nftnd", c_int32_p), ("nsmp", c_int32_p), ("un", c_double_p),
                ("us", c_double_p), ("ud", c_double_p), ("arn", c_double_p),
                ("fric", c_double_p), ("fnft", c_double_p)]
STATION_FIELDS = [("anonfs", c_int32_p), ("idhist", c_int32_p),
                  ("onFaultQuantHistSCECForm", c_double_p), ("OffFaultStGramSCEC", c_double_p),
                  ("onFaultTPHist", c_double_p)]


class EqdHostArrays(C.Structure):
    _fields_ = ([("nnode", C.c_int32), ("nelem", C.c_int32), ("neq", C.c_int32),
                 ("size_eqidx", C.c_int32), ("size_stress", C.c_int64)]
                + HOST_ARRAY_FIELDS
                + [("ntotft", C.c_int32), ("nftmx", C.c_int32)]
                + FAULT_FIELDS
                + [("numOnFaultSt", C.c_int32), ("numOffFaultSt", C.c_int32)]
                + STATION_FIELDS)


ARRAY_NAMES = [n for n, _ in HOST_ARRAY_FIELDS + FAULT_FIELDS + STATION_FIELDS]
INT_ARRAYS = {n for n, t in HOST_ARRAY_FIELDS + FAULT_FIELDS + STATION_FIELDS if t is c_int32_p}


class EqdOptions(C.Structure):
    _fields_ = [("precision", C.c_int32), ("learned_guess", C.c_int32),
                ("record_tp_hist", C.c_int32), ("tile_shape", C.c_int32),
                ("use_graph", C.c_int32), ("device", C.c_int32), ("table_layout", C.c_int32),
                ("block_node", C.c_int32), ("block_fault", C.c_int32), ("sequential_fault", C.c_int32)]


PREC_FP64 = 0
PREC_FP32 = 1

TABLE_LAYOUTS = {"auto": 0, "streamed": 1, "records": 2}

NEWTON_RECORD = 16
MLP_PARAMS = 5313
MLP_NORM = 34


class MlpTrainOptions(C.Structure):
    _fields_ = [("epochs", C.c_int32), ("batch", C.c_int32), ("lr", C.c_float), ("holdout", C.c_float),
                ("seed", C.c_uint64)]

STATUS = {0: "ok", 1: "bad input", 2: "CUDA error", 3: "device out of memory", 4: "NaN velocity",
          5: "unsupported option", 6: "no CUDA device", 7: "bounded wait timed out",
          8: "call out of order"}


class EqdError(RuntimeError):
    def __init__(self, code, where, detail=""):
        self.code = code
        super().__init__(f"{where}: status {code} ({STATUS.get(code, '?')}){': ' + detail if detail else ''}")


_case_lib = None
_gpu_lib = None


def _load(path):
    if not os.path.exists(path):
        raise NativeLibraryMissing(
            f"{path} is missing; build it with `python -m eqdyna_gb300.build` (or "
            "__graft_entry__.build()).  There is no fallback implementation.")
    return C.CDLL(path)


def case_lib():
    global _case_lib
    if _case_lib is None:
        lib = _load(_build.CASE_LIB)
        lib.eqd_case_build.argtypes = [C.c_char_p, C.POINTER(C.c_void_p)]
        lib.eqd_case_build.restype = C.c_int
        lib.eqd_case_build_opt.argtypes = [C.c_char_p, C.c_int32, C.POINTER(C.c_void_p)]
        lib.eqd_case_build_opt.restype = C.c_int
        lib.eqd_case_view.argtypes = [C.c_void_p, C.POINTER(EqdScalars), C.POINTER(EqdHostArrays)]
        lib.eqd_case_view.restype = C.c_int
        lib.eqd_case_array_len.argtypes = [C.c_void_p, C.c_char_p, C.POINTER(C.c_int32)]
        lib.eqd_case_array_len.restype = C.c_int64
        lib.eqd_case_dims.argtypes = [C.c_void_p] + [C.POINTER(C.c_int32)] * 3 + [
            C.POINTER(C.c_int64), C.POINTER(C.c_int32)]
        lib.eqd_case_dims.restype = C.c_int
        lib.eqd_case_lines.argtypes = [C.c_void_p] + [C.POINTER(c_double_p)] * 3
        lib.eqd_case_lines.restype = C.c_int
        lib.eqd_case_phase_seconds.argtypes = [C.c_void_p, c_double_p]
        lib.eqd_case_phase_seconds.restype = C.c_int
        lib.eqd_case_free.argtypes = [C.c_void_p]
        lib.eqd_case_free.restype = None
        lib.eqd_case_last_error.argtypes = []
        lib.eqd_case_last_error.restype = C.c_char_p
        _case_lib = lib
    return _case_lib


def gpu_lib():
    """The GB300 hot-path library.  Raises if it is not built."""
    global _gpu_lib
    if _gpu_lib is None:
        lib = _load(_build.GPU_LIB)
        lib.eqd_gpu_init.argtypes = [C.POINTER(EqdScalars), C.POINTER(EqdHostArrays),
                                     C.POINTER(EqdOptions), C.POINTER(C.c_void_p)]
        lib.eqd_gpu_init.restype = C.c_int
        lib.eqd_gpu_step.argtypes = [C.c_void_p, C.c_int32, C.c_int32]
        lib.eqd_gpu_step.restype = C.c_int
        lib.eqd_gpu_fetch.argtypes = [C.c_void_p, C.POINTER(EqdHostArrays)]
        lib.eqd_gpu_fetch.restype = C.c_int
        lib.eqd_gpu_fetch_fault.argtypes = [C.c_void_p, c_double_p, c_double_p]
        lib.eqd_gpu_fetch_fault.restype = C.c_int
        lib.eqd_gpu_finalize.argtypes = [C.c_void_p]
        lib.eqd_gpu_finalize.restype = C.c_int
        lib.eqd_gpu_status_string.argtypes = [C.c_int]
        lib.eqd_gpu_status_string.restype = C.c_char_p
        lib.eqd_gpu_stats.argtypes = [C.c_void_p] + [C.POINTER(C.c_int64)] * 4
        lib.eqd_gpu_stats.restype = C.c_int
        lib.eqd_gpu_time.argtypes = [C.c_void_p]
        lib.eqd_gpu_time.restype = C.c_double
        lib.eqd_gpu_profile.argtypes = [C.c_void_p, C.c_int32]
        lib.eqd_gpu_profile.restype = C.c_int
        lib.eqd_gpu_kernel_time.argtypes = [C.c_void_p, C.c_int32, C.POINTER(C.c_double),
                                            C.POINTER(C.c_int64)]
        lib.eqd_gpu_kernel_time.restype = C.c_int
        f_p, d_p, i64_p = C.POINTER(C.c_float), C.POINTER(C.c_double), C.POINTER(C.c_int64)
        lib.eqd_gpu_newton_log.argtypes = [C.c_void_p, C.c_int32, C.c_int32]
        lib.eqd_gpu_newton_records.argtypes = [C.c_void_p, d_p, C.c_int64, i64_p]
        lib.eqd_gpu_mlp_train.argtypes = [C.c_void_p, C.POINTER(MlpTrainOptions), f_p, f_p]
        lib.eqd_gpu_mlp_get.argtypes = [C.c_void_p, f_p, f_p]
        lib.eqd_gpu_mlp_set.argtypes = [C.c_void_p, f_p, f_p]
        lib.eqd_gpu_mlp_enable.argtypes = [C.c_void_p, C.c_int32]
        lib.eqd_gpu_newton_replay.argtypes = [C.c_void_p, C.c_int32, C.c_int32, i64_p, d_p]
        lib.eqd_gpu_newton_replay_records.argtypes = [C.c_void_p, C.c_int32, C.c_int32, d_p, d_p,
                                                      C.POINTER(C.c_int32)]
        lib.eqd_mlp_gradient.argtypes = [C.c_int32, f_p, f_p, f_p, C.c_int32, f_p, f_p]
        for name in ("eqd_gpu_newton_log", "eqd_gpu_newton_records", "eqd_gpu_mlp_train", "eqd_gpu_mlp_get",
                     "eqd_gpu_mlp_set", "eqd_gpu_mlp_enable", "eqd_gpu_newton_replay", "eqd_mlp_gradient",
                     "eqd_gpu_newton_replay_records"):
            getattr(lib, name).restype = C.c_int
        lib.eqd_gpu_element_tables.argtypes = [C.c_int32, C.POINTER(EqdHostArrays), d_p, d_p, d_p, d_p, d_p, d_p, d_p]
        lib.eqd_gpu_element_tables.restype = C.c_int
        lib.eqd_gpu_check_conversions.argtypes = [C.c_int32, C.c_int64, C.c_uint64, C.POINTER(C.c_int64)]
        lib.eqd_gpu_check_conversions.restype = C.c_int
        lib.eqd_gpu_wait_selftest.argtypes = [C.c_int32, C.c_int32, C.POINTER(C.c_int32), d_p]
        lib.eqd_gpu_wait_selftest.restype = C.c_int
        lib.eqd_gpu_fetch_fric_rows.argtypes = [C.c_void_p, C.POINTER(C.c_int32), C.c_int32, d_p]
        lib.eqd_gpu_fetch_fric_rows.restype = C.c_int
        lib.eqd_gpu_step_async.argtypes = [C.c_void_p, C.c_int32, C.c_int32]
        lib.eqd_gpu_step_async.restype = C.c_int
        lib.eqd_gpu_fetch_fric_rows_async.argtypes = [C.c_void_p, C.POINTER(C.c_int32), C.c_int32, d_p,
                                                      C.POINTER(C.c_int64)]
        lib.eqd_gpu_fetch_fric_rows_async.restype = C.c_int
        lib.eqd_gpu_fetch_wait.argtypes = [C.c_void_p, C.c_int64]
        lib.eqd_gpu_fetch_wait.restype = C.c_int
        lib.eqd_gpu_output_setup.argtypes = [C.c_void_p, C.POINTER(C.c_int32), C.c_int32, C.c_int32, C.c_int32]
        lib.eqd_gpu_output_setup.restype = C.c_int
        lib.eqd_gpu_output_drain.argtypes = [C.c_void_p, d_p, d_p, C.c_int32, C.POINTER(C.c_int32),
                                             C.POINTER(C.c_int32)]
        lib.eqd_gpu_output_drain.restype = C.c_int
        lib.eqd_host_alloc.argtypes = [C.c_int64]
        lib.eqd_host_alloc.restype = C.c_void_p
        lib.eqd_host_free.argtypes = [C.c_void_p]
        lib.eqd_host_free.restype = C.c_int
        lib.eqd_gpu_init_times.argtypes = [C.c_void_p, d_p]
        lib.eqd_gpu_init_times.restype = C.c_int
        lib.eqd_ensemble_create.argtypes = [C.POINTER(C.c_void_p), C.c_int32, C.POINTER(C.c_void_p)]
        lib.eqd_ensemble_step.argtypes = [C.c_void_p, C.c_int32]
        lib.eqd_ensemble_destroy.argtypes = [C.c_void_p]
        lib.eqd_ensemble_time.argtypes = [C.c_void_p, d_p]
        lib.eqd_ensemble_mode.argtypes = [C.c_void_p, C.c_int32]
        for name in ("eqd_ensemble_create", "eqd_ensemble_step", "eqd_ensemble_destroy", "eqd_ensemble_time",
                     "eqd_ensemble_mode"):
            getattr(lib, name).restype = C.c_int
        lib.eqd_gpu_newton_counts.argtypes = [C.c_void_p, C.POINTER(C.c_int64)]
        lib.eqd_gpu_newton_counts.restype = C.c_int
        lib.eqd_gpu_table_info.argtypes = [C.c_void_p, C.c_int32, C.POINTER(C.c_int64)]
        lib.eqd_gpu_table_info.restype = C.c_int
        lib.eqd_gpu_fp64_fma_peak.argtypes = [C.c_int32, C.POINTER(C.c_double)]
        lib.eqd_gpu_fp64_fma_peak.restype = C.c_int
        lib.eqd_host_element_order.argtypes = [C.POINTER(EqdHostArrays), C.c_int32, C.c_int32,
                                               C.POINTER(C.c_int32), C.c_int64, i64_p, d_p]
        lib.eqd_host_element_order.restype = C.c_int
        lib.eqd_host_node_order.argtypes = [C.POINTER(EqdHostArrays), C.POINTER(C.c_int32), C.c_int64, i64_p,
                                            C.POINTER(C.c_int32)]
        lib.eqd_host_node_order.restype = C.c_int
        _gpu_lib = lib
    return _gpu_lib


# Entry points the C ABI must export (checked by the CPU test suite).
GPU_SYMBOLS = ["eqd_gpu_init", "eqd_gpu_step", "eqd_gpu_fetch", "eqd_gpu_fetch_fault",
               "eqd_gpu_finalize", "eqd_gpu_status_string", "eqd_gpu_stats", "eqd_gpu_time",
               "eqd_gpu_profile", "eqd_gpu_kernel_time", "eqd_gpu_newton_counts", "eqd_gpu_table_info",
               "eqd_gpu_fetch_fric_rows", "eqd_host_alloc", "eqd_host_free", "eqd_host_element_order",
               "eqd_host_node_order",
               "eqd_gpu_step_async",
               "eqd_gpu_fetch_fric_rows_async", "eqd_gpu_fetch_wait", "eqd_gpu_output_setup",
               "eqd_gpu_output_drain",
               "eqd_ensemble_create", "eqd_ensemble_step", "eqd_ensemble_destroy", "eqd_ensemble_time",
               "eqd_ensemble_mode",
               "eqd_gpu_init_times",
               "eqd_gpu_newton_log", "eqd_gpu_newton_records", "eqd_gpu_mlp_train", "eqd_gpu_mlp_get",
               "eqd_gpu_mlp_set", "eqd_gpu_mlp_enable", "eqd_gpu_newton_replay", "eqd_mlp_gradient",
               "eqd_gpu_newton_replay_records", "eqd_gpu_element_tables",
               "eqd_gpu_fp64_fma_peak", "eqd_gpu_check_conversions", "eqd_gpu_wait_selftest", "eqd_gpu_elem_forces_noalloc"]
CASE_SYMBOLS = ["eqd_case_build", "eqd_case_build_opt", "eqd_case_view", "eqd_case_array_len", "eqd_case_dims",
                "eqd_case_lines", "eqd_case_phase_seconds", "eqd_case_free", "eqd_case_last_error"]


class PinnedArray:
    """A numpy view of page-locked host memory (eqd_host_alloc); freed by close()."""

    def __init__(self, shape, dtype=None):
        import numpy as np
        dtype = np.dtype(dtype or np.float64)
        n = int(np.prod(shape)) * dtype.itemsize
        lib = gpu_lib()
        self._p = lib.eqd_host_alloc(max(n, 1))
        if not self._p:
            raise EqdError(2, "eqd_host_alloc")
        buf = (C.c_char * max(n, 1)).from_address(self._p)
        self.array = np.frombuffer(buf, dtype=dtype, count=int(np.prod(shape))).reshape(shape)

    def close(self):
        if self._p:
            gpu_lib().eqd_host_free(self._p)
            self._p = None
