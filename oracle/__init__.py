"""ORACLE (test infrastructure only): ctypes wrapper of oracle/liboracle.so.

Only tests/, __graft_entry__.smoke() and the CPU-baseline leg of bench.py import this module, and
only as the checker.  The product package eqdyna_gb300 never imports it.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            from eqdyna_gb300 import build
            build.build_oracle()
        from eqdyna_gb300 import _native as N
        L = C.CDLL(LIB_PATH)
        L.oracle_create.argtypes = [C.POINTER(N.EqdScalars), C.POINTER(N.EqdHostArrays), C.c_int]
        L.oracle_create.restype = C.c_void_p
        L.oracle_step.argtypes = [C.c_void_p, C.c_int, C.c_int]
        L.oracle_step.restype = C.c_int
        L.oracle_time.argtypes = [C.c_void_p]
        L.oracle_time.restype = C.c_double
        L.oracle_stats.argtypes = [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                   C.POINTER(C.c_int32)]
        L.oracle_stats.restype = None
        L.oracle_log_newton.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.c_int64]
        L.oracle_log_newton.restype = C.c_int64
        L.oracle_free.argtypes = [C.c_void_p]
        L.oracle_free.restype = None
        _lib = L
    return _lib


class Oracle:
    """Runs the binary64 CPU restatement in place on a Case's arrays."""

    def __init__(self, case, nthreads=1):
        self.case = case
        self._ha = case.host_arrays()
        self._h = lib().oracle_create(C.byref(case.scalars), C.byref(self._ha), nthreads)
        self.nt = 0

    def step(self, nsteps=1):
        rc = lib().oracle_step(self._h, self.nt + 1, nsteps)
        if rc != 0:
            raise RuntimeError(f"oracle step failed with status {rc}")
        self.nt += nsteps

    def run(self):
        self.step(self.case.nstep - self.nt)

    @property
    def time(self):
        return lib().oracle_time(self._h)

    def stats(self):
        it, mh, nc = C.c_int64(), C.c_int64(), C.c_int32()
        lib().oracle_stats(self._h, C.byref(it), C.byref(mh), C.byref(nc))
        return {"newton_iters": it.value, "newton_maxhits": mh.value, "colours": nc.value}

    def start_newton_log(self, cap):
        lib().oracle_log_newton(self._h, None, int(cap))

    def newton_log(self, cap):
        buf = np.zeros((int(cap), 7), dtype=np.float64)
        n = lib().oracle_log_newton(self._h, buf.ctypes.data_as(C.POINTER(C.c_double)), int(cap))
        return buf[:n]

    def close(self):
        if self._h:
            lib().oracle_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
