"""Python host API over the C ABI: the call sequence the Fortran driver makes.

    solver = GpuSolver(case)            # eqd_gpu_init   (after init_vel, src/eqdyna3d.f90:70)
    solver.step(n)                      # eqd_gpu_step   (src/driver.f90:19-29, n steps)
    solver.fetch()                      # eqd_gpu_fetch  (before output_*, src/eqdyna3d.f90:75)
    solver.close()                      # eqd_gpu_finalize

The solver writes results back into the Case's own numpy arrays (the Fortran globalvar view).
There is no CPU fallback: without the built library or a CUDA device the constructor raises.
"""
import ctypes as C

import numpy as np

from . import _native as N

PRECISIONS = {"fp64": N.PREC_FP64, "fp32": N.PREC_FP32}


class GpuSolver:
    def __init__(self, case, precision="fp64", learned_guess=False, use_graph=True, device=0,
                 record_tp_hist=False, table_layout="auto", tile_shape=0, block_node=0, block_fault=0,
                 sequential_fault=False):
        self.lib = N.gpu_lib()
        self.case = case
        self._ha = case.host_arrays()
        opt = N.EqdOptions()
        opt.precision = PRECISIONS[precision]
        opt.learned_guess = int(bool(learned_guess))
        opt.record_tp_hist = int(bool(record_tp_hist))
        opt.use_graph = int(bool(use_graph))
        opt.device = int(device)
        opt.table_layout = N.TABLE_LAYOUTS[table_layout]
        opt.tile_shape = int(tile_shape)
        opt.block_node = int(block_node)
        opt.block_fault = int(block_fault)
        opt.sequential_fault = int(bool(sequential_fault))
        self._opt = opt
        h = C.c_void_p()
        rc = self.lib.eqd_gpu_init(C.byref(case.scalars), C.byref(self._ha), C.byref(opt), C.byref(h))
        if rc != 0:
            raise N.EqdError(rc, "eqd_gpu_init")
        self._h = h
        self.nt = 0
        self.precision = precision

    def step(self, nsteps=1):
        rc = self.lib.eqd_gpu_step(self._h, self.nt + 1, int(nsteps))
        if rc != 0:
            raise N.EqdError(rc, "eqd_gpu_step")
        self.nt += int(nsteps)

    def step_async(self, nsteps=1):
        """Queue nsteps steps without waiting (errors surface at the next fetch_wait or step)."""
        self._rc(self.lib.eqd_gpu_step_async(self._h, self.nt + 1, int(nsteps)), "eqd_gpu_step_async")
        self.nt += int(nsteps)

    def fetch_fric_rows_async(self, rows, out):
        """Queue the read of fric rows (1-based) after the queued steps into out[len(rows)][npair]
        (pinned, e.g. a PinnedArray's array); returns the ticket for fetch_wait."""
        r = np.ascontiguousarray(rows, dtype=np.int32)
        assert out.shape == (len(r), self.case.npair) and out.dtype == np.float64 and out.flags.c_contiguous
        t = C.c_int64()
        self._rc(self.lib.eqd_gpu_fetch_fric_rows_async(self._h, r.ctypes.data_as(N.c_int32_p), len(r),
                                                        out.ctypes.data_as(N.c_double_p), C.byref(t)),
                 "eqd_gpu_fetch_fric_rows_async")
        return t.value

    def fetch_wait(self, ticket):
        """Wait until read `ticket` is in host memory; raises on a NaN velocity or a device timeout."""
        self._rc(self.lib.eqd_gpu_fetch_wait(self._h, int(ticket)), "eqd_gpu_fetch_wait")

    def output_setup(self, surface_nodes, every=10, ring_frames=64):
        """Capture output_gm / output_src_evol frames on the device every `every` steps (first at
        step 1) for these Fortran (1-based) surface node numbers."""
        sn = np.ascontiguousarray(surface_nodes, dtype=np.int32)
        self._out_nsurf, self._out_ring = len(sn), int(ring_frames)
        self._rc(self.lib.eqd_gpu_output_setup(self._h, sn.ctypes.data_as(N.c_int32_p), len(sn), int(every),
                                               int(ring_frames)), "eqd_gpu_output_setup")

    def output_drain(self, max_frames=1 << 30):
        """(first_step, gm[k][n_surface][3], src_evol[k][npair]) of the frames not drained yet."""
        cnt, first = C.c_int32(), C.c_int32()
        n = min(int(max_frames), self._out_ring)  # at most a ring's worth is pending
        gm = np.zeros((n, self._out_nsurf, 3))
        src = np.zeros((n, self.case.npair))
        self._rc(self.lib.eqd_gpu_output_drain(self._h, gm.ctypes.data_as(N.c_double_p),
                                               src.ctypes.data_as(N.c_double_p), n, C.byref(cnt),
                                               C.byref(first)), "eqd_gpu_output_drain")
        return first.value, gm[: cnt.value], src[: cnt.value]

    def run(self):
        self.step(self.case.nstep - self.nt)

    def fetch(self):
        rc = self.lib.eqd_gpu_fetch(self._h, C.byref(self._ha))
        if rc != 0:
            raise N.EqdError(rc, "eqd_gpu_fetch")

    def fetch_fault(self, fric=None, fnft=None):
        fric = self.case.arrays["fric"] if fric is None else fric
        fnft = self.case.arrays["fnft"] if fnft is None else fnft
        rc = self.lib.eqd_gpu_fetch_fault(self._h, fric.ctypes.data_as(N.c_double_p),
                                          fnft.ctypes.data_as(N.c_double_p))
        if rc != 0:
            raise N.EqdError(rc, "eqd_gpu_fetch_fault")

    def stats(self):
        vals = [C.c_int64() for _ in range(4)]
        rc = self.lib.eqd_gpu_stats(self._h, *[C.byref(v) for v in vals])
        if rc != 0:
            raise N.EqdError(rc, "eqd_gpu_stats")
        return dict(zip(["newton_iters", "newton_maxhits", "elem_updates", "kernel_launches"],
                        [v.value for v in vals]))

    def profile(self, enable=True, reset=False, calls_only=False):
        """Per-launch CUDA events (the reference's order, no graph), or with calls_only events around
        each step call only (the production path: graphs and the overlapped schedule)."""
        if reset:
            self.lib.eqd_gpu_profile(self._h, 2)
        self._rc(self.lib.eqd_gpu_profile(self._h, (3 if calls_only else 1) if enable else 0), "eqd_gpu_profile")

    KERNEL_KINDS = {"step": 0, "node_update": 1, "elem_interior": 2, "elem_pml": 3, "fault": 4}

    def kernel_times(self):
        """{kind: (total ms, launches)} accumulated while profiling."""
        out = {}
        for name, k in self.KERNEL_KINDS.items():
            ms, n = C.c_double(), C.c_int64()
            self.lib.eqd_gpu_kernel_time(self._h, k, C.byref(ms), C.byref(n))
            out[name] = (ms.value, n.value)
        return out

    def newton_counts(self):
        """Rate-and-state Newton counters since init: iterations as the reference counts them,
        solves that hit the 20-iteration cap, iterations executed, learned guesses used, learned
        solves repeated from the plain guess."""
        out = (C.c_int64 * 5)()
        rc = self.lib.eqd_gpu_newton_counts(self._h, out)
        if rc != 0:
            raise N.EqdError(rc, "eqd_gpu_newton_counts")
        return dict(zip(["iterations", "ivmax_hits", "executed", "learned", "fallbacks"], list(out)))

    def fetch_fric_rows(self, rows, out):
        """Copy fric rows (1-based) into out[len(rows)][npair] (e.g. a PinnedArray's array)."""
        r = np.ascontiguousarray(rows, dtype=np.int32)
        assert out.shape == (len(r), self.case.npair) and out.dtype == np.float64 and out.flags.c_contiguous
        self._rc(self.lib.eqd_gpu_fetch_fric_rows(self._h, r.ctypes.data_as(N.c_int32_p), len(r),
                                                  out.ctypes.data_as(N.c_double_p)), "eqd_gpu_fetch_fric_rows")

    def init_times(self):
        """Wall time (s) of the phases of eqd_gpu_init."""
        ms = (C.c_double * 8)()
        self._rc(self.lib.eqd_gpu_init_times(self._h, ms), "eqd_gpu_init_times")
        names = ["nodes", "element_order", "element_tables", "tiles", "tables_upload", "fault_stations"]
        return {n: round(ms[k] / 1e3, 3) for k, n in enumerate(names)}

    # ---- learned Newton initial guess ----
    def newton_log(self, nsteps, stride=1):
        """Log the rate-and-state Newton solves of the next nsteps * stride steps (one in stride)."""
        self._rc(self.lib.eqd_gpu_newton_log(self._h, int(nsteps), int(stride)), "eqd_gpu_newton_log")

    def newton_records(self):
        """Logged solves as an array [n][16] (column meaning: EQD_NEWTON_RECORD)."""
        n = C.c_int64()
        self._rc(self.lib.eqd_gpu_newton_records(self._h, None, 0, C.byref(n)), "eqd_gpu_newton_records")
        buf = np.zeros((n.value, N.NEWTON_RECORD))
        self._rc(self.lib.eqd_gpu_newton_records(self._h, buf.ctypes.data_as(N.c_double_p), n.value, C.byref(n)),
                 "eqd_gpu_newton_records")
        return buf

    def train_mlp(self, epochs=8, batch=4096, lr=1e-3, holdout=0.05, seed=20261203):
        """Train the guess on the logged solves and enable it; returns the loss history."""
        opt = N.MlpTrainOptions(int(epochs), int(batch), float(lr), float(holdout), int(seed))
        el = np.zeros(max(int(epochs), 1), dtype=np.float32)
        hl = C.c_float()
        self._rc(self.lib.eqd_gpu_mlp_train(self._h, C.byref(opt), el.ctypes.data_as(C.POINTER(C.c_float)),
                                            C.byref(hl)), "eqd_gpu_mlp_train")
        return {"epoch_loss": el[: int(epochs)].tolist(), "holdout_loss": hl.value}

    def mlp_state(self):
        params = np.zeros(N.MLP_PARAMS, dtype=np.float32)
        norm = np.zeros(N.MLP_NORM, dtype=np.float32)
        self._rc(self.lib.eqd_gpu_mlp_get(self._h, params.ctypes.data_as(C.POINTER(C.c_float)),
                                          norm.ctypes.data_as(C.POINTER(C.c_float))), "eqd_gpu_mlp_get")
        return params, norm

    def set_mlp(self, params, norm):
        params = np.ascontiguousarray(params, dtype=np.float32)
        norm = np.ascontiguousarray(norm, dtype=np.float32)
        self._rc(self.lib.eqd_gpu_mlp_set(self._h, params.ctypes.data_as(C.POINTER(C.c_float)),
                                          norm.ctypes.data_as(C.POINTER(C.c_float))), "eqd_gpu_mlp_set")

    def enable_mlp(self, on=True):
        self._rc(self.lib.eqd_gpu_mlp_enable(self._h, int(bool(on))), "eqd_gpu_mlp_enable")

    def replay(self, learned=False, fast=True, values=False):
        """Re-solve the logged records from the plain or learned guess, with the fault kernel's
        loop (fast) or the reference's loop verbatim: counts (+ slip rates when values=True)."""
        counts = (C.c_int64 * 5)()
        v = None
        vp = None
        if values:
            n = C.c_int64()
            self._rc(self.lib.eqd_gpu_newton_records(self._h, None, 0, C.byref(n)), "eqd_gpu_newton_records")
            v = np.zeros(n.value)
            vp = v.ctypes.data_as(N.c_double_p)
        self._rc(self.lib.eqd_gpu_newton_replay(self._h, int(bool(learned)), int(bool(fast)), counts, vp),
                 "eqd_gpu_newton_replay")
        out = dict(zip(["iterations", "ivmax_hits", "executed", "records", "fallbacks"], list(counts)))
        return (out, v) if values else out

    def replay_records(self, learned=False, fast=True):
        """Per logged record of the same replay: converged slip rate, step ratio of the last
        evaluation, iterations, reached-20, repeated-from-the-plain-guess and (fast loop) how the
        loop ended (0 exit test or cap, 1 fixed point, 2/3 a 2-cycle)."""
        n = C.c_int64()
        self._rc(self.lib.eqd_gpu_newton_records(self._h, None, 0, C.byref(n)), "eqd_gpu_newton_records")
        v, step = np.zeros(n.value), np.zeros(n.value)
        flags = np.zeros(n.value, dtype=np.int32)
        self._rc(self.lib.eqd_gpu_newton_replay_records(self._h, int(bool(learned)), int(bool(fast)),
                                                        v.ctypes.data_as(N.c_double_p),
                                                        step.ctypes.data_as(N.c_double_p),
                                                        flags.ctypes.data_as(C.POINTER(C.c_int32))),
                 "eqd_gpu_newton_replay_records")
        return {"v": v, "step": step, "iters": flags & 0xFF, "capped": (flags >> 8) & 1,
                "fallback": (flags >> 9) & 1, "exit": flags >> 10}

    @staticmethod
    def _rc(rc, what):
        if rc != 0:
            raise N.EqdError(rc, what)

    def table_info(self):
        """Binary32 element-table layout per group: {"interior"|"pml": {layout, elements, records,
        record_floats}}; layout is "records", "streamed" or None (empty group / binary64 form)."""
        out = {}
        for name, grp in (("interior", 0), ("pml", 1)):
            info = (C.c_int64 * 8)()
            rc = self.lib.eqd_gpu_table_info(self._h, grp, info)
            if rc != 0:
                raise N.EqdError(rc, "eqd_gpu_table_info")
            out[name] = {"layout": {0: None, 1: "streamed", 2: "records"}[info[0]], "elements": info[1],
                         "records": info[2], "record_floats": info[3], "tiles": info[4], "slots": info[5],
                         "max_tile_nodes": info[6], "tile_nodes": info[7]}
        return out

    @property
    def time(self):
        return self.lib.eqd_gpu_time(self._h)

    def close(self):
        if getattr(self, "_h", None):
            self.lib.eqd_gpu_finalize(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Ensemble:
    """Several GpuSolver members (scenarios of any size and time step, binary32 form with
    record-indexed tables) advanced together: one launch per kernel per step over all members."""

    def __init__(self, solvers, persistent=False):
        self.lib = N.gpu_lib()
        self.solvers = list(solvers)
        hs = (C.c_void_p * len(self.solvers))(*[s._h for s in self.solvers])
        h = C.c_void_p()
        rc = self.lib.eqd_ensemble_create(hs, len(self.solvers), C.byref(h))
        if rc != 0:
            raise N.EqdError(rc, "eqd_ensemble_create")
        self._h = h
        if persistent:
            self.set_mode(1)

    def set_mode(self, mode):
        """0: one launch per kernel per step, step graphs; 1: one persistent launch per step() call."""
        rc = self.lib.eqd_ensemble_mode(self._h, int(mode))
        if rc != 0:
            raise N.EqdError(rc, "eqd_ensemble_mode")

    def step(self, nsteps=1):
        rc = self.lib.eqd_ensemble_step(self._h, int(nsteps))
        if rc != 0:
            raise N.EqdError(rc, "eqd_ensemble_step")
        for s in self.solvers:
            s.nt += int(nsteps)

    @property
    def last_step_ms(self):
        """Device time (CUDA events on the ensemble's stream) of the last step() call."""
        ms = C.c_double()
        rc = self.lib.eqd_ensemble_time(self._h, C.byref(ms))
        if rc != 0:
            raise N.EqdError(rc, "eqd_ensemble_time")
        return ms.value

    def close(self):
        if self._h:
            self.lib.eqd_ensemble_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def mlp_gradient(params, x, t, device=0):
    """Loss sum((y - t)^2) / (2 n) and its gradient computed by the tensor-core training kernel
    (x: [n][6] normalised inputs, t: [n] normalised targets)."""
    lib = N.gpu_lib()
    params = np.ascontiguousarray(params, dtype=np.float32)
    x = np.ascontiguousarray(x, dtype=np.float32)
    t = np.ascontiguousarray(t, dtype=np.float32)
    loss = C.c_float()
    grad = np.zeros(N.MLP_PARAMS, dtype=np.float32)
    fp = C.POINTER(C.c_float)
    rc = lib.eqd_mlp_gradient(int(device), params.ctypes.data_as(fp), x.ctypes.data_as(fp), t.ctypes.data_as(fp),
                              int(len(t)), C.byref(loss), grad.ctypes.data_as(fp))
    if rc != 0:
        raise N.EqdError(rc, "eqd_mlp_gradient")
    return loss.value, grad
