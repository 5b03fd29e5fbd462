#!/usr/bin/env python3
"""Benchmark of the EQdyna explicit-dynamics hot path on GB300.

Metric: element-updates/s = elements advanced x steps / step-loop time, for the binary32 form with
the learned Newton guess against the plain binary64 form on one GB300, at <= 1 % slip-rate error.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--config C1] [--precision fp64|fp32]
                  [--learned 0|1] [--scale S] [--impl ours|reference]

Workload: the configuration the metric is quoted on, C1 (rate-and-state aging law, dx = 100 m,
20,216,000 elements with a 40-layer PML), synthetic seeded inputs (eqdyna_gb300.configs).
A "step" is one time step of the hot path over the whole mesh.

value      device time of exactly K steps, CUDA events recorded on the library's own stream
           around every kernel launch (inputs resident in HBM, working set far above L2).
e2e        the same metric through the C ABI with host buffers: eqd_gpu_init (host->device copy
           of every table), then per step eqd_gpu_step + eqd_gpu_fetch_fault (device->host read
           of the fault state), then eqd_gpu_fetch; host wall clock around all of it.
roofline   dominant kernel (the element kernel with the largest event time): algorithmic bytes per
           launch / average launch duration, against the measured HBM copy bandwidth.
cpu_baseline the oracle (binary64 C++ restatement of the reference step, OpenMP over all host
           cores) on a bounded sample of the same mesh.
--impl reference times that CPU implementation alone (the reference's Fortran/MPI/netCDF build
           is not available on this stack), printing the same JSON line with impl=reference.
Multi-GPU: the hot path runs one mesh per GPU (no domain decomposition); N ranks run N independent
           replicas, value = all elements x steps / max time over ranks ("weak").
"""
import argparse
import json
import os
import shutil
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "element-updates/s, FP32+learned vs plain FP64 on 1 GB300 at ≤1% slip-rate L2 error"
UNIT = "element-updates/s"

# Algorithmic bytes per element update: the compulsory traffic of the layout the kernel uses, with
# perfect reuse of nodal data.
#   fp64 (per-element tables): connectivity 32, shape gradients 192, det 8, lambda/mu 16, stress
#     read+write 96 (PML 240), hourglass vectors 256 and stiffness 48, PML factors 48.
#   fp32 streamed: incidence list 16 (replaces connectivity), then the fp64 tables in binary32.
#   fp32 record-indexed: incidence list 16, record index 4, stress read+write 48 (PML 120), PML
#     axis indices 8; plus the record table once per launch (records x floats x 4).
# Node share: gather of velocity and displacement plus the force scatter (+ split fields on PML
# nodes).
ELEM_BYTES = {"fp64": {"interior": 32 + 192 + 8 + 16 + 96 + 256 + 48,
                       "pml": 32 + 192 + 8 + 16 + 240 + 256 + 48 + 48},
              "fp32": {"interior": 16 + 96 + 4 + 8 + 48 + 128 + 24,
                       "pml": 16 + 96 + 4 + 8 + 120 + 128 + 24 + 24}}
REC_ELEM_BYTES = {"interior": 16 + 4 + 48, "pml": 16 + 4 + 120 + 8}
# Node update (per node): fp64 form 152 B (3-DOF) / 536 B (PML); fp32 form 148 B / 340 B
# (binary64 velocity and displacement, binary32 forces, 1/m and PML split fields, plus the
# binary32 copies the element kernels gather).
NODE_BYTES = {"fp64": (152, 536), "fp32": (148, 340)}
# DRAM traffic (dram__bytes_read.sum + dram__bytes_write.sum) per unit of the binary32 kernels on
# the full C1 mesh (20,216,000 elements, 20,477,812 nodes; one record per group), from one 1-pass
# ncu capture of the bench's own launches (profiles/dram_C1_full_fp32.md), scaled to a launch by
# its unit count.  At full size the node update moves 0.97 of its algorithmic bytes; the element
# passes 1.29 (PML) and 1.38 (interior): node data gathered again by neighbouring tiles, and the
# interior pass's 2 KB slot table per tile.
NCU_TRAFFIC_PER_UNIT = {("elem_interior", "fp32", "records", 1): (1.0086e9 + 0.29488e9) / 9000000,
                        ("elem_pml", "fp32", "records", 1): (2.0250e9 + 1.1671e9) / 11216000,
                        ("node_update", "fp32", None, None): (2.3376e9 + 2.7196e9) / 20477812}
JOB_STEPS = {"C0": 1000, "C1": 4000, "C2": 6000, "C3": 5000}
# the result a host program reads after every step: fric rows 71-76 (slip s/d/n, slip rate s/d,
# peak slip rate) of every fault pair
RESULT_ROWS = [71, 72, 73, 74, 75, 76]
NODE_GATHER_BYTES = {"fp64": 48 + 24, "fp32": 24 + 12}
PML_NODE_EXTRA = {"fp64": 72, "fp32": 36}
FP64_FLOPS_PER_ELEM = {"interior": 2 * 423, "pml": 2 * 470}


def _peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        if shutil.which("nvidia-smi"):
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            t0 = time.perf_counter()
            while not self.lines and time.perf_counter() - t0 < 5.0 and self.proc.poll() is None:
                time.sleep(0.01)  # the sampler is running before the timed region starts
        self.first = max(len(self.lines) - 1, 0)  # the last sample before the region, then all inside
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines[getattr(self, "first", 0):]:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def build_case(config, scale, nsteps, workdir, tables=True, hourglass=0):
    """The configuration's case; tables=False builds the mesh only (eqd_gpu_init then builds the
    per-element tables and nodal masses on the device); hourglass = 1 or 2 sets C_hg (C0 only:
    its "hourglass coefficient 0.1" is the viscous form's kapa_hg)."""
    from eqdyna_gb300 import configs
    from eqdyna_gb300.case import Case
    extra = {"C_hg": hourglass} if (hourglass and config == "C0") else {}
    configs.CONFIGS[config](workdir, scale=scale, nsteps=nsteps, **extra)
    return Case.from_dir(workdir, tables=tables)


def algorithmic_bytes(case, precision, tables=None):
    """Per-launch algorithmic bytes of the two element kernels (interior, PML) for the table
    layout each group runs with (`tables` = GpuSolver.table_info())."""
    import numpy as np
    a = case.arrays
    et = a["elemTypeArr"]
    conn = a["nodeElemIdRelation"].reshape(-1, 8)
    nd = a["numOfDofPerNodeArr"]
    out = {}
    for name, mask in (("interior", et != 2), ("pml", et == 2)):
        ne = int(mask.sum())
        nodes = np.unique(conn[mask]) - 1 if ne else np.zeros(0, dtype=np.int64)
        npml_nodes = int((nd[nodes] == 12).sum()) if ne else 0
        t = (tables or {}).get(name) or {}
        if precision == "fp32" and t.get("layout") == "records":
            elem = ne * REC_ELEM_BYTES[name] + t["records"] * t["record_floats"] * 4
        else:
            elem = ne * ELEM_BYTES[precision][name]
        out[name] = (elem + len(nodes) * NODE_GATHER_BYTES[precision] + npml_nodes * PML_NODE_EXTRA[precision], ne)
    n12 = int((nd == 12).sum())
    n3 = len(nd) - n12
    out["node"] = (n3 * NODE_BYTES[precision][0] + n12 * NODE_BYTES[precision][1], len(nd))
    return out


def fault_result(case):
    """Copies of the arrays the accuracy condition compares: fric, rupture times, station histories."""
    a = case.arrays
    out = {"fric": case.fric().copy(), "fnft": a["fnft"][: case.npair].copy()}
    for k in ("onFaultQuantHistSCECForm", "OffFaultStGramSCEC"):
        out[k] = a[k].copy() if a.get(k) is not None and a[k].size else None
    return out


def compare_fault_results(got, ref, dt):
    """Errors of `got` against `ref` (the plain binary64 form): relative L2 of the final slip rate
    (against the larger of the final and the peak slip-rate fields: after arrest the final rate is
    round-off), slip, peak slip rate and the station histories; rupture times in steps."""
    import numpy as np
    fa, fb = got["fric"], ref["fric"]

    def rel(x, y):
        return float(np.linalg.norm(x - y) / max(np.linalg.norm(y), 1e-300))
    scale = max(np.linalg.norm(fb[:, 73:75]), np.linalg.norm(fb[:, 75]), 1e-300)
    ta, tb = got["fnft"], ref["fnft"]
    ra, rb = ta < 1e4, tb < 1e4
    both = ra & rb
    out = {"slip_rate_rel_l2": float(np.linalg.norm(fa[:, 73:75] - fb[:, 73:75]) / scale),
           "slip_rel_l2": rel(fa[:, 70:72], fb[:, 70:72]),
           "peak_rate_rel_l2": rel(fa[:, 75], fb[:, 75]),
           "ruptured": int(rb.sum()), "ruptured_fp32": int(ra.sum()),
           "rupture_flips": int((ra != rb).sum()),
           "rupture_dt_max": float(np.abs(ta[both] - tb[both]).max() / dt) if both.any() else None,
           "rupture_dt_mean": float(np.abs(ta[both] - tb[both]).mean() / dt) if both.any() else None}
    if both.any():  # distribution of the rupture-time differences (steps) over the pairs ruptured in both
        d = np.abs(ta[both] - tb[both]) / dt
        out["rupture_within_1_step"] = float((d <= 1.0 + 1e-9).mean())
        out["rupture_dt_p99"] = float(np.quantile(d, 0.99))
    for key, name in (("onFaultQuantHistSCECForm", "onfault_stations_rel_l2"),
                      ("OffFaultStGramSCEC", "offfault_stations_rel_l2")):
        if got.get(key) is not None and ref.get(key) is not None:
            out[name] = rel(got[key], ref[key])
    return out


def kernel_rooflines(kt, ab, precision, tables, hbm_peak, traffic_measured=None):
    """Per kernel: algorithmic bytes per launch / average event time against the HBM peak, its
    share of the sequential step and (binary32 form) the DRAM bytes ncu measured per launch."""
    step_ms_total = kt["step"][0]
    per_kernel = {}
    for kname, key in (("node_update", "node"), ("elem_interior", "interior"), ("elem_pml", "pml")):
        ms, nl = kt[kname]
        if nl == 0:
            continue
        avg_s = ms / 1e3 / nl
        tkey = (kname, precision, (tables.get(key) or {}).get("layout"), (tables.get(key) or {}).get("records"))
        traffic = (traffic_measured or {}).get(tkey)
        d = {"achieved": ab[key][0] / avg_s / 1e9, "frac": ab[key][0] / avg_s / 1e9 / hbm_peak,
             "algorithmic_bytes_per_launch": ab[key][0], "units_per_launch": ab[key][1],
             "avg_launch_ms": avg_s * 1e3, "share": ms / step_ms_total,
             "traffic": traffic * ab[key][1] if traffic else None}
        if d["traffic"]:
            d["achieved_dram"] = d["traffic"] / avg_s / 1e9
            d["frac_dram"] = d["achieved_dram"] / hbm_peak
        per_kernel[kname] = d
    return per_kernel


def fp64_compute_roofline(kt, ab, lib, device):
    """Binary64 FMA throughput of the busier element kernel against the measured FP64 peak."""
    import ctypes as C
    fp64 = C.c_double()
    key = "interior" if kt["elem_interior"][0] >= kt["elem_pml"][0] else "pml"
    ms, nl = kt["elem_" + key]
    if lib.eqd_gpu_fp64_fma_peak(device, C.byref(fp64)) != 0 or not nl:
        return None
    fl = FP64_FLOPS_PER_ELEM[key] * ab[key][1] / (ms / 1e3 / nl) / 1e12
    return {"kernel": "elem_" + key, "achieved_tflops": fl, "peak_tflops": fp64.value,
            "frac": fl / fp64.value, "flops_per_element": FP64_FLOPS_PER_ELEM[key],
            "peak_source": "measured FMA-chain kernel"}


def newton_classes(rec, plain, learned, log_nt0, stride, npair, split_step):
    """Iterations of the logged solves per class, from the plain and from the learned guess.
    Classes: a solve whose plain run reached the 20-iteration cap (creeping pairs at round-off) or
    met the exit test; slipping (converged slip rate >= 1e-3 m/s, the rupture-time threshold) or
    not; logged before or after `split_step` (the step where the job switches to the learned
    guess)."""
    import numpy as np
    n = rec.shape[0]
    step = log_nt0 + (np.arange(n) // npair + 1) * stride
    capped = plain["capped"] == 1
    sliding = rec[:, 14] >= 1e-3
    out = {}
    for phase, pm in (("before_training", step <= split_step), ("after_training", step > split_step)):
        for cname, cm in (("capped", capped), ("converged", ~capped)):
            for sname, sm in (("slipping", sliding), ("creeping", ~sliding)):
                m = pm & cm & sm
                k = int(m.sum())
                if k == 0:
                    continue
                pi = int(plain["iters"][m].sum())
                li = int(learned["iters"][m].sum())
                out[f"{phase}/{cname}/{sname}"] = {
                    "solves": k, "plain_iterations": pi, "learned_iterations": li,
                    "change": round((li - pi) / pi, 4) if pi else None,
                    "repeats_from_plain": int(learned["fallback"][m].sum())}
    return out


def run_cpu_baseline(case, max_seconds=20.0):
    from oracle import Oracle
    nth = os.cpu_count() or 1
    cpu = case.clone()
    o = Oracle(cpu, nth)
    o.step(1)  # first step outside the timing (touches every page)
    n, t0 = 0, time.perf_counter()
    while True:
        o.step(1)
        n += 1
        el = time.perf_counter() - t0
        if el > max_seconds or n >= 50:
            break
    o.close()
    return {"value": case.sizes["nelem"] * n / el, "unit": UNIT, "cores": nth, "kind": "port",
            "sample": f"{n} time steps of the full mesh ({case.sizes['nelem']} elements) after one "
                      "untimed step, binary64 C++ restatement of the reference step, OpenMP"}


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allreduce_max(x, world):
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def allreduce_sum(x, world):
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def bench_reference(args, world, rank):
    """CPU implementation of the reference step (the oracle restatement), all host cores."""
    if rank != 0:
        return None
    with tempfile.TemporaryDirectory(prefix="eqd_bench_") as tmp:
        if args.config == "C4":  # one member of the ensemble (the oracle runs one scenario at a time)
            from eqdyna_gb300.case import Case
            from eqdyna_gb300.configs import config_c4
            case = Case.from_dir(config_c4(tmp, 0, nsteps=max(args.steps + args.warmup + 2, 10)))
        else:
            case = build_case(args.config, args.scale, max(args.steps + args.warmup + 2, 10), tmp)
        from oracle import Oracle
        nth = os.cpu_count() or 1
        o = Oracle(case, nth)
        o.step(max(args.warmup - 1, 0))
        t0 = time.perf_counter()
        o.step(1)  # the last warm-up step sizes the timed sample (about 60 s of CPU work at most)
        per_step = time.perf_counter() - t0
        nsteps = max(1, min(args.steps, int(60.0 / max(per_step, 1e-9))))
        t0 = time.perf_counter()
        o.step(nsteps)
        el = time.perf_counter() - t0
        ne = case.sizes["nelem"]
        v = ne * nsteps / el
        from eqdyna_gb300.configs import WORKLOADS
        line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": el / nsteps * 1e3,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic (seeded config generator)",
                "config": {"workload": f"{args.config}: {WORKLOADS[args.config]}", "elements": ne,
                           "scale": args.scale},
                "cpu_baseline": {"value": v, "unit": UNIT, "cores": nth, "kind": "port",
                                 "sample": f"{nsteps} full-mesh time steps (of the {args.steps} asked, "
                                           "bounded to about 60 s of CPU work) after "
                                           f"{args.warmup} untimed; the reference Fortran build needs "
                                           "MPI and netCDF, which this stack does not have"},
                "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        return line


def bench_ours(args, world, rank, local):
    import ctypes as C
    import numpy as np
    from eqdyna_gb300 import _native as N
    from eqdyna_gb300.configs import WORKLOADS
    from eqdyna_gb300.solver import GpuSolver

    lib = N.gpu_lib()
    t_setup = time.perf_counter()
    tmp = tempfile.mkdtemp(prefix="eqd_bench_")
    job = args.job_steps if args.job_steps > 0 else JOB_STEPS[args.config]
    total_steps = max(job, args.warmup + min(args.steps, 40) + args.steps + 4)
    mesh_only = bool(args.mesh_only) if args.mesh_only >= 0 else (args.config == "C2" and args.scale < 1.5)
    case = build_case(args.config, args.scale, total_steps, tmp, tables=not mesh_only, hourglass=args.hourglass)
    shutil.rmtree(tmp, ignore_errors=True)
    ne = case.sizes["nelem"]
    host_bytes_in = sum(v.nbytes for k, v in case.arrays.items() if v is not None)
    setup_s = time.perf_counter() - t_setup
    npair = case.npair
    d2h_per_step = len(RESULT_ROWS) * npair * 8  # the step's result rows of fric
    from eqdyna_gb300.autotune import tuned_options
    launch = tuned_options(args.config, local) if (args.tuned and args.precision == "fp32") else {}
    args.learned = int(bool(args.learned) and case.scalars.friclaw in (3, 4))  # rate-and-state only
    log_stride, log_steps = args.log_stride, args.log_steps
    if args.learned and log_steps * log_stride > job // 2:
        # a short job: the logged warm-up takes about half of it (one step in log_stride)
        log_stride = max(1, min(log_stride, job // 4))
        log_steps = max(1, (job // 2) // log_stride)
    nlog = log_steps * log_stride if args.learned else 0

    # ---- end to end: the whole job through the C ABI with host buffers ----
    e2e_case = case.clone()
    rows = RESULT_ROWS
    pinned = [N.PinnedArray((len(rows), npair)) for _ in range(2)]

    def run_steps(n):
        # each step's result rows are read into pinned memory; step k+1 is queued before the host
        # waits for step k's rows, so the device does not idle between steps
        prev = None
        for k in range(n):
            s.step_async(1)
            ticket = s.fetch_fric_rows_async(rows, pinned[k % 2].array)
            if prev is not None:
                s.fetch_wait(prev)
            prev = ticket
        if prev is not None:
            s.fetch_wait(prev)

    barrier(world)
    t0 = time.perf_counter()
    s = GpuSolver(e2e_case, precision=args.precision, learned_guess=args.learned, device=local,
                  table_layout=args.tables, **launch)
    t_init = time.perf_counter() - t0
    init_phases = s.init_times()
    done, train_s, hist, warm_s = 0, 0.0, None, 0.0
    if args.learned:  # plain warm-up whose Newton solves are the training data, then training
        t1 = time.perf_counter()
        s.newton_log(nlog // log_stride, log_stride)
        run_steps(nlog)
        done = nlog
        warm_s = time.perf_counter() - t1
        t1 = time.perf_counter()
        hist = s.train_mlp(epochs=args.epochs, batch=4096, lr=1e-3, holdout=0.05, seed=20261203)
        train_s = time.perf_counter() - t1
    t1 = time.perf_counter()
    run_steps(job - done)
    steps_s = time.perf_counter() - t1
    t1 = time.perf_counter()
    s.fetch()
    fetch_s = time.perf_counter() - t1
    e2e_s = time.perf_counter() - t0
    for pa in pinned:
        pa.close()
    job_newton = s.newton_counts()
    learned = None
    if args.learned:
        plain = s.replay(learned=False)
        guess = s.replay(learned=True)
        params, norm = s.mlp_state()
        learned = {"records": plain["records"], "logged_steps": nlog // log_stride,
                   "log_stride": log_stride, "train_s": round(train_s, 2), "epochs": args.epochs,
                   "epoch_loss": [round(x, 5) for x in hist["epoch_loss"]],
                   "holdout_loss": round(hist["holdout_loss"], 5),
                   "replay_plain_guess": plain, "replay_learned_guess": guess, "job_newton": job_newton}
    s.close()
    e2e_breakdown = {"init_s": round(t_init, 2), "init_phases_s": init_phases, "logged_warmup_s": round(warm_s, 2), "train_s": round(train_s, 2),
                     "steps_s": round(steps_s, 2), "final_fetch_s": round(fetch_s, 2)}
    e2e_s = allreduce_max(e2e_s, world)
    e2e_result = fault_result(e2e_case)
    del e2e_case

    # ---- device-timed steps (inputs resident in HBM) ----
    dev_case = case.clone()
    s = GpuSolver(dev_case, precision=args.precision, learned_guess=args.learned, device=local,
                  table_layout=args.tables, **launch)
    if args.learned:
        s.set_mlp(params, norm)
    s.step(args.warmup)
    # per-kernel times: CUDA events around every launch over a short segment, issued in the
    # reference's order (no graph, no overlap); they give the kernel shares and rooflines
    s.profile(True, reset=True)
    s.step(min(args.steps, 40))
    s.profile(False)
    kt = s.kernel_times()
    # the timed region: the production path (16-step CUDA graphs, the fault phase overlapped with the
    # next step's node update), CUDA events around the whole call on the library's stream
    n_before = s.newton_counts()
    s.profile(True, reset=True, calls_only=True)
    barrier(world)
    with ClockSampler(local) as clk:
        w0 = time.perf_counter()
        s.step(args.steps)
        wall = time.perf_counter() - w0
    barrier(world)
    s.profile(False)
    timed_ms = s.kernel_times()["step"][0]
    stats = s.stats()
    n_after = s.newton_counts()
    newton = {k: n_after[k] - n_before[k] for k in n_after}
    tables = s.table_info()
    dev_s = allreduce_max(timed_ms / 1e3, world)
    units = allreduce_sum(float(ne) * args.steps, world)
    value = units / dev_s
    s.close()
    del dev_case

    # ---- the plain binary64 method (reference Newton iteration, no learned guess) over the whole
    # job: its speed on the same step indices as the device-timed run (the metric's comparison), the
    # accuracy condition of the metric (this job's final fault state, station histories and rupture
    # times against it; the binary64 form itself matches the oracle to 1e-9 in tests/), its own
    # roofline, and its Newton solves logged across the job for the per-class replay of the learned
    # guess ----
    plain = None
    hbm_peak, peak_kind = _peaks()
    if args.precision == "fp32" and args.plain_check:
        ref_case = case.clone()
        seg0 = args.warmup + min(args.steps, 40)
        with GpuSolver(ref_case, precision="fp64", device=local) as r:
            lstride = max(1, job // 70)
            lsteps = job // lstride
            if args.learned:
                r.newton_log(lsteps, lstride)
            t1 = time.perf_counter()
            res64 = None
            if seg0 + args.steps > job:  # a short job: compare after it, then time the later steps
                r.step(job)
                r.fetch()
                res64 = fault_result(ref_case)
            r.step(args.warmup)
            r.profile(True, reset=True)
            r.step(min(args.steps, 40))
            r.profile(False)
            kt64 = r.kernel_times()
            r.profile(True, reset=True, calls_only=True)
            r.step(args.steps)
            r.profile(False)
            fp64_ms = r.kernel_times()["step"][0]
            if res64 is None:
                r.step(job - seg0 - args.steps)
                r.fetch()
                res64 = fault_result(ref_case)
            job64_s = time.perf_counter() - t1
            classes = None
            if args.learned:
                rec = r.newton_records()
                r.set_mlp(params, norm)
                rp = r.replay_records(learned=False)
                rl = r.replay_records(learned=True)
                classes = newton_classes(rec, rp, rl, 0, lstride, npair, nlog)
                classes = {"logged_steps": lsteps, "log_stride": lstride, "records": int(rec.shape[0]),
                           "plain_iterations": int(rp["iters"].sum()), "learned_iterations": int(rl["iters"].sum()),
                           "classes": classes}
                del rec, rp, rl
        cmp = compare_fault_results(e2e_result, res64, case.scalars.dt)
        fp64_value = ne * args.steps / (fp64_ms / 1e3)
        ab64 = algorithmic_bytes(case, "fp64")
        k64 = kernel_rooflines(kt64, ab64, "fp64", {}, hbm_peak)
        dom64 = max(k64, key=lambda k: k64[k]["share"])
        plain = {"value": fp64_value, "ms_per_step": fp64_ms / args.steps,
                 "speedup": value / world / fp64_value if fp64_value > 0 else None,
                 "steps_compared": job,
                 **cmp,
                 "job_s": round(job64_s, 1),
                 "roofline": {"bound": "fp64", "kernel": dom64, "hbm_frac": k64[dom64]["frac"],
                              "hbm_peak": hbm_peak, "kernels": k64,
                              "fp64": fp64_compute_roofline(kt64, ab64, lib, local)},
                 "newton_replay": classes,
                 "note": "plain binary64 method (reference iteration, no learned guess) on this GPU: speed over "
                         "the same step indices as the device-timed run; errors of the end-to-end job "
                         "(binary32 form, plain warm-up then the learned guess) against it after the whole "
                         "job: final fault state, station histories, rupture times (steps)"}
        del ref_case
        if learned is not None and classes is not None:
            learned["replay_across_job"] = plain.pop("newton_replay")

    # ---- rooflines: every kernel, the one with the largest time share on top ----
    ab = algorithmic_bytes(case, args.precision, tables)
    working_set = ab["interior"][0] + ab["pml"][0] + ab["node"][0]
    # the measured traffic per unit belongs to the mesh it was captured on: full-size C1
    measured = NCU_TRAFFIC_PER_UNIT if (args.config == "C1" and args.scale == 1.0) else None
    per_kernel = kernel_rooflines(kt, ab, args.precision, tables, hbm_peak, measured)
    step_ms_total = kt["step"][0]
    dom = max(per_kernel, key=lambda k: per_kernel[k]["share"])
    d = per_kernel[dom]
    roofline = {"bound": "hbm", "kernel": f"{dom}_{args.precision}", "achieved": d["achieved"], "peak": hbm_peak,
                "unit": "GB/s", "frac": d["frac"], "peak_source": peak_kind, "traffic": d["traffic"],
                "algorithmic_bytes_per_launch": d["algorithmic_bytes_per_launch"],
                "units_per_launch": d["units_per_launch"], "avg_launch_ms": d["avg_launch_ms"],
                "kernels": per_kernel, "kernel_share": {k: v[0] / step_ms_total for k, v in kt.items() if k != "step"}}
    if d.get("frac_dram") is not None:
        roofline["achieved_dram"] = d["achieved_dram"]
        roofline["frac_dram"] = d["frac_dram"]
    if args.precision == "fp64":
        roofline["fp64"] = fp64_compute_roofline(kt, ab, lib, local)
    # (the oracle reads the host tables, which a mesh-only case does not have)
    cpu = (run_cpu_baseline(case, args.cpu_seconds)
           if (rank == 0 and world == 1 and args.cpu_seconds > 0 and not mesh_only) else None)

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dev_s * 1e3 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if args.precision == "fp64" else "f32 elements + f64 state",
            "data": "synthetic (seeded config generator, no external dataset)",
            "config": {"workload": f"{args.config}: {WORKLOADS[args.config]}", "elements": ne,
                       "physical_elements": case.dims["n_phys_elem"], "precision": args.precision,
                       "hourglass": {1: "stiffness (KF78)", 2: f"viscous, kapa_hg {case.scalars.kapa_hg}"}[
                           case.scalars.C_hg],
                       "learned_guess": bool(args.learned), "scale": args.scale,
                       "l2": f"inputs larger than L2: working set {working_set / 1e9:.2f} GB per step "
                             "vs 129 MB L2, no flush",
                       "element_tables": {k: {"layout": v["layout"], "records": v["records"], "tiles": v["tiles"],
                                              "max_tile_nodes": v["max_tile_nodes"],
                                              "node_gathers_per_element": round(v["tile_nodes"] / max(v["elements"], 1), 3),
                                              "live_slots": round(v["elements"] / max(v["slots"], 1), 4)}
                                          for k, v in tables.items()},
                       "launch": launch or "defaults",
                       "setup_tables": "device (mesh-only host case)" if mesh_only else "host case builder",
                       "parallelism": "replicas" if world > 1 else "single GPU",
                       "setup_s": round(setup_s, 1), "setup_phases_s": case.build_phases_s,
                       "wall_ms_per_step": wall * 1e3 / args.steps,
                       "timing": "value: CUDA events around the K-step call on the library's stream (16-step "
                                 "graphs, fault phase beside the next node update); kernel shares and "
                                 "rooflines: per-launch events over up to 40 steps in the reference's order",
                       "sequential_ms_per_step": round(step_ms_total / max(kt["step"][1], 1), 4)},
            "e2e": {"value": ne * job * world / e2e_s, "unit": UNIT, "steps": job,
                    "h2d_bytes_per_step": int(host_bytes_in / job),
                    "d2h_bytes_per_step": int(d2h_per_step + host_bytes_in / job),
                    "breakdown": e2e_breakdown,
                    "note": "whole job through the C ABI: init (every host table to the device), each step "
                            "followed by a read of its result (fric rows 71-76 into pinned host memory; the "
                            "next step is queued before the host waits for that read), final fetch of every "
                            "array"
                            + ("; the first steps run the plain Newton with solve logging, then training"
                               if args.learned else "")},
            "plain_fp64": plain,
            "gpu_launches": int(stats["kernel_launches"]),
            "newton": newton,
            "learned": learned,
            "roofline": roofline, "clocks": clk.summary()}
    if cpu:
        line["cpu_baseline"] = cpu
    return line if rank == 0 else None


def bench_ensemble(args, world, rank, local):
    """C4: an ensemble of members of different mesh sizes and time steps advanced together."""
    import concurrent.futures as cf
    import numpy as np
    from eqdyna_gb300 import _native as N
    from eqdyna_gb300.case import Case
    from eqdyna_gb300.configs import WORKLOADS, config_c4
    from eqdyna_gb300.solver import Ensemble, GpuSolver

    job = args.job_steps if args.job_steps > 0 else 1500
    nsteps = max(job, args.steps + args.warmup + 4)
    t_setup = time.perf_counter()

    def build(k):
        d = tempfile.mkdtemp(prefix=f"eqd_c4_{k}_")
        c = Case.from_dir(config_c4(d, k, nsteps=nsteps))
        shutil.rmtree(d, ignore_errors=True)
        return c
    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        cases = list(ex.map(build, range(args.members)))
    setup_s = time.perf_counter() - t_setup
    ne = [c.sizes["nelem"] for c in cases]
    total = float(sum(ne))
    dxs = {}
    for c in cases:
        dxs[str(int(round(c.scalars.dx)))] = dxs.get(str(int(round(c.scalars.dx))), 0) + 1

    # ---- end to end: the whole ensemble job through the C ABI, every member's peak slip rate
    # (fric row 76) read into pinned memory after every step ----
    pinned = [N.PinnedArray((1, c.npair)) for c in cases]
    barrier(world)
    t0 = time.perf_counter()
    solvers = [GpuSolver(c.clone(), precision="fp32", device=local) for c in cases]
    ens = Ensemble(solvers, persistent=args.ens_mode == 1)
    t_init = time.perf_counter() - t0
    for _ in range(job):
        ens.step(1)
        for sv, pa in zip(solvers, pinned):
            sv.fetch_fric_rows([76], pa.array)
    for sv in solvers:
        sv.fetch()
    e2e_s = time.perf_counter() - t0
    ens.close()
    for sv in solvers:
        sv.close()
    for pa in pinned:
        pa.close()
    e2e_s = allreduce_max(e2e_s, world)

    # ---- device-timed steps ----
    solvers = [GpuSolver(c.clone(), precision="fp32", device=local) for c in cases]
    ens = Ensemble(solvers, persistent=args.ens_mode == 1)
    ens.step(args.warmup)
    barrier(world)
    with ClockSampler(local) as clk:
        ens.step(args.steps)
        dev_ms = ens.last_step_ms
    barrier(world)
    ens.close()
    for sv in solvers:
        sv.close()
    dev_s = allreduce_max(dev_ms / 1e3, world)
    units = allreduce_sum(total * args.steps, world)
    value = units / dev_s
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dev_s * 1e3 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 elements + f64 state",
            "data": "synthetic (seeded config generator, no external dataset)",
            "config": {"workload": f"C4: {WORKLOADS['C4']}", "members": args.members, "elements": int(total),
                       "member_elements": [min(ne), max(ne)], "members_per_dx": dxs,
                       "precision": "fp32", "parallelism": "replicas" if world > 1 else "single GPU",
                       "launch": "one persistent cooperative launch per call" if args.ens_mode == 1
                                 else "one launch per kernel per step, 16-step graphs",
                       "l2": "inputs larger than L2, no flush", "setup_s": round(setup_s, 1)},
            "e2e": {"value": total * job * world / e2e_s, "unit": UNIT, "steps": job,
                    "init_s": round(t_init, 2),
                    "h2d_bytes_per_step": int(sum(sum(v.nbytes for v in c.arrays.values() if v is not None)
                                                  for c in cases) / job),
                    "d2h_bytes_per_step": int(sum(c.npair for c in cases) * 8),
                    "note": "whole ensemble job through the C ABI: init of every member, one ensemble step "
                            "per call followed by a read of every member's peak slip rate into pinned "
                            "memory, final fetch of every member"},
            "gpu_launches": 1 if args.ens_mode == 1 else 4 * args.steps, "clocks": clk.summary()}
    return line if rank == 0 else None


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--config", default="C1")
    ap.add_argument("--scale", type=float, default=1.0)
    ap.add_argument("--precision", default="fp32", choices=["fp64", "fp32"])
    ap.add_argument("--learned", type=int, default=1, help="learned Newton initial guess (rate-and-state)")
    ap.add_argument("--log-steps", type=int, default=70, help="logged warm-up steps (training data)")
    ap.add_argument("--log-stride", type=int, default=10, help="one logged step in this many")
    ap.add_argument("--epochs", type=int, default=8)
    ap.add_argument("--job-steps", type=int, default=0, help="steps of the end-to-end job (0: the config's)")
    ap.add_argument("--tuned", type=int, default=1, help="use the autotuned launch shapes when recorded")
    ap.add_argument("--members", type=int, default=64, help="C4 ensemble size")
    ap.add_argument("--ens-mode", type=int, default=1, choices=[0, 1],
                    help="C4: 0 batched launches in step graphs, 1 one persistent launch per call "
                         "(19 %% faster on the 64-member C4)")
    ap.add_argument("--tables", default="auto", choices=["auto", "streamed", "records"],
                    help="binary32 element-table layout")
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--plain-check", type=int, default=1,
                    help="also run the plain binary64 method on the same steps (speed and accuracy)")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--hourglass", type=int, default=0, choices=[0, 1, 2],
                    help="C0: hourglass form, 1 stiffness (KF78), 2 viscous with kapa_hg 0.1 (0: the config's)")
    ap.add_argument("--mesh-only", type=int, default=-1,
                    help="1: host case without element tables, built on the device by eqd_gpu_init; 0: host "
                         "tables; -1: by size (C2 at its stated size)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    world, rank, local = dist_setup(args)
    if args.impl == "reference":
        line = bench_reference(args, world, rank)
    elif args.config == "C4":
        line = bench_ensemble(args, world, rank, local)
    else:
        from eqdyna_gb300 import build
        if not os.path.exists(build.GPU_LIB):
            build.build_all()
        line = bench_ours(args, world, rank, local)
    if line is not None:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
