"""Benchmark of the indirect INC par_loop on one GB300 (or N replicas).

Workload: P1 tetrahedral Laplacian operator action y += K_e x_e on the unit
cube, 128^3 hexes x 6 Kuhn tets = 12,582,912 cells, 2,146,689 vertices,
lexicographic vertex numbering, FP64 (the second benchmark configuration;
the first is the small CPU-runnable 2D case, used as a parity test).
A step is one op2.par_loop over all cells.

Prints one JSON line (rank 0).  ``--impl reference`` times the CPU
restatement of the reference's sequential backend instead (all host cores,
one private output per thread as MPI ranks would have, summed at the end).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "INC par_loop cells/s + % of HBM peak; adjoint/forward time ratio vs plain GPU"
N_CUBE = 128


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class _Nvml:
    """Read-only NVML queries through ctypes: SM clock, maximum SM clock and
    the clock-event (throttle) reason bits of the GPU behind CUDA ordinal
    ``ordinal`` (matched by PCI bus id, so CUDA_VISIBLE_DEVICES is honoured).
    Nothing is ever set."""

    SM = 1   # NVML_CLOCK_SM
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown",
               0x40: "hw_thermal_slowdown", 0x80: "hw_power_brake_slowdown"}

    def __init__(self, ordinal):
        import ctypes
        self.c = ctypes
        self.nv = ctypes.CDLL("libnvidia-ml.so.1")
        if self.nv.nvmlInit_v2() != 0:
            raise RuntimeError("nvmlInit failed")
        cu = ctypes.CDLL("libcuda.so.1")
        cu.cuInit(0)
        dev = ctypes.c_int()
        if cu.cuDeviceGet(ctypes.byref(dev), int(ordinal)) != 0:
            raise RuntimeError("cuDeviceGet failed")
        bus = ctypes.create_string_buffer(64)
        if cu.cuDeviceGetPCIBusId(bus, 64, dev) != 0:
            raise RuntimeError("cuDeviceGetPCIBusId failed")
        self.h = ctypes.c_void_p()
        if self.nv.nvmlDeviceGetHandleByPciBusId_v2(bus.value, ctypes.byref(self.h)) != 0:
            raise RuntimeError("no NVML handle for %s" % bus.value)
        self._reasons = getattr(self.nv, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            self.nv.nvmlDeviceGetCurrentClocksThrottleReasons

    def sm_mhz(self):
        v = self.c.c_uint()
        self.nv.nvmlDeviceGetClockInfo(self.h, self.SM, self.c.byref(v))
        return v.value

    def sm_max_mhz(self):
        v = self.c.c_uint()
        self.nv.nvmlDeviceGetMaxClockInfo(self.h, self.SM, self.c.byref(v))
        return v.value

    def reasons(self):
        v = self.c.c_ulonglong()
        self._reasons(self.h, self.c.byref(v))
        return [nm for bit, nm in self.REASONS.items() if v.value & bit]


class ClockSampler:
    """SM clocks and throttle reasons sampled DURING the timed region: an NVML
    poller thread (every 2 ms, first sample taken before the region starts);
    ``nvidia-smi -lms 200`` when NVML cannot be opened."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index, period_s=0.002):
        self.gpu = gpu_index
        self.period = period_s
        self.proc = None
        self.lines = []
        self.samples = []      # (sm_mhz, [reasons]) from NVML
        self.nvml = None
        self.smax = None

    def __enter__(self):
        try:
            self.nvml = _Nvml(self.gpu)
            self.smax = self.nvml.sm_max_mhz()
            self._stop = threading.Event()
            self.samples.append((self.nvml.sm_mhz(), self.nvml.reasons()))
            self._t = threading.Thread(target=self._poll, daemon=True)
            self._t.start()
            return self
        except Exception:
            self.nvml = None
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except Exception:
            self.proc = None
        return self

    def _poll(self):
        while not self._stop.wait(self.period):
            try:
                self.samples.append((self.nvml.sm_mhz(), self.nvml.reasons()))
            except Exception:
                return

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.nvml is not None:
            self._stop.set()
            self._t.join(timeout=5)
            try:
                self.samples.append((self.nvml.sm_mhz(), self.nvml.reasons()))
            except Exception:
                pass
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if self.nvml is not None and self.samples:
            reasons = sorted(set(r for _, rs in self.samples for r in rs))
            return {"sm_mhz": statistics.median(m for m, _ in self.samples),
                    "sm_max_mhz": self.smax, "reasons": reasons,
                    "samples": len(self.samples), "source": "nvml, 2 ms poll"}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "reasons": sorted(reasons), "samples": len(sm), "source": "nvidia-smi -lms 200"}


def max_over_ranks(value, device=None):
    """Max of a per-rank float over all ranks of the default process group
    (identity without one): the job time is the slowest replica's."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_rank, steps, max_ms, world):
    """Whole-job throughput of `world` replicas (weak scaling)."""
    return world * steps * units_per_rank / (max_ms * 1e-3)


def _dist():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def cpu_baseline(problem_np, threads=1, reps=3, max_cells=None):
    """Time the oracle's sequential wrapper (the reference's CPU backend
    restated in C, compiled with the reference's flags) on host cores.

    With threads > 1 each thread runs a contiguous cell range into its own
    output, as one MPI rank of the reference would; the ranks' halo exchange
    is not modelled, so only the parallel element loop is timed."""
    from oracle import op2 as O
    coords, cells, x0 = problem_np
    C = cells.shape[0] if max_cells is None else min(max_cells, cells.shape[0])
    V = coords.shape[0]
    verts = O.Set(V)
    cset = O.Set(cells.shape[0])
    c2v = O.Map(cset, verts, 4, cells)
    X = O.Dat(O.DataSet(verts, 3), coords)
    x = O.Dat(verts, x0)
    y = O.Dat(verts, np.zeros(V))
    from pyop2_gb300 import workloads
    k = O.Kernel(workloads.P1_3D_LAPLACE_ACTION, "p1_laplace_3d")
    loop = O.ParLoop(k, cset, y(O.INC, c2v), X(O.READ, c2v), x(O.READ, c2v), profile="timing")
    ys = [np.zeros(V) for _ in range(threads)]
    bounds = np.linspace(0, C, threads + 1).astype(np.int64)
    best = None
    for _ in range(reps):
        for yy in ys:
            yy[:] = 0
        t0 = time.perf_counter()
        if threads == 1:
            loop.compute(0, C, overrides={0: ys[0]})
        else:
            ths = [threading.Thread(target=loop.compute,
                                    args=(int(bounds[i]), int(bounds[i + 1])),
                                    kwargs={"overrides": {0: ys[i]}}) for i in range(threads)]
            for t in ths:
                t.start()
            for t in ths:
                t.join()
        dt = time.perf_counter() - t0
        best = dt if best is None else min(best, dt)
    return C / best, C, best


def _config(cells, vertices, permute):
    """The workload description, identical in both arms."""
    from pyop2_gb300 import workloads
    alg = workloads.bytes_c2a(cells, vertices)
    return {"workload": "p1_tet_laplace_action_128cube", "cells": cells, "vertices": vertices,
            "numbering": "random_permutation" if permute else "lexicographic",
            "l2": "working set %.0f MB > 129 MB L2, no flush" % (alg / 1e6)}


def run_reference(args):
    world, rank, local = _dist()
    if rank != 0:
        return 0
    from pyop2_gb300 import meshes
    coords, cells = meshes.unit_cube_tets(N_CUBE, permute=False, seed=0)
    x0 = np.random.default_rng(1).uniform(-1, 1, coords.shape[0])
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_baseline((coords, cells, x0), threads=threads, reps=1)
    times = []
    for _ in range(args.steps):
        rate, C, dt = cpu_baseline((coords, cells, x0), threads=threads, reps=1)
        times.append(dt)
    tot = sum(times)
    value = args.steps * cells.shape[0] / tot
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "cells/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * tot / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": _config(int(cells.shape[0]), int(coords.shape[0]), False),
        "cpu_baseline": {"value": value, "unit": "cells/s", "cores": threads, "kind": "port",
                         "sample": "full workload per step; oracle C wrapper built with the "
                                   "reference's flags, one thread per contiguous cell range "
                                   "with a private y (MPI-rank emulation, halo sum not timed)"},
        "e2e": {"value": value, "unit": "cells/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def _time_loop(loop, steps, warmup):
    """Mean device ms per compute() of a prebuilt ParLoop (CUDA events)."""
    import torch
    for _ in range(warmup):
        loop.compute()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        loop.compute()
    e1.record()
    e1.synchronize()
    return e0.elapsed_time(e1) / steps


def e2e_pipelined(op2, p, loop0, steps, barrier):
    """Device ms for `steps` end-to-end steps (H2D x, action, D2H y), with
    two buffer sets, an upload stream and a download stream, so that step k's
    compute overlaps the upload of step k+1 and the download of step k-1.
    Returns the max over ranks."""
    import torch
    V = p["verts"].size
    x_host = [torch.from_numpy(p["x"].data_ro.copy()).pin_memory() for _ in range(2)]
    y_host = [torch.empty(V, dtype=torch.float64).pin_memory() for _ in range(2)]
    xs = [p["x"], op2.Dat(p["verts"], p["x"].data_ro.copy())]
    ys = [p["y"], op2.Dat(p["verts"])]
    loops = [loop0, op2.ParLoop(p["kernel"], p["cells"], ys[1](op2.INC, p["c2v"]),
                                p["X"](op2.READ, p["c2v"]), xs[1](op2.READ, p["c2v"]))]
    for lp in loops:
        lp.compute()
    main = torch.cuda.current_stream()
    h2d, d2h = torch.cuda.Stream(), torch.cuda.Stream()
    up = [torch.cuda.Event() for _ in range(2)]
    done = [torch.cuda.Event() for _ in range(2)]
    down = [torch.cuda.Event() for _ in range(2)]

    def run(n):
        for k in range(n):
            b = k & 1
            with torch.cuda.stream(h2d):
                h2d.wait_event(done[b])          # step k-2 no longer reads x[b]
                xs[b].tensor.copy_(x_host[b], non_blocking=True)
                up[b].record(h2d)
            main.wait_event(up[b])
            main.wait_event(down[b])             # step k-2's y[b] has left the device
            xs[b].mark_device_modified()
            loops[b].compute()
            done[b].record(main)
            with torch.cuda.stream(d2h):
                d2h.wait_event(done[b])
                y_host[b].copy_(ys[b].tensor, non_blocking=True)
                down[b].record(d2h)
        main.wait_stream(h2d)
        main.wait_stream(d2h)
    for b in range(2):
        done[b].record(main)
        down[b].record(main)
    run(2)
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(main)
    run(steps)
    e1.record(main)
    barrier()
    return max_over_ranks(e0.elapsed_time(e1), device=torch.device("cuda"))


def e2e_serial(op2, p, steps, warmup, barrier):
    """Wall-clock ms for `steps` end-to-end steps through PyOP2's own data
    API, one after another: ``x.data[:] = host`` (the host array becomes the
    newer copy), ``y.zero()``, ``op2.par_loop(...)`` (uploads x, runs the
    action) and ``y.data_ro`` (waits, downloads y).  Nothing overlaps.
    Returns the max over ranks."""
    import torch
    x_host = p["x"].data_ro.copy()

    def step():
        p["x"].data[:] = x_host
        p["y"].zero()
        op2.par_loop(p["kernel"], p["cells"], p["y"](op2.INC, p["c2v"]),
                     p["X"](op2.READ, p["c2v"]), p["x"](op2.READ, p["c2v"]))
        return p["y"].data_ro
    for _ in range(warmup):
        step()
    barrier()
    t0 = time.perf_counter()
    for _ in range(steps):
        step()
    ms = 1e3 * (time.perf_counter() - t0)
    barrier()
    return max_over_ranks(ms, device=torch.device("cuda"))


def measure_strategies(op2, p, steps, warmup):
    """The benchmark action under each INC conflict strategy (hardware
    atomics, warp-aggregated atomics, greedy colouring, per-CTA shared-memory
    staging), for the given problem's numbering."""
    from pyop2_gb300.configuration import configuration
    out = {}
    old = configuration["scatter"]
    try:
        for sc in ("atomic", "warp", "colour", "shared", "staged"):
            configuration["scatter"] = sc
            lp = op2.ParLoop(p["kernel"], p["cells"], p["y"](op2.INC, p["c2v"]),
                             p["X"](op2.READ, p["c2v"]), p["x"](op2.READ, p["c2v"]))
            t0 = time.perf_counter()
            lp.compute()                    # builds the colouring plan when needed
            import torch
            torch.cuda.synchronize()
            setup = time.perf_counter() - t0
            out[sc] = {"ms": _time_loop(lp, steps, warmup), "first_call_s": setup}
            if sc == "colour":
                from pyop2_gb300.parloop import colour_plan
                plan = colour_plan(lp)
                out[sc]["colours"] = plan.ncolours if plan is not None else None
    finally:
        configuration["scatter"] = old
    return out


def measure_adjoint(op2, steps, warmup, n=64):
    """Forward residual, its adjoint (VJP) and the fused forward+adjoint on
    64^3 x 6 = 1,572,864 P1 tets (the differentiation configuration)."""
    from pyop2_gb300 import workloads as W
    p = W.build_nonlinear(op2, n=n, seed=0)
    V, C = p["verts"].size, p["cells"].size
    c2v, X = p["c2v"], p["X"]
    F = op2.Dat(p["verts"], np.zeros(V))
    lam = op2.Dat(p["verts"], p["lam"])
    u = op2.Dat(p["verts"], p["u"])
    k = op2.Dat(p["cells"], p["kappa"])
    du = op2.Dat(p["verts"], np.zeros(V))
    dk = op2.Dat(p["cells"], np.zeros(C))
    fwd = op2.ParLoop(op2.Kernel(W.NL_RESIDUAL, "nl_residual"), p["cells"], F(op2.INC, c2v),
                      X(op2.READ, c2v), u(op2.READ, c2v), k(op2.READ))
    bwd = op2.ParLoop(op2.Kernel(W.NL_RESIDUAL_VJP, "nl_residual_vjp"), p["cells"],
                      lam(op2.READ, c2v), X(op2.READ, c2v), u(op2.READ, c2v), k(op2.READ),
                      du(op2.INC, c2v), dk(op2.WRITE))
    fus = op2.ParLoop(op2.Kernel(W.NL_RESIDUAL_FUSED, "nl_residual_fused"), p["cells"],
                      F(op2.INC, c2v), lam(op2.READ, c2v), X(op2.READ, c2v), u(op2.READ, c2v),
                      k(op2.READ), du(op2.INC, c2v), dk(op2.WRITE))
    tf = _time_loop(fwd, steps, warmup)
    tb = _time_loop(bwd, steps, warmup)
    tu = _time_loop(fus, steps, warmup)
    out = {"workload": "nonlinear_residual_p1_tet_64cube", "cells": C, "vertices": V,
           "forward_ms": tf, "adjoint_ms": tb, "fused_forward_adjoint_ms": tu,
           "ratio_forward_plus_adjoint_over_forward": (tf + tb) / tf,
           "ratio_fused_over_forward": tu / tf, "launches": 3 * (steps + warmup)}
    out["autograd"] = measure_adjoint_autograd(op2, p, steps, warmup)
    return out


def measure_adjoint_autograd(op2, p, steps, warmup):
    """The adjoint on the path a user takes: AdjointParLoop behind
    torch.autograd.Function.  Forward = F = loop(u, kappa) with u and kappa
    requiring gradients; forward + backward = the same followed by
    F.backward(lambda), which runs the VJP loop and fills u.grad and
    kappa.grad.  Timed with CUDA events on the launch stream and on the wall
    clock (host overhead included), per step."""
    import torch
    from pyop2_gb300 import workloads as W
    from pyop2_gb300.adjoint import AdjointParLoop
    loop = AdjointParLoop(
        p["cells"], op2.Kernel(W.NL_RESIDUAL, "nl_residual"),
        op2.Kernel(W.NL_RESIDUAL_VJP, "nl_residual_vjp"),
        output=(p["verts"] ** 1, p["c2v"]),
        inputs=[(p["verts"] ** 1, p["c2v"]), (p["cells"] ** 1, None)],
        constants=[(p["X"], p["c2v"])])
    dev = torch.device("cuda")
    u = torch.tensor(p["u"], device=dev, requires_grad=True)
    k = torch.tensor(p["kappa"], device=dev, requires_grad=True)
    lam = torch.tensor(p["lam"], device=dev)

    def fwd():
        return loop(u, k)

    def fwd_bwd():
        u.grad = None
        k.grad = None
        loop(u, k).backward(lam)

    res = {}
    for name, fn in (("forward", fwd), ("forward_backward", fwd_bwd)):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0 = time.perf_counter()
        e0.record()
        for _ in range(steps):
            fn()
        e1.record()
        e1.synchronize()
        res[name + "_ms"] = e0.elapsed_time(e1) / steps
        res[name + "_wall_ms"] = 1e3 * (time.perf_counter() - t0) / steps
    res["ratio_forward_backward_over_forward"] = res["forward_backward_ms"] / res["forward_ms"]
    res["ratio_wall"] = res["forward_backward_wall_ms"] / res["forward_wall_ms"]
    return res


def measure_batch(op2, steps, warmup, nmeshes=256):
    """256 P2 meshes with log-uniform cell counts in [1e3, 1e6]: per-mesh
    par_loop launches against one persistent launch replayed from a CUDA graph
    (chunk and CTA size picked by the batch autotuner)."""
    import torch
    from pyop2_gb300 import meshes
    from pyop2_gb300 import workloads as W
    from pyop2_gb300.batch import autotune_batch
    sizes = meshes.batch_sizes(nmeshes, seed=0)
    probs = W.build_p2_batch(op2, sizes, seed=0)
    loops = [op2.ParLoop(p["kernel"], p["cells"], *p["args"]) for p in probs]
    ncells = sum(lp.iterset.size for lp in loops)

    def plain():
        for lp in loops:
            lp.compute()

    def plain_api():
        for pr in probs:
            op2.par_loop(pr["kernel"], pr["cells"], *pr["args"])
    for _ in range(warmup):
        plain_api()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        plain_api()
    e1.record()
    e1.synchronize()
    t_api = e0.elapsed_time(e1) / steps
    for _ in range(warmup):
        plain()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        plain()
    e1.record()
    e1.synchronize()
    t_plain = e0.elapsed_time(e1) / steps
    batch, tuned = autotune_batch(loops)
    for _ in range(warmup):
        batch.replay()
    torch.cuda.synchronize()
    e0.record()
    for _ in range(steps):
        batch.replay()
    e1.record()
    e1.synchronize()
    t_batch = e0.elapsed_time(e1) / steps
    return {"workload": "p2_mass_laplace_256_meshes", "meshes": nmeshes, "cells": ncells,
            "plain_par_loop_ms": t_api, "plain_prebuilt_ms": t_plain,
            "batched_graph_ms": t_batch, "speedup_vs_par_loop": t_api / t_batch,
            "speedup_vs_prebuilt": t_plain / t_batch,
            "batched_cells_per_s": ncells / (t_batch * 1e-3), "tuned": tuned,
            "flops_per_cell": W.P2_FLOPS}


def _time_sparsity_build(dsets, pairs, reps=3):
    """Best-of-reps wall time (ms) of a Sparsity build, bypassing the object
    cache; returns (ms, sparsity)."""
    import torch
    from pyop2_gb300.types.mat import Sparsity
    best, sp = None, None
    for _ in range(reps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sp = Sparsity.__new__(Sparsity, dsets, pairs)
        sp._initialized = False           # force a rebuild (bypass the object cache)
        sp.__init__(dsets, pairs)
        torch.cuda.synchronize()
        dt = 1e3 * (time.perf_counter() - t0)
        best = dt if best is None else min(best, dt)
    return best, sp


def _time_spmv(op2, A, x, steps, warmup):
    """Mean time of y = A x (ms, CUDA events over `steps` back-to-back
    products) and the bandwidth it implies over the compulsory bytes: block
    values, column indices, row pointers, x and y once each."""
    import torch
    y = op2.Dat(A.sparsity.dsets[0])
    for _ in range(warmup):
        A.mult(x, y)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        A.mult(x, y)
    e1.record()
    e1.synchronize()
    ms = e0.elapsed_time(e1) / steps
    sp = A.sparsity
    rdim, cdim = A.dims[0][0]
    nrows, ncols = sp.dsets[0].size, sp.dsets[1].size
    nbytes = (sp.nblocks * (rdim * cdim * 8 + 4) + (nrows + 1) * 8
              + ncols * cdim * 8 + nrows * rdim * 8)
    return ms, nbytes / (ms * 1e-3) / 1e9


def measure_sparsity_assembly(op2, p, steps, warmup):
    """Configuration 2b on the benchmark mesh: GPU sparsity build (block CSR,
    bit-exact pattern), CSR assembly of the 4x4 element matrices and SpMV."""
    from pyop2_gb300 import workloads as W
    t_sp, sp = _time_sparsity_build((p["verts"] ** 1, p["verts"] ** 1),
                                    [(p["c2v"], p["c2v"], None)])
    A = op2.Mat(sp)
    asm = op2.ParLoop(op2.Kernel(W.P1_3D_LAPLACE_MATRIX, "p1_laplace_3d_mat"), p["cells"],
                      A(op2.INC, (p["c2v"], p["c2v"])), p["X"](op2.READ, p["c2v"]))
    t_asm = _time_loop(asm, steps, warmup)
    t_spmv, gbs = _time_spmv(op2, A, p["x"], max(steps, 5), max(warmup, 3))
    C = p["cells"].size
    nnz = sp.nblocks
    out = {"workload": "p1_tet_laplace_128cube_csr", "nnz": nnz, "rows": p["verts"].size,
           "sparsity_build_ms": t_sp, "assembly_ms": t_asm,
           "assembly_cells_per_s": C / (t_asm * 1e-3), "spmv_ms": t_spmv, "spmv_gbs": gbs}
    del A, sp
    return out


def measure_prisms(op2, steps, warmup, n=256):
    """Configuration 5: 256^2 x 64 extruded prisms, P1 elasticity with 8 RHS:
    matrix-free action, its adjoint (displacement and Lame fields), both in
    one CUDA graph; BAIJ 3x3 sparsity and assembly."""
    import torch
    from pyop2_gb300 import workloads as W
    p = W.build_prisms(op2, n=n, layers=65, seed=0)
    NR = p["nrhs"]
    nodes, cells, c2n, c2c = p["nodes"], p["cells"], p["c2n"], p["c2c"]
    ds = op2.DataSet(nodes, (NR, 3))
    u = op2.Dat(ds, p["u"])
    w = op2.Dat(ds, p["w"])
    y = op2.Dat(ds)
    du = op2.Dat(ds)
    dL = op2.Dat(p["prisms"] ** 2)
    act = op2.ParLoop(op2.Kernel(W.PRISM_ELASTICITY_ACTION, "prism_elasticity"), cells,
                      y(op2.INC, c2n), p["X"](op2.READ, c2n), u(op2.READ, c2n),
                      p["L"](op2.READ, c2c))
    adj = op2.ParLoop(op2.Kernel(W.PRISM_ELASTICITY_VJP, "prism_elasticity_vjp"), cells,
                      w(op2.READ, c2n), p["X"](op2.READ, c2n), u(op2.READ, c2n),
                      p["L"](op2.READ, c2c), du(op2.INC, c2n), dL(op2.WRITE, c2c))
    t_act = _time_loop(act, steps, warmup)
    t_adj = _time_loop(adj, steps, warmup)
    # both in one CUDA graph
    from pyop2_gb300.graph import LoopGraph
    g = LoopGraph([act, adj])
    for _ in range(warmup):
        g.replay()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        g.replay()
    e1.record()
    e1.synchronize()
    t_graph = e0.elapsed_time(e1) / steps
    C = p["ncell"]
    out = {"workload": "prism_elasticity_%dx%dx64_8rhs" % (n, n), "cells": C, "nodes": p["nnodes"],
           "rhs": NR, "action_ms": t_act, "adjoint_ms": t_adj,
           "graph_action_adjoint_ms": t_graph,
           "action_cell_rhs_per_s": C * NR / (t_act * 1e-3),
           "adjoint_over_action": t_adj / t_act}
    out.update(measure_prism_assembly(op2, p))
    return out


def measure_prism_assembly(op2, p=None, n=256):
    """BAIJ 3x3 sparsity, assembly of the 18x18 prism elasticity matrices and
    SpMV on the extruded prism mesh (built here unless given)."""
    from pyop2_gb300 import workloads as W
    if p is None:
        p = W.build_prisms(op2, n=n, layers=65, seed=0)
    nodes, cells, c2n, c2c = p["nodes"], p["cells"], p["c2n"], p["c2c"]
    t_sp, sp = _time_sparsity_build((nodes ** 3, nodes ** 3), [(c2n, c2n, None)])
    A = op2.Mat(sp)
    asm = op2.ParLoop(op2.Kernel(W.PRISM_ELASTICITY_MATRIX, "prism_elasticity_mat"), cells,
                      A(op2.INC, (c2n, c2n)), p["X"](op2.READ, c2n), p["L"](op2.READ, c2c))
    t_asm = _time_loop(asm, 2, 1)
    xs = op2.Dat(nodes ** 3, np.random.default_rng(0).uniform(-1, 1, (p["nnodes"], 3)))
    t_spmv, gbs = _time_spmv(op2, A, xs, 5, 3)
    out = {"baij_blocks": sp.nblocks, "sparsity_build_ms": t_sp,
           "assembly_ms": t_asm, "assembly_cells_per_s": p["ncell"] / (t_asm * 1e-3),
           "values_gb": sp.nblocks * 9 * 8 / 1e9, "spmv_ms": t_spmv, "spmv_gbs": gbs}
    del A, sp
    return out


def measure_small(op2, calls=500, with_cpu=True):
    """The small 2D configuration (64^2 x 2 = 8,192 triangles, P1 action plus
    an area Global): device-side it is a few microseconds, so this reports
    the cost of a whole op2.par_loop call (validation, launch, bookkeeping)
    and of a reused ParLoop, next to the oracle's sequential C wrapper on one
    host core for the same loop."""
    import torch
    from pyop2_gb300 import workloads as W
    p = W.build_p1_2d(op2)
    for _ in range(20):
        p["run"]()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(calls):
        p["run"]()
    torch.cuda.synchronize()
    per_call = (time.perf_counter() - t0) / calls
    pl = op2.ParLoop(p["kernel"], p["cells"], p["y"](op2.INC, p["c2v"]),
                     p["X"](op2.READ, p["c2v"]), p["x"](op2.READ, p["c2v"]),
                     p["area"](op2.INC))
    pl.compute()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(calls):
        pl.compute()
    torch.cuda.synchronize()
    per_compute = (time.perf_counter() - t0) / calls
    # the same loop recorded into a CUDA graph, once and as 10 consecutive
    # steps (the form a time-stepping loop over a small mesh would take)
    from pyop2_gb300.graph import LoopGraph
    graph_us = {}
    for nrep in (1, 10):
        g = LoopGraph([pl] * nrep)
        g.replay()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(calls // nrep):
            g.replay()
        torch.cuda.synchronize()
        graph_us[nrep] = (time.perf_counter() - t0) / (calls // nrep * nrep) * 1e6
    C = p["cells"].size
    out = {"workload": "p1_tri_laplace_action_64sq", "cells": C,
           "par_loop_us_per_call": per_call * 1e6, "parloop_compute_us_per_call": per_compute * 1e6,
           "graph_replay_us_per_loop": graph_us[1],
           "graph_of_10_steps_us_per_loop": graph_us[10],
           "par_loop_cells_per_s": C / per_call}
    if with_cpu:
        from oracle import op2 as O
        o = W.build_p1_2d(O)
        loop = O.ParLoop(o["kernel"], o["cells"], o["y"](O.INC, o["c2v"]),
                         o["X"](O.READ, o["c2v"]), o["x"](O.READ, o["c2v"]),
                         o["area"](O.INC), profile="timing")
        best = None
        for _ in range(20):
            t0 = time.perf_counter()
            loop.compute()
            dt = time.perf_counter() - t0
            best = dt if best is None else min(best, dt)
        out["cpu_1core_us_per_loop"] = best * 1e6
        out["cpu_1core_cells_per_s"] = C / best
    return out


def cpu_sections(reps=2):
    """The secondary configurations on ONE host core, through the oracle (the
    reference's CPU path restated in C and compiled with the reference's
    flags), each on a bounded sample of its workload: rates in the units the
    GPU sections report, to sit beside them."""
    from oracle import op2 as O
    from pyop2_gb300 import meshes
    from pyop2_gb300 import workloads as W

    def best(fn):
        b = None
        for _ in range(reps):
            t0 = time.perf_counter()
            fn()
            dt = time.perf_counter() - t0
            b = dt if b is None else min(b, dt)
        return b

    def loop(*a, **kw):
        return O.ParLoop(*a, profile="timing", **kw)

    out = {}
    # configuration 2b: sparsity build and CSR assembly, 48^3 x 6 tets
    p = W.build_p1_3d(O, n=48, seed=0)
    C = p["cells"].size
    built = []
    t_sp = best(lambda: built.append(O.Sparsity((p["verts"] ** 1, p["verts"] ** 1),
                                                [(p["c2v"], p["c2v"], None)])))
    sp = built[-1]
    A = O.Mat(sp)
    asm = loop(O.Kernel(W.P1_3D_LAPLACE_MATRIX, "p1_laplace_3d_mat"), p["cells"],
               A(O.INC, (p["c2v"], p["c2v"])), p["X"](O.READ, p["c2v"]))
    t_asm = best(asm.compute)
    out["sparsity_assembly"] = {"sample": "48^3 x 6 = %d tets, %d nonzeros" % (C, len(sp.colidx)),
                                "sparsity_nnz_per_s": len(sp.colidx) / t_sp,
                                "assembly_cells_per_s": C / t_asm}
    # configuration 4: residual and its VJP, 32^3 x 6 tets
    q = W.build_nonlinear(O, n=32, seed=0)
    V, C = q["verts"].total_size, q["cells"].size
    c2v, X = q["c2v"], q["X"]
    F, du = O.Dat(q["verts"], np.zeros(V)), O.Dat(q["verts"], np.zeros(V))
    lam, u = O.Dat(q["verts"], q["lam"]), O.Dat(q["verts"], q["u"])
    k, dk = O.Dat(q["cells"], q["kappa"]), O.Dat(q["cells"], np.zeros(C))
    fwd = loop(O.Kernel(W.NL_RESIDUAL, "nl_residual"), q["cells"], F(O.INC, c2v),
               X(O.READ, c2v), u(O.READ, c2v), k(O.READ))
    bwd = loop(O.Kernel(W.NL_RESIDUAL_VJP, "nl_residual_vjp"), q["cells"], lam(O.READ, c2v),
               X(O.READ, c2v), u(O.READ, c2v), k(O.READ), du(O.INC, c2v), dk(O.WRITE))
    out["adjoint"] = {"sample": "32^3 x 6 = %d tets" % C,
                      "forward_cells_per_s": C / best(fwd.compute),
                      "adjoint_cells_per_s": C / best(bwd.compute)}
    # configuration 3: the first 24 meshes of the batch, one loop each
    sizes = meshes.batch_sizes(256, seed=0)[:24]
    probs = W.build_p2_batch(O, sizes, seed=0)
    loops = [loop(b["kernel"], b["cells"], *b["args"]) for b in probs]
    ncells = sum(b["cells"].size for b in probs)
    out["batch"] = {"sample": "the first 24 of the 256 meshes, %d cells" % ncells,
                    "cells_per_s": ncells / best(lambda: [lp.compute() for lp in loops])}
    # configuration 5: prism action with 8 RHS, 32^2 x 2 x 64 prisms
    r = W.build_prisms(O, n=32, layers=65, seed=0)
    ds = O.DataSet(r["nodes"], (r["nrhs"], 3))
    ur, yr = O.Dat(ds, r["u"]), O.Dat(ds)
    act = loop(O.Kernel(W.PRISM_ELASTICITY_ACTION, "prism_elasticity"), r["cells"],
               yr(O.INC, r["c2n"]), r["X"](O.READ, r["c2n"]), ur(O.READ, r["c2n"]),
               r["L"](O.READ, r["c2c"]))
    out["prisms"] = {"sample": "32^2 x 2 x 64 = %d prisms x %d RHS" % (r["ncell"], r["nrhs"]),
                     "action_cell_rhs_per_s": r["ncell"] * r["nrhs"] / best(act.compute)}
    return out


GATHER_COPY = ("static void gc(double *o, const double *x) "
               "{ o[0] = x[0]; o[1] = x[1]; o[2] = x[2]; o[3] = x[3]; }")


def measure_data_path(op2, p, steps, warmup):
    """Loops with little or no arithmetic on the benchmark mesh, to show the
    wrapper's memory path against HBM: a direct copy, a gather through the
    map that sums the four values (three FP64 adds per cell) and one that
    copies them out, an INC scatter through the map.  Bytes are compulsory
    ones (map read once, per-cell Dats once, vertex Dats once; INC targets
    read and written)."""
    import numpy as np
    import torch
    from pyop2_gb300.parloop import LegacyParloop
    cells, c2v, x, y = p["cells"], p["c2v"], p["x"], p["y"]
    C, V = cells.size, p["verts"].size
    w = op2.Dat(cells, np.random.default_rng(3).uniform(0, 1, C))
    out = op2.Dat(cells, np.zeros(C))
    K = op2.Kernel
    loops = {
        "direct_copy": (LegacyParloop(K("static void cp(double *o, const double *w) { o[0] = w[0]; }",
                                        "cp"), cells, out(op2.WRITE), w(op2.READ)), 16 * C),
        "gather": (LegacyParloop(K("static void ga(double *o, const double *x) "
                                   "{ o[0] = x[0] + x[1] + x[2] + x[3]; }", "ga"),
                                 cells, out(op2.WRITE), x(op2.READ, c2v)), 24 * C + 8 * V),
        "scatter_inc": (LegacyParloop(K("static void sc(double *y, const double *w) "
                                        "{ for (int i = 0; i < 4; ++i) y[i] += w[0]; }", "sc"),
                                      cells, y(op2.INC, c2v), w(op2.READ)), 24 * C + 16 * V),
    }
    # the gather alone: the four vertex values copied out, no FP64 arithmetic
    out4 = op2.Dat(cells ** 4, np.zeros((C, 4)))
    loops["gather_copy"] = (LegacyParloop(K(GATHER_COPY, "gc"), cells, out4(op2.WRITE),
                                          x(op2.READ, c2v)), 48 * C + 8 * V)
    from pyop2_gb300 import _lib
    pl = LegacyParloop(K("static void ga(double *o, const double *x) "
                         "{ o[0] = x[0] + x[1] + x[2] + x[3]; }", "ga"),
                       cells, out(op2.WRITE), x(op2.READ, c2v))
    pl.build(_lib.SCATTER_STAGED)
    loops["gather_staged"] = (pl, 24 * C + 8 * V)
    for sc, nm in ((_lib.SCATTER_WARP, "scatter_inc_warp"), (_lib.SCATTER_SHARED, "scatter_inc_shared"),
                   (_lib.SCATTER_STAGED, "scatter_inc_staged")):
        pl = LegacyParloop(K("static void sc(double *y, const double *w) "
                             "{ for (int i = 0; i < 4; ++i) y[i] += w[0]; }", "sc"),
                           cells, y(op2.INC, c2v), w(op2.READ))
        pl.build(sc)
        loops[nm] = (pl, 24 * C + 16 * V)
    # contention extreme: every cell INCs one of 16 targets
    hot_set = op2.Set(16)
    hot = op2.Map(cells, hot_set, 1, (np.arange(C) % 16).astype(np.int32))
    yh = op2.Dat(hot_set, np.zeros(16))
    for sc, nm in ((_lib.SCATTER_ATOMIC, "hot16_atomic"), (_lib.SCATTER_WARP, "hot16_warp"),
                   (_lib.SCATTER_SHARED, "hot16_shared")):
        pl = LegacyParloop(K("static void hs(double *y, const double *w) { y[0] += w[0]; }",
                             "hs"), cells, yh(op2.INC, hot), w(op2.READ))
        pl.build(sc)
        loops[nm] = (pl, 12 * C)
    peak, _ = _peaks()
    st = torch.cuda.current_stream()
    res = {}
    for name, (pl, alg) in loops.items():
        for _ in range(warmup):
            pl.compute()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(steps)]
        torch.cuda.synchronize()
        for a, b in ev:
            a.record(st)
            pl.compute()
            b.record(st)
        torch.cuda.synchronize()
        ms = statistics.median(a.elapsed_time(b) for a, b in ev)
        res[name] = {"ms": ms, "alg_bytes": alg, "gbs": alg / ms / 1e6,
                     "frac_hbm": alg / ms / 1e6 / peak}
    y.zero()
    return res


def _profile_number(name, key):
    """A number recorded in a profiles/ summary as ``key: value``."""
    import re
    path = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(path):
        return None
    with open(path) as f:
        m = re.search(key + r":\s*([0-9.]+)", f.read())
    return float(m.group(1)) if m else None


def run_ours(args):
    import torch
    world, rank, local = _dist()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from pyop2_gb300.csrc import build as _b
    _b.build()
    from pyop2_gb300 import _lib, device, op2, workloads
    from pyop2_gb300.configuration import configuration
    configuration["device"] = local
    if args.scatter:
        configuration["scatter"] = args.scatter
    device.require()
    dev = device.device()

    p = workloads.build_p1_3d(op2, n=N_CUBE, permute=args.permute, seed=0)
    C = p["cells"].size
    V = p["verts"].size
    loop = op2.ParLoop(p["kernel"], p["cells"], p["y"](op2.INC, p["c2v"]),
                       p["X"](op2.READ, p["c2v"]), p["x"](op2.READ, p["c2v"]))
    loop.compute()                         # compile + upload
    torch.cuda.synchronize()
    st = torch.cuda.current_stream()

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        loop.compute()
    barrier()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    with ClockSampler(local) as clk:
        barrier()
        t0 = time.perf_counter()
        for e0, e1 in ev:
            e0.record(st)
            loop.compute()
            e1.record(st)
        barrier()
        wall = time.perf_counter() - t0
    kern_ms = [a.elapsed_time(b) for a, b in ev]
    total_ms = max_over_ranks(sum(kern_ms), device=dev)
    value = job_rate(C, args.steps, total_ms, world)

    # End to end through the public API with host buffers: every step copies
    # its x in from pinned host memory, runs the par_loop and copies its y
    # back.  Two buffer sets and a copy stream overlap step k's compute with
    # the copies of steps k-1 and k+1, as a user streaming inputs would.
    e2e_ms = e2e_pipelined(op2, p, loop, args.steps, barrier)
    e2e = job_rate(C, args.steps, e2e_ms, world)
    # ... and one step after another through the PyOP2 data API
    e2e_serial_ms = e2e_serial(op2, p, args.steps, args.warmup, barrier)

    # FP64 ceiling: measured DFMA throughput of this GPU, with the SM clock
    # sampled while the probe runs
    import ctypes
    fl = ctypes.c_double()
    with ClockSampler(local) as pclk:
        _lib.call("op2g_probe_fp64_peak", ctypes.byref(fl), device.stream_handle())
    fp64_peak = fl.value / 1e12
    probe_clocks = pclk.summary()

    if rank != 0:
        return 0
    peak, peak_kind = _peaks()
    per_launch_ms = total_ms / args.steps
    alg_bytes = workloads.bytes_c2a(C, V)
    achieved = alg_bytes / (per_launch_ms * 1e-3) / 1e9
    flops = workloads.P1_3D_FLOPS * C
    fp64_achieved = flops / (per_launch_ms * 1e-3) / 1e12
    traffic = None
    tf = os.path.join(ROOT, "profiles", "op2g_wrap_p1_laplace_3d_128cube.md")
    if os.path.exists(tf) and not args.permute:
        import re
        with open(tf) as f:
            m = re.search(r"dram_bytes_per_launch:\s*(\d+)", f.read())
        traffic = int(m.group(1)) if m else None
    # FP64 issue roofline: the kernel's FP64 instructions per cell (ncu
    # instruction mix, recorded in the profile) at the sampled clock
    clocks = clk.summary()
    sms = device.sm_count()
    # the nominal FP64 rate at a clock: 2 FMA lanes per SM per clock (304 per
    # clock on 152 SMs), 2 flop each
    nominal_at = (lambda mhz: sms * 2 * 2 * mhz * 1e6 / 1e12) if sms else None
    probe_mhz = probe_clocks.get("sm_mhz")
    kern_mhz = clocks.get("sm_mhz")
    fp64_ipc = _profile_number("op2g_wrap_p1_laplace_3d_128cube.md", "fp64_instructions_per_cell")
    issue_frac = None
    if fp64_ipc and clocks.get("sm_mhz"):
        issue_frac = fp64_ipc * C / (per_launch_ms * 1e-3) / (304 * clocks["sm_mhz"] * 1e6)
    strategies = None
    if not args.skip_extras:
        strategies = {"lexicographic": measure_strategies(op2, p, 5, 2)}
        pr = workloads.build_p1_3d(op2, n=N_CUBE, permute=True, seed=0)
        strategies["random_permutation"] = measure_strategies(op2, pr, 5, 2)
        del pr
    data_path = measure_data_path(op2, p, 10, 3) if not args.skip_extras else None
    small = measure_small(op2, with_cpu=not args.no_cpu_baseline) if not args.skip_extras else None
    sparsity = measure_sparsity_assembly(op2, p, 5, 3) if not args.skip_extras else None
    adjoint = measure_adjoint(op2, max(args.steps, 5), 3) if not args.skip_extras else None
    batch = measure_batch(op2, 5, 3) if not args.skip_extras else None
    prisms = measure_prisms(op2, 5, 2) if not args.skip_extras else None
    if not args.skip_extras and not args.no_cpu_baseline and world == 1:
        # the same configurations on one host core, beside each GPU section
        # (a failure there is reported in the line, not fatal to it)
        try:
            cs = cpu_sections()
        except Exception as e:
            cs = {k: {"error": repr(e)[:200]} for k in
                  ("sparsity_assembly", "adjoint", "batch", "prisms")}
        for sec, key in ((sparsity, "sparsity_assembly"), (adjoint, "adjoint"),
                         (batch, "batch"), (prisms, "prisms")):
            sec["cpu_1core"] = cs[key]
    cpu = None
    if not args.no_cpu_baseline and world == 1 and rank == 0:
        coords = p["coords"]
        cells = p["cellmap"]
        x0 = p["x"].data_ro.copy()
        rate, ncells, dt = cpu_baseline((coords, cells, x0), threads=1, reps=2)
        cpu = {"value": rate, "unit": "cells/s", "cores": 1, "kind": "port",
               "sample": "all %d cells, best of 2 passes, 1 core, oracle C wrapper built with "
                         "the reference's -O3 -march=native -ffast-math" % ncells}
    line = {
        "metric": METRIC, "value": value, "unit": "cells/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": per_launch_ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": _config(C, V, args.permute),
        "scatter": configuration["scatter"],
        "parallelism": "replicas" if world > 1 else "1gpu",
        "pct_hbm_peak": 100.0 * achieved / peak,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "peak_source": peak_kind,
                     "traffic_source": "dram__bytes_read.sum + dram__bytes_write.sum of one ncu "
                                       "capture of this kernel on this workload, recorded in "
                                       "profiles/op2g_wrap_p1_laplace_3d_128cube.md",
                     "alg_bytes_per_launch": alg_bytes},
        "roofline_fp64": {"achieved": fp64_achieved, "peak": fp64_peak, "unit": "TFLOP/s",
                          "frac": fp64_achieved / fp64_peak, "flops_per_cell": workloads.P1_3D_FLOPS,
                          "peak_source": "measured live (DFMA probe: 16 independent FMA chains "
                                         "per thread, 8 x 256 threads per SM, best of 5)",
                          "probe_clocks": probe_clocks,
                          "probe_fma_per_sm_per_clk": (fl.value / 2 / sms / (probe_mhz * 1e6)
                                                       if probe_mhz and sms else None),
                          "nominal_peak_at_probe_clock": nominal_at(probe_mhz) if probe_mhz else None,
                          "probe_frac_of_nominal_at_its_clock": (fp64_peak / nominal_at(probe_mhz)
                                                                 if probe_mhz else None),
                          "nominal_peak_at_kernel_clock": nominal_at(kern_mhz) if kern_mhz else None,
                          "frac_of_nominal_at_kernel_clock": (fp64_achieved / nominal_at(kern_mhz)
                                                              if kern_mhz else None),
                          "nominal_source": "2 FP64 FMA lanes per SM per clock (ncu peak of "
                                            "sm__sass_thread_inst_executed_op_dfma: 304 per "
                                            "clock on 152 SMs) x 2 flop x the sampled SM clock",
                          "fp64_pipe_active_ncu": 0.887,
                          "fp64_instr_per_cell_ncu": fp64_ipc,
                          "fp64_instr_source": "profiles/op2g_wrap_p1_laplace_3d_128cube.md "
                                               "(ncu instruction mix of this kernel)",
                          "issue_frac": issue_frac,
                          "issue_peak_source": "304 FP64 instructions/clk x median SM clock "
                                               "sampled in the timed region"},
        "cpu_baseline": cpu,
        "e2e": {"value": e2e, "unit": "cells/s", "h2d_bytes_per_step": 8 * V,
                "d2h_bytes_per_step": 8 * V,
                "mode": "streaming throughput: x in from pinned host memory and y back every "
                        "step, two buffer sets, copies on their own streams overlapped with "
                        "the previous and next steps' compute (CUDA events on the compute "
                        "stream)"},
        "e2e_serial": {"value": job_rate(C, args.steps, e2e_serial_ms, world), "unit": "cells/s",
                       "ms_per_step": e2e_serial_ms / args.steps,
                       "h2d_bytes_per_step": 8 * V, "d2h_bytes_per_step": 8 * V,
                       "mode": "one step after another through the PyOP2 data API: "
                               "x.data[:] = host; y.zero(); op2.par_loop(...); y.data_ro "
                               "(pageable numpy arrays, wall clock)"},
        "strategies": strategies,
        "sparsity_assembly": sparsity,
        "adjoint": adjoint,
        "batch": batch,
        "prisms": prisms,
        "data_path": data_path,
        "small_2d": small,
        "gpu_launches": args.steps,
        "clocks": clocks,
        "wall_s_timed": wall,
    }
    print(json.dumps(line), flush=True)
    return 0


def scatter_pair(op2, n=N_CUBE, launches=2):
    """The INC scatter loop y[map(e, i)] += w_e on the n^3 x 6 tet mesh,
    `launches` times with hardware atomics, then `launches` times on the
    staging plan (plan built before the first staged launch).  For one-kernel
    profiler captures of the two forms."""
    import torch
    from pyop2_gb300 import _lib
    from pyop2_gb300 import workloads as W
    from pyop2_gb300.parloop import LegacyParloop
    p = W.build_p1_3d(op2, n=n, seed=0)
    cells, c2v, y = p["cells"], p["c2v"], p["y"]
    w = op2.Dat(cells, np.random.default_rng(3).uniform(0, 1, cells.size))
    K = op2.Kernel("static void sc(double *y, const double *w) "
                   "{ for (int i = 0; i < 4; ++i) y[i] += w[0]; }", "sc")
    la = LegacyParloop(K, cells, y(op2.INC, c2v), w(op2.READ))
    la.build(_lib.SCATTER_ATOMIC)
    ls = LegacyParloop(K, cells, y(op2.INC, c2v), w(op2.READ))
    ls.build(_lib.SCATTER_STAGED)
    ls.launch_desc()
    torch.cuda.synchronize()
    for lp in [la] * launches + [ls] * launches:
        lp.compute()
    torch.cuda.synchronize()
    return {"cells": cells.size, "launches": 2 * launches,
            "y_checksum": float(y.data_ro.sum())}


def gather_pair(op2, n=N_CUBE, permute=False, launches=2):
    """The gather loops on the n^3 x 6 tet mesh: `launches` times the sum
    o_e = x[map(e, 0)] + ... + x[map(e, 3)] (three FP64 adds per cell), then
    `launches` times the copy o_e[i] = x[map(e, i)] (no arithmetic).  For
    one-kernel profiler captures of the two forms."""
    import torch
    from pyop2_gb300 import workloads as W
    from pyop2_gb300.parloop import LegacyParloop
    p = W.build_p1_3d(op2, n=n, permute=permute, seed=0)
    cells, c2v, x = p["cells"], p["c2v"], p["x"]
    out = op2.Dat(cells, np.zeros(cells.size))
    out4 = op2.Dat(cells ** 4, np.zeros((cells.size, 4)))
    ls = LegacyParloop(op2.Kernel("static void ga(double *o, const double *x) "
                                  "{ o[0] = x[0] + x[1] + x[2] + x[3]; }", "ga"),
                       cells, out(op2.WRITE), x(op2.READ, c2v))
    lc = LegacyParloop(op2.Kernel(GATHER_COPY, "gc"), cells, out4(op2.WRITE), x(op2.READ, c2v))
    ls.launch_desc()
    lc.launch_desc()
    torch.cuda.synchronize()
    for lp in [ls] * launches + [lc] * launches:
        lp.compute()
    torch.cuda.synchronize()
    return {"cells": cells.size, "launches": 2 * launches,
            "checksum": float(out.data_ro.sum() + out4.data_ro.sum())}


def run_only(args):
    """One secondary measurement on its own (used for ncu captures); prints
    its JSON object."""
    from pyop2_gb300.csrc import build as _b
    _b.build()
    from pyop2_gb300 import device, op2, workloads
    device.require()
    if args.only == "sparsity":
        p = workloads.build_p1_3d(op2, n=args.size or N_CUBE, seed=0)
        out = measure_sparsity_assembly(op2, p, args.steps, args.warmup)
    elif args.only == "adjoint":
        out = measure_adjoint(op2, args.steps, args.warmup, n=args.size or 64)
    elif args.only == "batch":
        out = measure_batch(op2, args.steps, args.warmup)
    elif args.only == "small":
        out = measure_small(op2, with_cpu=False)
    elif args.only == "prism_assembly":
        out = measure_prism_assembly(op2, n=args.size or 256)
    elif args.only == "scatter":
        out = scatter_pair(op2, n=args.size or N_CUBE)
    elif args.only == "gather":
        out = gather_pair(op2, n=args.size or N_CUBE, permute=args.permute)
    elif args.only == "data_path":
        p = workloads.build_p1_3d(op2, n=args.size or N_CUBE, permute=args.permute, seed=0)
        out = measure_data_path(op2, p, args.steps, args.warmup)
    else:
        out = measure_prisms(op2, args.steps, args.warmup, n=args.size or 256)
    print(json.dumps({"only": args.only, "result": out}), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--permute", action="store_true", help="random vertex numbering")
    ap.add_argument("--scatter", default=None, choices=["atomic", "warp", "colour", "staged"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--skip-extras", action="store_true",
                    help="only the headline action (no adjoint / batch measurements)")
    ap.add_argument("--only", default=None,
                    choices=["sparsity", "adjoint", "batch", "prisms", "small",
                             "prism_assembly", "scatter", "gather", "data_path"],
                    help="run one secondary measurement alone (profiling runs)")
    ap.add_argument("--size", type=int, default=None,
                    help="with --only: mesh size (cube edge / prism base edge)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    if args.only:
        return run_only(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
