"""Benchmark of the accelerate-fft GPU path on GB300.

Default workload: fft2D Forward on a 4096 x 4096 Complex Float array,
components i.i.d. N(0, 1) from a seed (the reference's headline
configuration: PTX.fft2D, PTX.hs:66-67).  Metric: FFT GFLOP/s with the
algorithmic count 5 N log2 N (N = 4096^2), plus the HBM roofline fraction of
the dominant kernel and of the whole transform.

One JSON line on rank 0.  `--impl reference` times the reference's CPU
implementation of the same path (the oracle's restatement of the pure
Accelerate transform, oracle/adhoc.cpp) on the host cores instead.

Timing: W warm-up steps, then K timed steps; each step is timed with CUDA
events on the launching stream and L2 is flushed (a 256 MiB write) between
steps, outside the events.  The working set (2 x 128 MiB) also exceeds L2.
"""
import argparse
import ctypes
import json
import math
import os
import re
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "accelerate-fft_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = ("FFT GFLOP/s (5N·log2N/t) + % HBM roofline: split-FP16 vs FP32 at "
          "≤2e-6 rel err")


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            pk = json.load(f)
        return float(pk["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.QUERY,
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.thread.join(timeout=2)
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
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def max_over_ranks(ms, world, device):
    """The slowest rank's time: replicas run in parallel, so the job takes as
    long as its slowest rank (a no-op for one process)."""
    if world <= 1:
        return ms
    import torch
    import torch.distributed as dist
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(units_per_rank, world, ms):
    """Whole-job rate: the units every rank processed over the slowest rank's
    time (weak scaling: each rank runs the full workload)."""
    return units_per_rank * world / (ms * 1e-3) / 1e9


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


# ---------------------------------------------------------------------------
# workloads
WORKLOADS = {
    "fft2d_4096": dict(kind="full", shape=(4096, 4096), dtype="c32", mode="forward",
                       desc="fft2D Forward, Complex Float 4096x4096, N(0,1)"),
    "many_65536x1000": dict(kind="many", shape=(65536, 1000), dtype="c32", mode="forward",
                            desc="fft innermost, Complex Float 65536x1000 (8*5*5*5), N(0,1)"),
    "many_4096x1009": dict(kind="many", shape=(4096, 1009), dtype="c32", mode="forward",
                           desc="fft innermost, Complex Float 4096x1009 (Bluestein), N(0,1)"),
    "many_32768x1000": dict(kind="many", shape=(32768, 1000), dtype="c32", mode="forward",
                            desc="fft innermost (profiling size), Complex Float 32768x1000 (8*5*5*5), N(0,1)"),
    "fft3d_256": dict(kind="full", shape=(256, 256, 256), dtype="c32", mode="forward",
                      desc="fft3D Forward, Complex Float 256^3, N(0,1)"),
    "many_2048x65536": dict(kind="many", shape=(2048, 65536), dtype="c32", mode="forward",
                            desc="fft innermost, Complex Float 2048x65536 (four-step), N(0,1)"),
    "many_1024x65521": dict(kind="many", shape=(1024, 65521), dtype="c32", mode="forward",
                            desc="fft innermost, Complex Float 1024x65521 (four-pass Bluestein), N(0,1)"),
    "fft1d_1024_c64": dict(kind="full", shape=(1024,), dtype="c64", mode="roundtrip", dist="uniform",
                           desc="fft1D Forward then Inverse round trip, Complex Double N=1024, "
                                "re/im U[-1,1]"),
    "specconv_8x256": dict(kind="specconv", shape=(8, 256, 256, 256), dtype="c32",
                           desc="spectral convolution fwd+adjoint: 8 Gaussian random fields 256^3 "
                                "(|k|^-5/3 spectrum) and a 256^3 complex filter, Complex Float"),
    "ragged_2000": dict(kind="ragged", count=2000, dtype="c32",
                        desc="ragged batch (profiling size): 2000 Complex Float transforms, lengths "
                             "log-uniform in [16, 65536] (70% 7-smooth, 30% prime), Forward/Inverse "
                             "p=1/2, N(0,1), one persistent launch"),
    "ragged_20000": dict(kind="ragged", count=20000, dtype="c32",
                         desc="ragged batch: 20000 Complex Float transforms, lengths log-uniform in "
                              "[16, 65536] (70% 7-smooth, 30% prime), Forward/Inverse p=1/2, N(0,1), "
                              "one persistent launch"),
}


for _name, _wl in WORKLOADS.items():
    _wl["name"] = _name


# DRAM bytes (read + write) per launch of a workload's dominant kernel from one
# ncu capture (profiles/<kernel>_<workload>.md).  Under ncu's serialised
# replay part of a launch's writes is still in L2 when it ends, so these read
# below the algorithmic bytes.  The ragged figure is the 2000-transform
# capture scaled by elements (same length distribution, traffic proportional).
NCU_TRAFFIC = {
    "fft2d_4096": ("colfft4096_r16b_kernel", 134282496 + 78467072),
    "fft3d_256": ("strfft_tma_kernel", 134264320 + 51690752),
    "ragged_20000": ("ragged_kernel", 1.0691e9 * 157602267 / 16295261),
    "ragged_2000": ("ragged_kernel", 1.0691e9),
}


def ncu_traffic(workload, kernel):
    t = NCU_TRAFFIC.get(workload)
    return float(t[1]) if t and t[0] == kernel else None


def flops_of(shape, kind):
    if kind == "full":
        n = math.prod(shape)
        return 5.0 * n * math.log2(n)
    rows = math.prod(shape[:-1])
    n = shape[-1]
    return 5.0 * rows * n * math.log2(n) if n > 1 else 0.0


def make_input(shape, dtype, seed, dist="normal"):
    import torch
    g = torch.Generator().manual_seed(seed)
    real_t = torch.float64 if dtype == "c64" else torch.float32
    if dist == "uniform":  # i.i.d. uniform on [-1, 1]
        re = torch.rand(shape, generator=g, dtype=real_t) * 2 - 1
        im = torch.rand(shape, generator=g, dtype=real_t) * 2 - 1
    else:
        re = torch.randn(shape, generator=g, dtype=real_t)
        im = torch.randn(shape, generator=g, dtype=real_t)
    return torch.complex(re, im)


def step_modes(wl):
    """Modes one step runs: a round trip is Forward then Inverse."""
    return ("forward", "inverse") if wl["mode"] == "roundtrip" else (wl["mode"],)


def cpu_oracle_run(wl, x_np, threads):
    from oracle import lib as O
    fn = {"full": {1: O.fft1D, 2: O.fft2D, 3: O.fft3D}[len(wl["shape"])], "many": O.fft}[wl["kind"]]
    y = x_np
    for m in step_modes(wl):
        y = fn(0 if m == "forward" else 2, y, threads=threads)
    return y


def cpu_baseline(wl, x_np, budget_s=12.0):
    """The oracle timed on the host cores on a bounded sample of the workload."""
    threads = os.cpu_count() or 1
    shape = wl["shape"]
    sample = x_np
    rows_used = shape[0]
    if wl["kind"] == "many":
        # a bounded number of rows of the same length
        rows_used = min(shape[0], 4096)
        sample = x_np[:rows_used]
    t0 = time.perf_counter()
    cpu_oracle_run(wl, sample, threads)
    one = time.perf_counter() - t0
    reps = max(1, min(20, int(budget_s / max(one, 1e-6))))
    t0 = time.perf_counter()
    for _ in range(reps):
        cpu_oracle_run(wl, sample, threads)
    dt = (time.perf_counter() - t0) / reps
    sub_shape = (rows_used,) + tuple(shape[1:]) if wl["kind"] == "many" else shape
    fl = flops_of(sub_shape, wl["kind"]) * len(step_modes(wl))
    return {"value": fl / dt / 1e9, "unit": "GFLOP/s", "cores": threads, "kind": "port",
            "sample": "%d run(s) of %s on shape %s (oracle C++ restatement of Adhoc.hs, OpenMP)"
                      % (reps, wl["desc"], "x".join(map(str, sub_shape))),
            "seconds_per_run": dt}


def run_reference(args, wl):
    world, rank, _ = dist_init()
    if rank != 0:
        return
    import numpy as np
    x = make_input(wl["shape"], wl["dtype"], 1234, wl.get("dist", "normal")).numpy()
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_oracle_run(wl, x, threads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        cpu_oracle_run(wl, x, threads)
    dt = (time.perf_counter() - t0) / args.steps
    fl = flops_of(wl["shape"], wl["kind"]) * len(step_modes(wl))
    val = fl / dt / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": val, "unit": "GFLOP/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if wl["dtype"] == "c64" else "f32", "data": "synthetic",
        "config": {"workload": wl["desc"], "shape": list(wl["shape"]), "seed": 1234},
        "cpu_baseline": {"value": val, "unit": "GFLOP/s", "cores": threads, "kind": "port",
                         "sample": "each step one full %s on the host cores (oracle C++ "
                                   "restatement of the reference's pure-Accelerate transform; "
                                   "the Haskell reference cannot be built offline)" % wl["desc"]},
        "e2e": {"value": val, "unit": "GFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_gbfft(args, wl):
    line = measure_gbfft(args, wl)
    if line is not None:
        print(json.dumps(line), flush=True)
    finish_dist()


def finish_dist():
    if int(os.environ.get("WORLD_SIZE", "1")) > 1:
        import torch.distributed as dist
        if dist.is_initialized():
            dist.destroy_process_group()


def init_dist(local):
    import torch
    torch.cuda.set_device(local)
    if int(os.environ.get("WORLD_SIZE", "1")) > 1:
        import torch.distributed as dist
        if not dist.is_initialized():
            dist.init_process_group("nccl")


def measure_gbfft(args, wl, headline=True):
    """One plan workload (fft / fft1D / fft2D / fft3D): the JSON line's fields
    on rank 0, None on the other ranks.  headline=False skips the access-pattern
    probe (reported for the headline workload only)."""
    import numpy as np
    import torch

    import gbfft
    from gbfft import _lib as L

    world, rank, local = dist_init()
    init_dist(local)
    dev = torch.device("cuda", local)
    lib = L.lib()
    shape = wl["shape"]
    dtype = torch.complex128 if wl["dtype"] == "c64" else torch.complex64
    elem = 16 if wl["dtype"] == "c64" else 8
    nelem = math.prod(shape)
    x_cpu = make_input(shape, wl["dtype"], 1234 + rank, wl.get("dist", "normal"))
    x = x_cpu.to(dev)
    y = torch.empty_like(x)
    z = torch.empty_like(x)  # round trip: the Inverse of y
    tune_report = None
    if not args.no_tune:
        # plan creation with the autotuner (untimed, like any plan creation)
        tune_report = gbfft.autotune(shape, kind=wl["kind"], dtype=dtype, precision=args.precision)
    plan = gbfft.Plan(shape, kind=wl["kind"], dtype=dtype, precision=args.precision)
    info = plan.info
    npass = info["launches"]
    kernels = plan.pass_kernels()
    modes = [gbfft.mode_code(m) for m in step_modes(wl)]
    # (mode, input, output) of each transform of a step
    ops = [(modes[0], x, y)] + ([(modes[1], y, z)] if len(modes) > 1 else [])
    result = ops[-1][2]
    nlaunch = npass * len(ops)
    kernels = kernels * len(ops)
    stream = torch.cuda.current_stream(dev)
    sp = ctypes.c_void_p(stream.cuda_stream)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def one_step(events=None):
        if events is None:
            for m, a, b in ops:
                L.check(lib.gbfft_exec(plan.handle, m, ctypes.c_void_p(a.data_ptr()),
                                       ctypes.c_void_p(b.data_ptr()), sp))
            return
        events[0].record(stream)
        j = 0
        for m, a, b in ops:
            for i in range(npass):
                L.check(lib.gbfft_exec_range(plan.handle, m, i, 1, ctypes.c_void_p(a.data_ptr()),
                                             ctypes.c_void_p(b.data_ptr()), sp))
                j += 1
                events[j].record(stream)

    for _ in range(args.warmup):
        one_step()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    sampler = ClockSampler(torch.cuda.current_device()) if rank == 0 else None
    if sampler:
        sampler.start()
        time.sleep(1.0)  # let nvidia-smi finish starting before the timed region
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(nlaunch + 1)] for _ in range(args.steps)]
    torch.cuda.synchronize()
    for k in range(args.steps):
        flush.fill_(float(k))
        one_step(evs[k])
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clocks = sampler.stop() if sampler else None
    step_ms = [e[0].elapsed_time(e[-1]) for e in evs]
    pass_ms = [[e[i].elapsed_time(e[i + 1]) for e in evs] for i in range(nlaunch)]
    total_ms = max_over_ranks(sum(step_ms), world, dev)
    ms = total_ms / args.steps
    fl = flops_of(shape, wl["kind"]) * len(ops)
    value = job_throughput(fl, world, ms)

    peak, peak_kind = load_peaks()
    bytes_pass = 2.0 * nelem * elem  # one compulsory read + write of the array per pass
    avg_pass = [sum(p) / len(p) for p in pass_ms]
    dom = max(range(nlaunch), key=lambda i: avg_pass[i]) if nlaunch else 0
    ach = bytes_pass / (avg_pass[dom] * 1e-3) / 1e9 if nlaunch else 0.0
    ach_tr = bytes_pass * len(ops) / (ms * 1e-3) / 1e9

    # the access pattern's own ceiling (outside the timed region): a plain
    # copy of the same array in the column tiles of the plan's strided pass
    # (the cluster tile width the plan reports, else 16 columns) over all
    # rows -- what a strided pass moving such tiles cannot beat -- and the
    # contiguous copy of a row pass
    ceiling = None
    full2 = wl["kind"] == "full" and len(shape) >= 2
    rowsv = wl["kind"] == "many" and len(shape) >= 2 and shape[-1] % 2 == 0
    if rank == 0 and headline and (full2 or rowsv) and elem == 8 and nlaunch:
        rows, cols = (shape[0], nelem // shape[0]) if full2 else (nelem // shape[-1], shape[-1])
        mt = re.search(r"cluster-columns=(\d+)", plan.describe())
        tile_w = int(mt.group(1)) if mt else 16
        gbs = {}
        for w in ((tile_w, cols) if full2 else (cols,)):
            for _ in range(3):
                L.check(lib.gbfft_probe_tile_copy(rows, cols, w, ctypes.c_void_p(x.data_ptr()),
                                                  ctypes.c_void_p(z.data_ptr()), sp), "gbfft_probe_tile_copy")
            ts = []
            for k in range(10):
                flush.fill_(float(k))
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                L.check(lib.gbfft_probe_tile_copy(rows, cols, w, ctypes.c_void_p(x.data_ptr()),
                                                  ctypes.c_void_p(z.data_ptr()), sp), "gbfft_probe_tile_copy")
                b.record(stream)
                torch.cuda.synchronize()
                ts.append(a.elapsed_time(b))
            gbs[w] = bytes_pass / (statistics.median(ts) * 1e-3) / 1e9
        row_kernel = kernels[dom].startswith("row")
        rel = gbs[cols] if row_kernel else gbs.get(tile_w)
        ceiling = {"kernel": kernels[dom], "tile_columns": tile_w if full2 else None,
                   "tile_copy_gbs": gbs.get(tile_w) if full2 else None, "contiguous_copy_gbs": gbs[cols],
                   "frac_of_pattern": ach / rel if rel else None,
                   "note": "gbfft_probe_tile_copy over the %dx%d array: %s; frac_of_pattern = achieved / the "
                           "copy of the dominant kernel's pattern" % (
                               rows, cols, "%d-column tiles (the strided pass's pattern) and whole rows" % tile_w
                               if full2 else "whole rows (the row kernels' pattern)")}

    # accuracy of one result vs FP64 (numpy pocketfft), outside the timed region
    rel_err = None
    roundtrip_err = None
    ref = None
    if rank == 0 and not args.no_check:
        one_step()
        torch.cuda.synchronize()
        yy = y.cpu().numpy().astype(np.complex128)
        xx = x_cpu.numpy().astype(np.complex128)
        axes = tuple(range(len(shape))) if wl["kind"] == "full" else (-1,)
        ref = np.fft.fftn(xx, axes=axes) if step_modes(wl)[0] == "forward" else np.fft.ifftn(xx, axes=axes)
        rel_err = float(np.linalg.norm(yy - ref) / np.linalg.norm(ref))
        if len(ops) > 1:  # Inverse(Forward(x)) against x
            zz = z.cpu().numpy().astype(np.complex128)
            roundtrip_err = float(np.linalg.norm(zz - xx) / np.linalg.norm(xx))

    # the other precision of the same transform (split-FP16 tensor-core rows vs
    # plain FP32), timed the same way, with its own error vs FP64
    other_prec = None
    if rank == 0 and wl["dtype"] == "c32" and not args.no_compare:
        other = "split_fp16" if args.precision == "plain" else "plain"
        try:
            if not args.no_tune:
                gbfft.autotune(shape, kind=wl["kind"], dtype=dtype, precision=other)
            p2 = gbfft.Plan(shape, kind=wl["kind"], dtype=dtype, precision=other)
        except Exception as exc:  # the planner rejects shapes it has no kernel for
            other_prec = {"precision": other, "unavailable": str(exc)}
        else:
            mode = modes[0]
            for _ in range(max(3, args.warmup)):
                L.check(lib.gbfft_exec(p2.handle, mode, ctypes.c_void_p(x.data_ptr()),
                                       ctypes.c_void_p(y.data_ptr()), sp))
            ts = []
            for k in range(args.steps):
                flush.fill_(float(k))
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                L.check(lib.gbfft_exec(p2.handle, mode, ctypes.c_void_p(x.data_ptr()),
                                       ctypes.c_void_p(y.data_ptr()), sp))
                b.record(stream)
                torch.cuda.synchronize()
                ts.append(a.elapsed_time(b))
            ms2 = statistics.mean(ts)
            err2 = None
            if ref is not None:
                yy2 = y.cpu().numpy().astype(np.complex128)
                err2 = float(np.linalg.norm(yy2 - ref) / np.linalg.norm(ref))
            other_prec = {"precision": other, "ms_per_step": ms2, "transforms": 1,
                          "value": flops_of(shape, wl["kind"]) * world / (ms2 * 1e-3) / 1e9, "unit": "GFLOP/s",
                          "rel_err_vs_fp64": err2, "speedup_of_split_fp16_over_fp32":
                              (ms / len(ops) / ms2) if other == "split_fp16" else (ms2 * len(ops) / ms),
                          "kernels": p2.pass_kernels()}
            p2.close()

    # end to end through the C ABI with host buffers (pinned): every step
    # copies its input host -> device, runs its transforms and copies the
    # result back.  Single stream: one step at a time.  Pipelined: steps
    # rotate over NS streams with their own buffers, so one step's
    # host -> device copy overlaps another's device -> host copy (the link is
    # full duplex) and the transforms.
    e2e_line = None
    if not args.no_e2e:
        NS = 3
        hx = x_cpu.pin_memory()
        hy = [torch.empty_like(hx).pin_memory() for _ in range(NS)]

        def run_ops(bufs, st_ptr):
            # bufs: (input, intermediate, output) device buffers of one step
            for j, (m, _a, _b) in enumerate(ops):
                a = bufs[0] if j == 0 else bufs[1]
                b = bufs[1] if j == 0 and len(ops) > 1 else bufs[2]
                L.check(lib.gbfft_exec(plan.handle, m, ctypes.c_void_p(a.data_ptr()), ctypes.c_void_p(b.data_ptr()),
                                       st_ptr))

        e2e_ms = []
        for k in range(max(3, min(args.steps, 20)) + 2):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            x.copy_(hx, non_blocking=True)
            run_ops((x, y, result), sp)
            hy[0].copy_(result, non_blocking=True)
            e1.record(stream)
            torch.cuda.synchronize()
            if k >= 2:
                e2e_ms.append(e0.elapsed_time(e1))
        e2e_single = statistics.mean(e2e_ms)
        streamsN = [torch.cuda.Stream(dev) for _ in range(NS)]
        bufsN = [(torch.empty_like(x), torch.empty_like(x), torch.empty_like(x)) for _ in range(NS)]
        n_pipe = max(6, min(args.steps, 20))

        def pipelined(nsteps):
            for k in range(nsteps):
                st = streamsN[k % NS]
                bx, bm, bo = bufsN[k % NS]
                with torch.cuda.stream(st):
                    bx.copy_(hx, non_blocking=True)
                    run_ops((bx, bm, bo), ctypes.c_void_p(st.cuda_stream))
                    hy[k % NS].copy_(bo, non_blocking=True)

        pipelined(2)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        pipelined(n_pipe)
        torch.cuda.synchronize()
        e2e_pipe = (time.perf_counter() - t0) * 1e3 / n_pipe
        # the steady-state figure: steps issued back to back over NS streams
        e2e = fl * world / (e2e_pipe * 1e-3) / 1e9
        e2e_line = {"value": e2e, "unit": "GFLOP/s", "h2d_bytes_per_step": nelem * elem,
                    "d2h_bytes_per_step": nelem * elem, "ms_per_step": e2e_pipe,
                    "ms_per_step_single_stream": e2e_single, "ms_per_step_pipelined": e2e_pipe,
                    "timing": "pipelined over %d streams: host wall clock over %d steps between device "
                              "synchronisations (the reported value); single stream: CUDA events per step, "
                              "for reference" % (NS, n_pipe)}

    # cuFFT on the same input and timing (comparator only, not the product)
    cufft_ms = None
    if rank == 0 and not args.no_cufft:
        f1 = (lambda t: torch.fft.fftn(t)) if wl["kind"] == "full" else (lambda t: torch.fft.fft(t, dim=-1))
        fi = (lambda t: torch.fft.ifftn(t)) if wl["kind"] == "full" else (lambda t: torch.fft.ifft(t, dim=-1))
        f = (lambda t: fi(f1(t))) if len(ops) > 1 else f1
        for _ in range(3):
            f(x)
        ts = []
        for k in range(args.steps):
            flush.fill_(float(k))
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            f(x)
            b.record(stream)
            torch.cuda.synchronize()
            ts.append(a.elapsed_time(b))
        cufft_ms = statistics.mean(ts)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_baseline(wl, x_cpu.numpy())

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "GFLOP/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if wl["dtype"] == "c64" else "f32", "data": "synthetic",
            "config": {"workload": wl["desc"], "shape": list(shape), "kind": wl["kind"],
                       "precision": args.precision, "seed": 1234,
                       "l2": "flushed (256 MiB write) between timed steps; working set 2x%d MiB"
                             % (nelem * elem >> 20),
                       "plan": plan.describe(), "transforms_per_step": len(ops),
                       "parallelism": "replicas" if world > 1 else "single",
                       "autotune": tune_report.strip().splitlines()[-1] if tune_report else "off"},
            "roofline": {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s",
                         "frac": ach / peak,
                         "traffic": ncu_traffic(wl["name"], kernels[dom] if npass else None),
                         "peak_source": peak_kind,
                         "kernel": "pass %d of %d (%s)" % (dom, npass, kernels[dom] if npass else "-"),
                         "bytes_alg_per_launch": bytes_pass,
                         "kernel_ms": avg_pass[dom] if npass else None,
                         "pattern_ceiling": ceiling},
            "roofline_transform": {"achieved": ach_tr, "frac": ach_tr / peak, "kernels": kernels,
                                   "bytes_alg": bytes_pass, "pass_ms": avg_pass},
            "rel_err_vs_fp64": rel_err,
            "roundtrip_rel_err": roundtrip_err,
            "other_precision": other_prec,
            "e2e": e2e_line,
            "gpu_launches": args.steps * nlaunch,
            "clocks": clocks,
            "cufft_comparator_ms": cufft_ms,
            "cpu_baseline": cpu,
        }
        plan.close()
        return line
    plan.close()
    return None


def run_ragged(args, wl):
    line = measure_ragged(args, wl)
    if line is not None:
        print(json.dumps(line), flush=True)
    finish_dist()


def measure_ragged(args, wl, cpu_budget_s=12.0):
    import numpy as np
    import torch

    import gbfft
    from gbfft import _lib as L
    from gbfft import synth

    world, rank, local = dist_init()
    init_dist(local)
    dev = torch.device("cuda", local)
    lengths, modes = synth.ragged_lengths(wl["count"], seed=4)
    total = int(lengths.sum())
    g = torch.Generator().manual_seed(1234 + rank)
    x_cpu = torch.complex(torch.randn(total, generator=g), torch.randn(total, generator=g))
    x = x_cpu.to(dev)
    y = torch.empty_like(x)
    tune_report = None
    if not args.no_tune:
        # plan creation with the autotuner (untimed, like any plan creation)
        tune_report = gbfft.ragged_autotune(lengths, modes)
    t0 = time.perf_counter()
    plan = gbfft.RaggedPlan(lengths, modes)
    plan_s = time.perf_counter() - t0
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    fl = float(np.sum(5.0 * lengths * np.log2(np.maximum(lengths, 2))))
    bytes_alg = 2.0 * total * 8

    def timed(per_transform, steps, warm):
        for _ in range(warm):
            plan.exec_ptr(x.data_ptr(), y.data_ptr(), stream, per_transform)
        torch.cuda.synchronize()
        ts = []
        for k in range(steps):
            flush.fill_(float(k))
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            plan.exec_ptr(x.data_ptr(), y.data_ptr(), stream, per_transform)
            b.record(stream)
            torch.cuda.synchronize()
            ts.append(a.elapsed_time(b))
        return ts

    if world > 1:
        torch.distributed.barrier()
    sampler = ClockSampler(torch.cuda.current_device()) if rank == 0 else None
    if sampler:
        sampler.start()
        time.sleep(1.0)
    ts = timed(False, args.steps, args.warmup)
    if world > 1:
        torch.distributed.barrier()
    clocks = sampler.stop() if sampler else None
    ms = max_over_ranks(sum(ts) / len(ts), world, dev)
    status = plan.status()
    value = job_throughput(fl, world, ms)
    peak, peak_kind = load_peaks()
    ach = bytes_alg / (ms * 1e-3) / 1e9
    per_ms = statistics.mean(timed(True, 3, 1)) if rank == 0 and not args.no_compare else None
    # accuracy on a sample of transforms vs FP64
    rel = None
    if rank == 0 and not args.no_check:
        yy = y.cpu().numpy()
        xx = x_cpu.numpy()
        rng = np.random.default_rng(0)
        errs = []
        for i in rng.choice(len(lengths), 200, replace=False):
            n, o = int(lengths[i]), int(plan.offsets[i])
            r = np.fft.fft(xx[o:o + n].astype(np.complex128)) if modes[i] == -1 else \
                np.fft.ifft(xx[o:o + n].astype(np.complex128))
            errs.append(float(np.linalg.norm(yy[o:o + n] - r) / np.linalg.norm(r)))
        rel = max(errs)
    hx = x_cpu.pin_memory()
    hy = torch.empty_like(hx).pin_memory()
    e2e = []
    for k in range(5):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        x.copy_(hx, non_blocking=True)
        plan.exec_ptr(x.data_ptr(), y.data_ptr(), stream)
        hy.copy_(y, non_blocking=True)
        b.record(stream)
        torch.cuda.synchronize()
        if k >= 2:
            e2e.append(a.elapsed_time(b))
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_baseline_ragged(lengths, modes, plan.offsets, x_cpu.numpy(), budget_s=cpu_budget_s)
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "GFLOP/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": wl["desc"], "count": int(len(lengths)), "elements": total,
                       "seed": 4, "l2": "flushed (256 MiB write) between timed steps; working set "
                       "2x%d MiB" % (total * 8 >> 20), "plan_seconds": plan_s,
                       "autotune": tune_report.strip().splitlines()[-1] if tune_report else "off",
                       "parallelism": "replicas" if world > 1 else "single"},
            "roofline": {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s",
                         "frac": ach / peak, "traffic": ncu_traffic(wl["name"], "ragged_kernel"),
                         "peak_source": peak_kind,
                         "kernel": "ragged_kernel<float> (the single persistent launch)",
                         "bytes_alg_per_launch": bytes_alg, "kernel_ms": ms},
            "per_transform_comparator": {"ms_per_step": per_ms,
                                         "value": fl / (per_ms * 1e-3) / 1e9 if per_ms else None,
                                         "launches_per_step": "one launch sequence per transform"},
            "rel_err_vs_fp64_max_of_200": rel, "device_status": status,
            "e2e": {"value": fl * world / (statistics.mean(e2e) * 1e-3) / 1e9, "unit": "GFLOP/s",
                    "h2d_bytes_per_step": total * 8, "d2h_bytes_per_step": total * 8,
                    "ms_per_step": statistics.mean(e2e)},
            "gpu_launches": args.steps, "clocks": clocks, "cpu_baseline": cpu,
        }
        plan.close()
        return line
    plan.close()
    return None


def grf_fields(shape, seed, device="cpu"):
    """Gaussian random fields with power spectrum ~ |k|^-5/3: seeded white
    noise shaped in Fourier space, normalised to unit variance per component.
    Input synthesis only (torch's FFT on `device`), not the measured path."""
    import torch
    b, d, h, w = shape
    g = torch.Generator(device=device).manual_seed(seed)
    kz = torch.fft.fftfreq(d, device=device, dtype=torch.float64)[:, None, None]
    ky = torch.fft.fftfreq(h, device=device, dtype=torch.float64)[None, :, None]
    kx = torch.fft.fftfreq(w, device=device, dtype=torch.float64)[None, None, :]
    k = torch.sqrt(kx * kx + ky * ky + kz * kz)
    k[0, 0, 0] = 1.0
    amp = (k ** (-5.0 / 3.0)) ** 0.5
    amp[0, 0, 0] = 0.0
    out = torch.empty(shape, dtype=torch.complex64, device=device)
    for i in range(b):
        noise = torch.complex(torch.randn((d, h, w), generator=g, device=device, dtype=torch.float64),
                              torch.randn((d, h, w), generator=g, device=device, dtype=torch.float64))
        f = torch.fft.ifftn(torch.fft.fftn(noise) * amp)
        f = f / torch.sqrt(torch.mean(torch.abs(f) ** 2) / 2)
        out[i] = f.to(torch.complex64)
    return out


def run_specconv(args, wl):
    line = measure_specconv(args, wl)
    if line is not None:
        print(json.dumps(line), flush=True)
    finish_dist()


def measure_specconv(args, wl):
    import numpy as np
    import torch

    import gbfft

    world, rank, local = dist_init()
    init_dist(local)
    dev = torch.device("cuda", local)
    shape = wl["shape"]
    x_cpu = grf_fields(shape, 5 + rank, device=dev).cpu()
    g = np.random.default_rng(55)
    H_cpu = torch.from_numpy(((g.standard_normal(shape[1:]) + 1j * g.standard_normal(shape[1:]))
                              / np.sqrt(2)).astype(np.complex64))
    x = x_cpu.to(dev)
    H = H_cpu.to(dev)
    plan = gbfft.SpecConvPlan(*shape)
    stream = torch.cuda.current_stream(dev)
    y = torch.empty_like(x)
    gx = torch.empty_like(x)
    gH = torch.empty_like(H)
    N = shape[1] * shape[2] * shape[3]
    fl = (16 + 24) * 5.0 * N * math.log2(N)  # 8 fields: fwd 2, adjoint 3 transforms each
    import ctypes
    from gbfft import _lib as L
    lib = L.lib()
    sp = ctypes.c_void_p(stream.cuda_stream)
    P = lambda t: ctypes.c_void_p(t.data_ptr())

    def step(ev=None):
        if ev:
            ev[0].record(stream)
        L.check(lib.gbfft_specconv_fwd(plan.handle, P(x), P(H), P(y), sp))
        if ev:
            ev[1].record(stream)
        # L = 1/2 ||y||^2: g_y = y
        L.check(lib.gbfft_specconv_bwd(plan.handle, P(x), P(H), P(y), P(gx), P(gH), sp))
        if ev:
            ev[2].record(stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    sampler = ClockSampler(torch.cuda.current_device()) if rank == 0 else None
    if sampler:
        sampler.start()
        time.sleep(1.0)
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.steps)]
    for k in range(args.steps):
        step(evs[k])
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clocks = sampler.stop() if sampler else None
    fwd = [e[0].elapsed_time(e[1]) for e in evs]
    bwd = [e[1].elapsed_time(e[2]) for e in evs]
    ms = max_over_ranks((sum(fwd) + sum(bwd)) / args.steps, world, dev)
    value = job_throughput(fl, world, ms)
    peak, peak_kind = load_peaks()
    # algorithmic bytes: fwd reads x, H and writes y; adjoint reads x, g_y, H and writes g_x, g_H
    fb = (2 * x.numel() + H.numel()) * 8.0
    bb = (3 * x.numel() + 2 * H.numel()) * 8.0
    fms, bms = statistics.mean(fwd), statistics.mean(bwd)
    hx = x_cpu.pin_memory()
    hy = torch.empty_like(hx).pin_memory()
    e2e = []
    for k in range(4):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        x.copy_(hx, non_blocking=True)
        step()
        hy.copy_(gx, non_blocking=True)
        b.record(stream)
        torch.cuda.synchronize()
        if k >= 1:
            e2e.append(a.elapsed_time(b))
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "GFLOP/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": wl["desc"], "shape": list(shape), "seed": 5,
                       "l2": "working set > 5 GiB per step (no flush needed)",
                       "parallelism": "replicas" if world > 1 else "single"},
            "roofline": {"bound": "hbm", "achieved": (fb + bb) / (ms * 1e-3) / 1e9, "peak": peak,
                         "unit": "GB/s", "frac": (fb + bb) / (ms * 1e-3) / 1e9 / peak, "traffic": None,
                         "peak_source": peak_kind, "kernel": "whole fwd+adjoint step",
                         "fwd_ms": fms, "bwd_ms": bms, "bytes_alg_fwd": fb, "bytes_alg_bwd": bb},
            "e2e": {"value": fl * world / (statistics.mean(e2e) * 1e-3) / 1e9, "unit": "GFLOP/s",
                    "h2d_bytes_per_step": x.numel() * 8, "d2h_bytes_per_step": x.numel() * 8,
                    "ms_per_step": statistics.mean(e2e)},
            "gpu_launches": args.steps * 12, "clocks": clocks,
            "cpu_baseline": (cpu_baseline_specconv(x_cpu.numpy(), H_cpu.numpy(), fl / shape[0])
                             if world == 1 and not args.no_cpu else None),
        }
        plan.close()
        return line
    plan.close()
    return None


def cpu_baseline_specconv(x_np, H_np, flops_per_field):
    """The reference's composition of the spectral convolution and its
    gradient (fft3D Forward, product, fft3D Inverse; the adjoint as three more
    fft3D calls and two products) through the oracle's restatement of fft3D,
    on the host cores, for a bounded sample: one of the fields."""
    import numpy as np
    from oracle import lib as O
    threads = os.cpu_count() or 1
    x = x_np[0]
    t0 = time.perf_counter()
    X = O.fft3D(0, x, threads=threads)                      # Forward
    y = O.fft3D(2, X * H_np, threads=threads)               # Inverse (y; also g_y for L = 1/2|y|^2)
    gY = O.fft3D(0, y, threads=threads) / np.float32(y.size)  # g_Y = Forward(g_y) / N
    Xr = O.fft3D(0, x, threads=threads)                     # X recomputed, as the adjoint kernel does
    gH = np.conj(Xr) * gY                                   # this field's share of g_H
    gx = O.fft3D(1, np.conj(H_np) * gY, threads=threads)    # Reverse
    dt = time.perf_counter() - t0
    del gH, gx
    return {"value": flops_per_field / dt / 1e9, "unit": "GFLOP/s", "cores": threads, "kind": "port",
            "sample": "1 of the 8 fields: forward (2 fft3D) and adjoint (3 fft3D) composed from the oracle "
                      "C++ restatement of fft3D (FFT.hs:150-187) and elementwise products",
            "seconds": dt}


def cpu_baseline_ragged(lengths, modes, offsets, x_np, budget_s=12.0):
    """The oracle on a bounded prefix of the ragged batch, one transform at a
    time on all host cores (threads over transforms)."""
    import concurrent.futures as cf
    import numpy as np
    from oracle import lib as O
    threads = os.cpu_count() or 1
    x64 = x_np.astype(np.complex64)

    def one(i):
        n, o = int(lengths[i]), int(offsets[i])
        O.fft1D(0 if modes[i] == -1 else 2, x64[o:o + n], threads=1)
        return 5.0 * n * math.log2(max(n, 2))

    done_fl, done_n = 0.0, 0
    t0 = time.perf_counter()
    order = np.random.default_rng(0).permutation(len(lengths))
    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        for start in range(0, len(order), threads * 4):
            batch = order[start:start + threads * 4]
            done_fl += sum(ex.map(one, batch))
            done_n += len(batch)
            if time.perf_counter() - t0 > budget_s:
                break
    dt = time.perf_counter() - t0
    return {"value": done_fl / dt / 1e9, "unit": "GFLOP/s", "cores": threads, "kind": "port",
            "sample": "%d of the %d transforms (random order), oracle C++ restatement of Adhoc.hs, "
                      "one transform per host thread" % (done_n, len(lengths))}


def _compact(line):
    """The per-config summary carried in the headline line."""
    if line is None:
        return None
    keep = {}
    for k in ("ms_per_step", "value", "unit", "rel_err_vs_fp64", "roundtrip_rel_err", "cufft_comparator_ms",
              "cpu_baseline", "clocks", "gpu_launches"):
        if k in line:
            keep[k] = line[k]
    keep["workload"] = line["config"]["workload"]
    if "plan" in line["config"]:
        keep["plan"] = line["config"]["plan"]
    r = line.get("roofline", {})
    keep["roofline"] = {k: r.get(k) for k in ("bound", "achieved", "peak", "unit", "frac", "traffic", "kernel",
                                              "kernel_ms", "bytes_alg_per_launch") if k in r}
    if "roofline_transform" in line:
        keep["roofline_transform"] = {k: line["roofline_transform"][k] for k in ("achieved", "frac", "kernels")}
    e = line.get("e2e") or {}
    keep["e2e"] = {k: e.get(k) for k in ("value", "unit", "h2d_bytes_per_step", "d2h_bytes_per_step",
                                         "ms_per_step")}
    if line.get("other_precision"):
        keep["other_precision"] = line["other_precision"]
    return keep


def measure_config3(args):
    """Config 3: fft (innermost axis) over a 65536 x 1000 and a 4096 x 1009
    Complex Float array, plain FP32 and split-FP16 tensor-core plans; the
    workload's time is the sum of the two transforms."""
    a = measure_gbfft(args, WORKLOADS["many_65536x1000"], headline=False)
    b = measure_gbfft(args, WORKLOADS["many_4096x1009"], headline=False)
    if a is None or b is None:
        return None
    peak, _ = load_peaks()
    shapes = [(65536, 1000), (4096, 1009)]
    fl = [flops_of(sh, "many") for sh in shapes]
    byts = sum(2.0 * 8 * sh[0] * sh[1] for sh in shapes)
    ms = a["ms_per_step"] + b["ms_per_step"]
    out = {"workload": "fft innermost axis, Complex Float 65536x1000 (2^3*5^3) plus 4096x1009 (prime), N(0,1)",
           "ms_per_step": ms, "value": sum(fl) / (ms * 1e-3) / 1e9, "unit": "GFLOP/s",
           "rel_err_vs_fp64": max(a["rel_err_vs_fp64"] or 0, b["rel_err_vs_fp64"] or 0),
           "roofline": {"bound": "hbm", "achieved": byts / (ms * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
                        "frac": byts / (ms * 1e-3) / 1e9 / peak, "bytes_alg": byts}}
    oa, ob = a.get("other_precision") or {}, b.get("other_precision") or {}
    if "ms_per_step" in oa and "ms_per_step" in ob:
        ms2 = oa["ms_per_step"] + ob["ms_per_step"]
        out["split_fp16"] = {"ms_per_step": ms2, "value": sum(fl) / (ms2 * 1e-3) / 1e9, "unit": "GFLOP/s",
                             "roofline_frac": byts / (ms2 * 1e-3) / 1e9 / peak,
                             "rel_err_vs_fp64": max(oa.get("rel_err_vs_fp64") or 0, ob.get("rel_err_vs_fp64") or 0),
                             "speedup_of_split_fp16_over_fp32": ms / ms2,
                             "kernels": {"65536x1000": oa.get("kernels"), "4096x1009": ob.get("kernels")}}
    else:
        out["split_fp16"] = {"unavailable": [oa.get("unavailable"), ob.get("unavailable")]}
    ea, eb = a["e2e"], b["e2e"]
    if ea and eb:
        ems = ea["ms_per_step"] + eb["ms_per_step"]
        out["e2e"] = {"value": sum(fl) / (ems * 1e-3) / 1e9, "unit": "GFLOP/s",
                      "h2d_bytes_per_step": ea["h2d_bytes_per_step"] + eb["h2d_bytes_per_step"],
                      "d2h_bytes_per_step": ea["d2h_bytes_per_step"] + eb["d2h_bytes_per_step"], "ms_per_step": ems}
    ca, cb = a.get("cpu_baseline"), b.get("cpu_baseline")
    if ca and cb:
        t = fl[0] / (ca["value"] * 1e9) + fl[1] / (cb["value"] * 1e9)
        out["cpu_baseline"] = {"value": sum(fl) / t / 1e9, "unit": "GFLOP/s", "cores": ca["cores"], "kind": "port",
                               "sample": "%s; %s" % (ca["sample"], cb["sample"])}
    if a.get("cufft_comparator_ms") and b.get("cufft_comparator_ms"):
        out["cufft_comparator_ms"] = a["cufft_comparator_ms"] + b["cufft_comparator_ms"]
    out["arrays"] = {"65536x1000": _compact(a), "4096x1009": _compact(b)}
    return out


def run_all(args):
    """The default run: config 2 (fft2D 4096^2, the headline `value`) with
    configs 1, 3, 4 and 5 measured in the same process and reported under
    `configs`."""
    import copy
    head = measure_gbfft(args, WORKLOADS["fft2d_4096"])
    sub = copy.copy(args)
    sub.steps = max(3, min(args.steps, 10))
    sub.warmup = 3
    c1 = measure_gbfft(sub, WORKLOADS["fft1d_1024_c64"], headline=False)
    c3 = measure_config3(sub)
    subr = copy.copy(sub)
    subr.no_tune = True  # the ragged tuner keeps the defaults for this batch (measured); plan creation stays short
    c4 = measure_ragged(subr, WORKLOADS["ragged_20000"], cpu_budget_s=8.0)
    c5 = measure_specconv(sub, WORKLOADS["specconv_8x256"])
    if head is not None:
        c4c = _compact(c4)
        if c4 is not None:
            c4c["per_transform_comparator"] = c4.get("per_transform_comparator")
            c4c["rel_err_vs_fp64_max_of_200"] = c4.get("rel_err_vs_fp64_max_of_200")
            c4c["device_status"] = c4.get("device_status")
            pt = (c4.get("per_transform_comparator") or {}).get("ms_per_step")
            c4c["speedup_over_one_launch_per_transform"] = pt / c4["ms_per_step"] if pt else None
        c5c = _compact(c5)
        if c5 is not None:
            c5c["fwd_ms"] = c5["roofline"]["fwd_ms"]
            c5c["adjoint_ms"] = c5["roofline"]["bwd_ms"]
        head["configs"] = {
            "1": _compact(c1),
            "2": {"workload": head["config"]["workload"], "see": "the headline fields of this line"},
            "3": c3, "4": c4c, "5": c5c,
            "note": "configs 1, 3, 4, 5 timed as the headline (CUDA events, L2 flushed between steps) with "
                    "%d steps after 3 warm-up steps each" % sub.steps,
        }
        print(json.dumps(head), flush=True)
    finish_dist()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gbfft", choices=["gbfft", "reference"])
    ap.add_argument("--workload", default="all", choices=["all"] + sorted(WORKLOADS),
                    help="all (default): config 2 as the headline plus configs 1, 3, 4, 5 under `configs`")
    ap.add_argument("--precision", default="plain", choices=["plain", "split_fp16"])
    ap.add_argument("--no-check", action="store_true")
    ap.add_argument("--no-cufft", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true",
                    help="skip the end-to-end runs with host buffers (keeps device memory small for profiler captures)")
    ap.add_argument("--no-tune", action="store_true",
                    help="create plans with the planner defaults instead of autotuning them")
    ap.add_argument("--no-compare", action="store_true",
                    help="skip the comparison runs (the other precision; the ragged batch as "
                         "one launch sequence per transform)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args, WORKLOADS["fft2d_4096" if args.workload == "all" else args.workload])
        return
    if args.workload == "all":
        run_all(args)
        return
    wl = WORKLOADS[args.workload]
    if wl["kind"] == "ragged":
        run_ragged(args, wl)
    elif wl["kind"] == "specconv":
        run_specconv(args, wl)
    else:
        run_gbfft(args, wl)


if __name__ == "__main__":
    main()
