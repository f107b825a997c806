"""Benchmark: SAT throughput in GB/s (input + output bytes) against the
measured HBM copy bandwidth of one GB300.

Headline workload (one step = one SAT over one synthetic image already in
HBM): f32 -> f32 plain SAT of an 8192 x 8192 image, uniform [0,1) values.
Inputs (256 MiB) and outputs (256 MiB) are each larger than the 129 MB L2, so
no L2 flush is needed between steps.  The same line also reports the 8192^2
u8 -> u32 SAT, the compensated f32 SAT (and its time ratio to plain), the
4096^2 f64 SAT and the batched uneven-image case.

`--impl reference` times the reference's CPU integral image instead
(IntegralImageParallel, pengdada/SAT integralImage.h:129-146, as restated in
oracle/ with OpenMP over every host core) on the same workload.

Under torchrun (N > 1) every rank runs an independent replica on its own GPU
(no data exchange: images are independent), "scaling": "weak".
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

GB = 1e9
W_HEAD, H_HEAD = 8192, 8192


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def _traffic_from_profiles(key: str):
    """DRAM bytes per launch of the dominant kernel, from the committed ncu
    summary (profiles/*.md lines of the form `traffic_bytes_per_launch[key]: N`)."""
    d = os.path.join(ROOT, "profiles")
    if not os.path.isdir(d):
        return None
    for fn in sorted(os.listdir(d)):
        if not fn.endswith((".md", ".txt")):
            continue
        with open(os.path.join(d, fn)) as f:
            for line in f:
                tag = f"traffic_bytes_per_launch[{key}]:"
                if line.strip().startswith(tag):
                    try:
                        return int(float(line.split(":", 1)[1].strip().split()[0]))
                    except ValueError:
                        return None
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled in the background."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.proc = None
        self.gpu = gpu_index
        self.path = os.path.join("/tmp", f"satgb_clocks_{os.getpid()}.csv")

    def start(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons, n = [], [], set(), 0
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax.append(float(parts[2]))
                except ValueError:
                    continue
                n += 1
                for nm, v in zip(names, parts[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(nm)
        try:
            os.remove(self.path)
        except OSError:
            pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": n}


def max_over_ranks(ms: float, device) -> float:
    """The slowest rank's time (replicas: every rank processes its own image)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(world: int, steps: int, step_bytes: int, total_ms: float) -> float:
    """Whole-job GB/s: every rank's steps over the slowest rank's time."""
    return world * steps * step_bytes / (total_ms / 1e3) / GB


def _time_steps(fn, steps, warmup, stream, min_warm_s=1.0):
    """W untimed warm-up steps (at least min_warm_s of work, so the clock
    sampler sees the GPU under load), then exactly `steps` timed steps with
    one CUDA event pair per step on `stream`.  Returns (total_ms, per_step_ms)."""
    import torch
    t0 = time.time()
    i = 0
    while i < warmup or time.time() - t0 < min_warm_s:
        fn()
        i += 1
        if i % 50 == 0:
            stream.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    torch.cuda.synchronize()
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    start.record(stream)
    for k in range(steps):
        ev[k][0].record(stream)
        fn()
        ev[k][1].record(stream)
    end.record(stream)
    torch.cuda.synchronize()
    per = [a.elapsed_time(b) for a, b in ev]
    return start.elapsed_time(end), per


def run_gpu(args):
    import numpy as np
    import torch

    import sat_gb300

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream()
    sat_gb300._lib.load()

    peak, peak_kind = _peaks()
    g = torch.Generator(device=dev)
    g.manual_seed(1234 + rank)

    # ---- headline: f32 8192^2 plain -------------------------------------------
    x = torch.rand((H_HEAD, W_HEAD), dtype=torch.float32, device=dev, generator=g)
    y = torch.empty_like(x)
    step_bytes = x.numel() * 8
    sampler = ClockSampler(local)
    if rank == 0:
        sampler.start()
    l0 = sat_gb300.launch_count()

    def headline():
        sat_gb300.sat(x, torch.float32, out=y)

    # barrier + sync on both sides of the timed region, max over ranks
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    total_ms, per = _time_steps(headline, args.steps, args.warmup, stream)
    launches = sat_gb300.launch_count() - l0
    sat_gb300.stream_check()
    if world > 1:
        total_ms = max_over_ranks(total_ms, dev)
        torch.distributed.barrier()
    clocks = sampler.stop() if rank == 0 else None
    timed_launches = args.steps  # one launch per step
    warm_launches = launches - timed_launches
    value = replica_throughput(world, args.steps, step_bytes, total_ms)
    avg_launch_ms = statistics.mean(per)
    achieved = step_bytes / (avg_launch_ms / 1e3) / GB

    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return

    sub = {}
    # ---- u8 -> u32 8192^2 -------------------------------------------------------
    xb = torch.randint(0, 256, (H_HEAD, W_HEAD), dtype=torch.uint8, device=dev, generator=g)
    yb = torch.empty((H_HEAD, W_HEAD), dtype=torch.uint32, device=dev)
    ms, per_b = _time_steps(lambda: sat_gb300.scanrow_brlt(xb, torch.uint32, out=yb), 50, 5, stream, 0.2)
    bb = xb.numel() * 5
    sub["u8_u32_8192"] = {"gbs": round(bb / (statistics.median(per_b) / 1e3) / GB, 1),
                          "ms_median": round(statistics.median(per_b), 4)}
    sub["u8_u32_8192"]["frac_of_peak"] = round(sub["u8_u32_8192"]["gbs"] / peak, 4)
    # ---- compensated f32 8192^2 -------------------------------------------------
    ms, per_c = _time_steps(lambda: sat_gb300.sat(x, torch.float32, mode="compensated", out=y), 50, 5, stream, 0.2)
    ms, per_p = _time_steps(headline, 50, 5, stream, 0.2)
    sub["f32_compensated_8192"] = {"gbs": round(step_bytes / (statistics.median(per_c) / 1e3) / GB, 1),
                                   "ms_median": round(statistics.median(per_c), 4),
                                   "time_ratio_vs_plain": round(statistics.median(per_c) / statistics.median(per_p), 3)}
    # ---- f64 4096^2 ---------------------------------------------------------------
    xd = torch.rand((4096, 4096), dtype=torch.float64, device=dev, generator=g)
    yd = torch.empty_like(xd)
    ms, per_d = _time_steps(lambda: sat_gb300.sat(xd, torch.float64, out=yd), 50, 5, stream, 0.2)
    sub["f64_4096"] = {"gbs": round(xd.numel() * 16 / (statistics.median(per_d) / 1e3) / GB, 1),
                       "ms_median": round(statistics.median(per_d), 4)}
    sat_gb300.stream_check()
    # ---- row-only and column-only scans (ScanX / ScanY), f32 8192^2 --------------
    for nm, fn in (("scan_rows_f32_8192", sat_gb300.scan_rows), ("scan_cols_f32_8192", sat_gb300.scan_cols),
                   ("scan_rows_transposed_f32_8192", sat_gb300.scan_rows_transposed)):
        ms, per_s = _time_steps(lambda: fn(x, torch.float32, out=y), 50, 5, stream, 0.2)
        sub[nm] = {"gbs": round(step_bytes / (statistics.median(per_s) / 1e3) / GB, 1),
                   "ms_median": round(statistics.median(per_s), 4)}
        sub[nm]["frac_of_peak"] = round(sub[nm]["gbs"] / peak, 4)
    # the transposed row scan of u8 -> u32 (5 bytes a pixel; square, so yb takes the transpose)
    ms, per_s = _time_steps(lambda: sat_gb300.scan_rows_transposed(xb, torch.uint32, out=yb), 50, 5, stream, 0.2)
    nm = "scan_rows_transposed_u8_u32_8192"
    sub[nm] = {"gbs": round(xb.numel() * 5 / (statistics.median(per_s) / 1e3) / GB, 1),
               "ms_median": round(statistics.median(per_s), 4)}
    sub[nm]["frac_of_peak"] = round(sub[nm]["gbs"] / peak, 4)
    sat_gb300.stream_check()
    del xb, yb, xd, yd
    if not args.no_extra:
        sub["batch512_u8_u32"] = batch_result(dev, stream, peak)
        torch.cuda.empty_cache()
        sub["batch512_u8_u32_packed"] = batch_result(dev, stream, peak, pitched=False)
        torch.cuda.empty_cache()
        sub["box_filter_64x3x1024"] = box_result(dev, stream)
        torch.cuda.empty_cache()
        sub.update(stress_result(dev, stream, peak))
        torch.cuda.empty_cache()
        sub["reference_gpu_8192"] = reference_gpu_result()

    # ---- e2e: the same headline SAT through the public API with host buffers ----
    # Every step copies its input from pinned host memory, runs the SAT and
    # copies the result back.  Steps alternate between two streams and two sets
    # of buffers (double buffering, as a serving loop would), so one step's
    # device-to-host copy overlaps the next step's host-to-device copy.
    e2e_steps = max(4, min(args.steps, 20))
    hx = torch.empty((H_HEAD, W_HEAD), dtype=torch.float32, pin_memory=True)
    hx.copy_(x.cpu())
    hy = [torch.empty((H_HEAD, W_HEAD), dtype=torch.float32, pin_memory=True) for _ in range(2)]
    dx = [torch.empty_like(x) for _ in range(2)]
    dy = [torch.empty_like(x) for _ in range(2)]
    streams = [torch.cuda.Stream(device=dev) for _ in range(2)]

    def e2e_step(k):
        st = streams[k % 2]
        with torch.cuda.stream(st):
            dx[k % 2].copy_(hx, non_blocking=True)
            sat_gb300.sat(dx[k % 2], torch.float32, out=dy[k % 2], stream=st)
            hy[k % 2].copy_(dy[k % 2], non_blocking=True)

    for k in range(4):  # warm-up (workspaces of both streams)
        e2e_step(k)
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(streams[0])
    streams[1].wait_event(ev0)
    for k in range(e2e_steps):
        e2e_step(k)
    done1 = torch.cuda.Event()
    done1.record(streams[1])
    streams[0].wait_event(done1)
    ev1.record(streams[0])
    torch.cuda.synchronize()
    sat_gb300.stream_check(streams[0])
    sat_gb300.stream_check(streams[1])
    ms_e2e = ev0.elapsed_time(ev1)
    e2e = {"value": round(e2e_steps * step_bytes / (ms_e2e / 1e3) / GB, 2), "unit": "GB/s",
           "h2d_bytes_per_step": int(hx.numel() * 4), "d2h_bytes_per_step": int(hy[0].numel() * 4),
           "steps": e2e_steps, "pipelining": "two streams, double-buffered"}
    del hx, hy, dx, dy

    # ---- CPU baseline: the reference's IntegralImageParallel (oracle port) -----
    cpu = cpu_baseline(args.cpu_seconds)

    out = {
        "metric": "SAT GB/s (in+out bytes), f32 8192x8192 plain; % of measured HBM copy bandwidth in roofline.frac",
        "value": round(value, 1),
        "unit": "GB/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(total_ms / args.steps, 5),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic: torch.rand uniform [0,1) f32 (seeded); inputs and outputs 256 MiB each, larger than L2, no flush",
        "config": {"workload": "f32->f32 plain SAT, one 8192x8192 image per step",
                   "width": W_HEAD, "height": H_HEAD, "in_dtype": "f32", "out_dtype": "f32",
                   "l2": "inputs larger than L2 (no flush)", "parallelism": f"replicas{world}"},
        "e2e": e2e,
        "gpu_launches": int(timed_launches),
        "warmup_launches": int(warm_launches),
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "peak_kind": peak_kind,
                     "traffic": _traffic_from_profiles("f32_f32_8192_ws"),
                     "algorithmic_bytes_per_launch": step_bytes,
                     "kernel": "satgb::sat_tile_kernel_ws<float,float,float,fwd> (128-row tiles, direct stores)"},
        "cpu_baseline": cpu,
        "clocks": clocks,
        "sub_results": sub,
    }
    print(json.dumps(out))
    if world > 1:
        torch.distributed.destroy_process_group()


def cpu_model() -> str:
    """The host CPU's model name (lscpu, else /proc/cpuinfo), for the baseline's record."""
    import subprocess
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith("model name"):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


def cpu_baseline(seconds: float):
    """The reference's CPU integral image on the headline workload: the
    restatement of IntegralImageParallel (OpenMP over all host cores),
    repeated for about `seconds` of CPU time, and IntegralImageSerial on one
    core, a bounded sample of whole images."""
    import numpy as np
    from oracle import oracle as O
    O.build(with_ref=False)
    n = os.cpu_count() or 1
    a = O.gen("f32u", 1, (H_HEAD, W_HEAD))
    O.sat_parallel(a, np.float32, nthreads=n)  # warm
    t0 = time.time()
    reps = 0
    while True:
        O.sat_parallel(a, np.float32, nthreads=n)
        reps += 1
        if time.time() - t0 >= seconds:
            break
    dt = (time.time() - t0) / reps
    t0 = time.time()
    sreps = 0
    while True:
        O.sat_serial(a, np.float32)
        sreps += 1
        if time.time() - t0 >= min(seconds, 3.0):
            break
    sdt = (time.time() - t0) / sreps
    return {"value": round(a.size * 8 / dt / GB, 3), "unit": "GB/s", "cores": n, "kind": "port",
            "sample": f"{reps} full 8192x8192 f32 SATs with IntegralImageParallel (row pass then column pass), {n} OpenMP threads",
            "serial_1core": {"value": round(a.size * 8 / sdt / GB, 3), "unit": "GB/s", "cores": 1,
                             "sample": f"{sreps} full 8192x8192 f32 SATs with IntegralImageSerial"},
            "cpu_model": cpu_model()}


def run_reference(args):
    """Reference arm: the reference's CPU integral image on this host."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import numpy as np
    from oracle import oracle as O
    O.build(with_ref=False)
    n = os.cpu_count() or 1
    a = O.gen("f32u", 1, (H_HEAD, W_HEAD))
    for _ in range(args.warmup):
        O.sat_parallel(a, np.float32, nthreads=n)
    t0 = time.time()
    for _ in range(args.steps):
        O.sat_parallel(a, np.float32, nthreads=n)
    dt = time.time() - t0
    value = args.steps * a.size * 8 / dt / GB
    out = {
        "impl": "reference",
        "metric": "SAT GB/s (in+out bytes), f32 8192x8192 plain; % of measured HBM copy bandwidth in roofline.frac",
        "value": round(value, 3), "unit": "GB/s", "n_gpus": int(os.environ.get("WORLD_SIZE", "1")),
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(dt / args.steps * 1e3, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic: splitmix64 uniform [0,1) f32 (seeded)",
        "config": {"workload": "f32->f32 plain SAT, one 8192x8192 image per step",
                   "width": W_HEAD, "height": H_HEAD, "in_dtype": "f32", "out_dtype": "f32"},
        "cpu_baseline": {"value": round(value, 3), "unit": "GB/s", "cores": n, "kind": "port",
                         "sample": f"each step one full 8192x8192 f32 IntegralImageParallel (oracle restatement), {n} OpenMP threads"},
        "e2e": {"value": round(value, 3), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))


CASES = {
    # name: (in dtype, out dtype, mode, reverse, height, width)
    "f32_8192": ("float32", "float32", "plain", False, 8192, 8192),
    "f32c_8192": ("float32", "float32", "compensated", False, 8192, 8192),
    "u8_8192": ("uint8", "uint32", "plain", False, 8192, 8192),
    "u8_2048": ("uint8", "uint32", "plain", False, 2048, 2048),
    "u8_4096": ("uint8", "uint32", "plain", False, 4096, 4096),
    "u8_16384": ("uint8", "uint32", "plain", False, 16384, 16384),
    "u8_32768": ("uint8", "uint32", "plain", False, 32768, 32768),
    "u8r_8192": ("uint8", "uint32", "plain", True, 8192, 8192),
    "f64_4096": ("float64", "float64", "plain", False, 4096, 4096),
    "f32r_8192": ("float32", "float32", "plain", True, 8192, 8192),
    "f32_1024": ("float32", "float32", "plain", False, 1024, 1024),
    "f32_2048": ("float32", "float32", "plain", False, 2048, 2048),
    "f32_4096": ("float32", "float32", "plain", False, 4096, 4096),
    "f32_16384": ("float32", "float32", "plain", False, 16384, 16384),
    "u8_1024": ("uint8", "uint32", "plain", False, 1024, 1024),
    "f32c_2048": ("float32", "float32", "compensated", False, 2048, 2048),
    "f32c_16384": ("float32", "float32", "compensated", False, 16384, 16384),
    "f32t_8192": ("float32", "float32", "rows_transposed", False, 8192, 8192),
    "u8t_8192": ("uint8", "uint32", "rows_transposed", False, 8192, 8192),
    "f32rows_8192": ("float32", "float32", "rows", False, 8192, 8192),
    "u8rows_8192": ("uint8", "uint32", "rows", False, 8192, 8192),
    "f32cols_8192": ("float32", "float32", "cols", False, 8192, 8192),
}


def run_case(args):
    """A few launches of one workload (for ncu captures and quick timing):
    `--steps` timed launches after `--warmup` untimed ones, median printed."""
    import torch

    import sat_gb300
    ti, to, mode, rev, h, w = CASES[args.case]
    if args.config >= 0:
        sat_gb300.set_config(args.config)
    dev = torch.device("cuda", 0)
    g = torch.Generator(device=dev)
    g.manual_seed(7)
    tin, tout = getattr(torch, ti), getattr(torch, to)
    if tin.is_floating_point:
        x = torch.rand((h, w), dtype=tin, device=dev, generator=g)
    else:
        x = torch.randint(0, 256, (h, w), dtype=tin, device=dev, generator=g)
    y = torch.empty((h, w), dtype=torch.int32 if tout == torch.uint32 else tout, device=dev)
    if tout == torch.uint32:
        y = y.view(torch.uint32)
    stream = torch.cuda.current_stream()
    if mode == "rows_transposed":
        y = y.t().contiguous() if h != w else y
        fn = lambda: sat_gb300.scan_rows_transposed(x, tout, out=y)
    elif mode in ("rows", "cols"):
        scan = sat_gb300.scan_rows if mode == "rows" else sat_gb300.scan_cols
        fn = lambda: scan(x, tout, out=y)
    else:
        fn = lambda: sat_gb300.sat(x, tout, mode=mode, reverse=rev, out=y)
    total, per = _time_steps(fn, args.steps, args.warmup, stream, 0.0)
    sat_gb300.stream_check()
    nbytes = x.numel() * (x.element_size() + y.element_size())
    med = statistics.median(per)
    print(json.dumps({"case": args.case, "config": args.config, "ms_median": round(med, 5), "gbs": round(nbytes / (med / 1e3) / GB, 1),
                      "launches": args.steps + args.warmup}))


def _log_uniform_sizes(n, lo, hi, seed):
    import numpy as np
    rng = np.random.default_rng(seed)
    e = rng.uniform(np.log(lo), np.log(hi), size=(n, 2))
    return [(int(round(np.exp(a))), int(round(np.exp(b)))) for a, b in e]  # (width, height)


def _pitched(h, w, dtype, dev, row_align=128):
    """An (h, w) view whose rows start every `row_align` bytes, as a pitched
    allocation (the reference's GpuData, cudaMalloc3D) lays them out."""
    import torch
    esz = torch.empty((), dtype=dtype).element_size()
    pitch = -(-w * esz // row_align) * row_align // esz
    base_dt = torch.int32 if dtype == torch.uint32 else dtype
    base = torch.empty((h, pitch), dtype=base_dt, device=dev)
    if dtype == torch.uint32:
        base = base.view(torch.uint32)
    return base[:, :w]


def build_batch(dev, seed=512, pitched=True):
    """512 u8 images, width and height independently log-uniform in
    [64, 4096], u8 -> u32 outputs; rows pitched to 128 bytes, or packed."""
    import torch
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    sizes = _log_uniform_sizes(512, 64, 4096, seed)
    xs, ys = [], []
    for w, h in sizes:
        v = torch.randint(0, 256, (h, w), dtype=torch.uint8, device=dev, generator=g)
        if pitched:
            x = _pitched(h, w, torch.uint8, dev)
            x.copy_(v)
            xs.append(x)
            ys.append(_pitched(h, w, torch.uint32, dev))
        else:
            xs.append(v)
            ys.append(torch.empty((h, w), dtype=torch.int32, device=dev).view(torch.uint32))
    nbytes = sum(w * h * 5 for w, h in sizes)
    return xs, ys, nbytes


def batch_result(dev, stream, peak, pitched=True):
    """The batch workload as one graph replay of a persistent launch, against
    the same images as 512 per-image calls."""
    import torch

    import sat_gb300
    xs, ys, nbytes = build_batch(dev, pitched=pitched)
    plan = sat_gb300.BatchPlan(xs, ys, stream=stream)
    _, per_u = _time_steps(lambda: plan.exec(stream), 10, 3, stream, 0.1)
    untuned = [c["config"] for c in plan.classes()]
    plan.autotune(stream)
    _, per_g = _time_steps(lambda: plan.exec(stream), 20, 3, stream, 0.2)
    plan.check(stream)

    def per_image():
        for a, b in zip(xs, ys):
            sat_gb300.sat(a, torch.uint32, out=b)

    _, per_i = _time_steps(per_image, 5, 2, stream, 0.0)
    sat_gb300.stream_check()
    gm, im = statistics.median(per_g), statistics.median(per_i)
    res = {"images": len(xs), "bytes": int(nbytes), "graph_ms": round(gm, 4),
           "graph_gbs": round(nbytes / (gm / 1e3) / GB, 1), "frac_of_peak": round(nbytes / (gm / 1e3) / GB / peak, 4),
           "per_image_ms": round(im, 4), "per_image_gbs": round(nbytes / (im / 1e3) / GB, 1),
           "tiles": plan.info()["n_tiles"], "rows": "pitched to 128 B" if pitched else "packed",
           "classes": plan.classes(), "untuned_configs": untuned,
           "untuned_graph_gbs": round(nbytes / (statistics.median(per_u) / 1e3) / GB, 1)}
    plan.close()
    return res


def build_box(dev, n=64, c=3, h=1024, w=1024, radii=(3, 7, 15), seed=99):
    """The box-filter layer workload: f32 N(0,1) of shape (n, c, h, w), box
    means for three radii, gradient W ~ N(0,1) of the means' shape."""
    import torch
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    x = torch.randn((n, c, h, w), dtype=torch.float32, device=dev, generator=g)
    wts = torch.randn((n, c, len(radii), h, w), dtype=torch.float32, device=dev, generator=g)
    return x, wts, radii


def box_result(dev, stream):
    """Forward (SAT + box means) against forward + backward (dL/dmeans = W,
    adjoint gather + reverse SAT) of the box-filter layer."""
    import torch

    import sat_gb300
    x, wts, radii = build_box(dev)
    xg = x.clone().requires_grad_(True)

    def fwd():
        with torch.no_grad():
            sat_gb300.box_filter_means(x, radii)

    def fwd_bwd():
        xg.grad = None
        m = sat_gb300.box_filter_means(xg, radii)
        m.backward(wts)

    _, per_f = _time_steps(fwd, 10, 3, stream, 0.2)
    _, per_fb = _time_steps(fwd_bwd, 10, 3, stream, 0.2)
    sat_gb300.stream_check()
    f, fb = statistics.median(per_f), statistics.median(per_fb)
    sat_bytes = x.numel() * 8
    return {"shape": list(x.shape), "radii": list(radii), "fwd_ms": round(f, 4), "fwd_bwd_ms": round(fb, 4),
            "fwd_bwd_over_fwd": round(fb / f, 3), "forward_sat_bytes": int(sat_bytes)}


def reference_gpu_result(size=8192, reps=20):
    """The reference's own GPU kernels (its three two-launch algorithms, built
    from its sources for sm_103a by baseline/build_ref_gpu.sh into
    baseline/_ref/*.cubin) timed on this GPU by baseline/ref_gpu_bench.cu
    with the reference's launch shapes, each result checked on the host.
    Reported beside this library's figures; never part of the library."""
    ref = os.path.join(ROOT, "baseline", "_ref")
    cubins = ("ScanRow-BRLT.cubin", "BRLT-Scan.cubin", "ScanRowColumn.cubin")
    if not all(os.path.isfile(os.path.join(ref, c)) for c in cubins):
        return {"unavailable": "the reference's kernels were not built here (baseline/build_ref_gpu.sh needs the "
                               "reference sources)"}
    exe = os.path.join(ref, "ref_gpu_bench")
    src = os.path.join(ROOT, "baseline", "ref_gpu_bench.cu")
    from sat_gb300 import build as B
    r = subprocess.run([B.nvcc_path(), "-O2", "-std=c++17", "-o", exe, src, "-lcuda"], capture_output=True, text=True)
    if r.returncode != 0:
        return {"unavailable": "harness build failed: " + r.stderr.strip().splitlines()[-1] if r.stderr else "?"}
    r = subprocess.run([exe, ref, str(size), str(reps)], capture_output=True, text=True, timeout=600)
    if r.returncode != 0:
        return {"unavailable": "harness failed: " + (r.stderr.strip().splitlines() or ["?"])[-1]}
    res = {}
    for line in r.stdout.splitlines():
        if line.startswith("{"):
            d = json.loads(line)
            res[f"{d['algorithm']} {d['pair']}"] = {k: d[k] for k in ("ms_median", "gbs", "correct", "launches")}
    return res


def stress_result(dev, stream, peak):
    """32768^2 u8 -> u32 (wrapping mod 2^32) and 16384^2 f32 compensated."""
    import torch

    import sat_gb300
    res = {}
    g = torch.Generator(device=dev)
    g.manual_seed(5)
    xb = torch.randint(0, 256, (32768, 32768), dtype=torch.uint8, device=dev, generator=g)
    yb = torch.empty((32768, 32768), dtype=torch.int32, device=dev).view(torch.uint32)
    _, per = _time_steps(lambda: sat_gb300.sat(xb, torch.uint32, out=yb), 5, 3, stream, 0.0)
    nb = xb.numel() * 5
    res["u8_u32_32768"] = {"ms_median": round(statistics.median(per), 4),
                           "gbs": round(nb / (statistics.median(per) / 1e3) / GB, 1)}
    del xb, yb
    xf = torch.rand((16384, 16384), dtype=torch.float32, device=dev, generator=g)
    yf = torch.empty_like(xf)
    _, per = _time_steps(lambda: sat_gb300.sat(xf, torch.float32, mode="compensated", out=yf), 10, 3, stream, 0.0)
    nb = xf.numel() * 8
    res["f32_compensated_16384"] = {"ms_median": round(statistics.median(per), 4),
                                    "gbs": round(nb / (statistics.median(per) / 1e3) / GB, 1)}
    sat_gb300.stream_check()
    for v in res.values():
        v["frac_of_peak"] = round(v["gbs"] / peak, 4)
    return res


def run_workload(args):
    """Short runs of the non-SAT workloads (for ncu captures and quick timing)."""
    import torch

    import sat_gb300
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream()
    if args.case in ("batch512", "batch512_packed"):
        if args.config >= 0:
            sat_gb300.set_config(args.config)
        xs, ys, nbytes = build_batch(dev, pitched=args.case == "batch512")
        plan = sat_gb300.BatchPlan(xs, ys, stream=stream)
        if args.tune:
            plan.autotune(stream)
        _, per = _time_steps(lambda: plan.exec(stream), args.steps, args.warmup, stream, 0.0)
        plan.check(stream)
        med = statistics.median(per)
        print(json.dumps({"case": args.case, "config": plan.info()["config"], "tiles": plan.info()["n_tiles"],
                          "classes": plan.classes(), "ms_median": round(med, 5),
                          "gbs": round(nbytes / (med / 1e3) / GB, 1)}))
    elif args.case in ("box_fwd", "box_fwdbwd"):
        n = 8 if args.small else 64
        x, wts, radii = build_box(dev, n=n)
        xg = x.clone().requires_grad_(True)

        def step():
            if args.case == "box_fwd":
                with torch.no_grad():
                    sat_gb300.box_filter_means(x, radii)
            else:
                xg.grad = None
                sat_gb300.box_filter_means(xg, radii).backward(wts)

        _, per = _time_steps(step, args.steps, args.warmup, stream, 0.0)
        sat_gb300.stream_check()
        print(json.dumps({"case": args.case, "n": n, "ms_median": round(statistics.median(per), 5)}))
    elif args.case == "box_parts":
        # the four launches of the box-filter layer's forward + backward, each timed alone, and the
        # one-call backward (adjoint into the output, reverse SAT in place) that makes the last two
        from sat_gb300 import api
        n = 8 if args.small else 64
        x, wts, radii = build_box(dev, n=n)
        s = api.sat(x, torch.float32)
        gs = api.box_means_adjoint(wts, radii)
        parts = {"sat": lambda: api.sat(x, torch.float32, out=s),
                 "box_means": lambda: api.box_means_from_sat(s, radii),
                 "adjoint": lambda: api.box_means_adjoint(wts, radii, out=gs),
                 "reverse_sat": lambda: api.sat(gs, torch.float32, reverse=True, out=gs),
                 "grad_x": lambda: api.box_means_grad_x(wts, radii, out=gs)}
        plane = x.numel() * 4
        moved = {"sat": 2 * plane, "box_means": (1 + len(radii)) * plane, "adjoint": (len(radii) + 1) * plane,
                 "reverse_sat": 2 * plane, "grad_x": (len(radii) + 3) * plane}
        res = {"case": args.case, "n": n}
        for name, fn in parts.items():
            _, per = _time_steps(fn, args.steps, args.warmup, stream, 0.0)
            med = statistics.median(per)
            res[name] = {"ms_median": round(med, 4), "gbs": round(moved[name] / (med / 1e3) / GB, 1)}
        sat_gb300.stream_check()
        print(json.dumps(res))


WORKLOADS = ("batch512", "batch512_packed", "box_fwd", "box_fwdbwd", "box_parts")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--case", default=None, choices=sorted(CASES) + list(WORKLOADS))
    ap.add_argument("--small", action="store_true", help="box workloads: 8 images instead of 64")
    ap.add_argument("--no-extra", action="store_true", help="skip the batch, box-filter and stress sub-results")
    ap.add_argument("--config", type=int, default=-1, help="force a tile configuration (--case only)")
    ap.add_argument("--tune", action="store_true", help="batch cases: run the batch autotuner first")
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    args = ap.parse_args()
    if args.warmup < 3 and not args.case:
        args.warmup = 3
    if args.case:
        from sat_gb300 import build as B
        B.build()
        run_workload(args) if args.case in WORKLOADS else run_case(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        from sat_gb300 import build as B
        B.build()
        run_gpu(args)


if __name__ == "__main__":
    main()
