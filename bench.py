"""Benchmark of the GB300 Signalsmith-FFT transform path.

Default workload (the batched RealFFT<float> configuration): N in {480, 960, 1920, 3840}, 16384
frames per size, each frame N(0,1) noise plus 3 sinusoids (seeded); one step = forward (real ->
N/2 bins, DC/Nyquist in bin 0) and inverse of every size.  Metric: GFLOP/s with 2.5 N log2 N
flops per real transform.

Reported on one JSON line:
* value        -- device-resident throughput (inputs already in HBM), CUDA events over K steps;
* e2e          -- the same work through the C ABI's host-buffer entry point ssfft_exec_host
                  (pinned host input -> device -> pinned host output, copies inside the timing);
* roofline     -- the dominant kernel's algorithmic bytes / its mean CUDA-event duration,
                  against the measured HBM copy bandwidth;
* cpu_baseline -- the reference algorithm (the C restatement in oracle/, one plan per thread) on
                  all host cores over the same frames.
`--impl reference` times that CPU implementation alone, as the reference arm.

Multi-GPU: every rank runs an independent replica of the workload (the transforms are
independent; there is no exchange step), `value` sums all ranks' work over the slowest rank.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "batched+served FFT GFLOP/s, p99 lat vs plain GPU FFT @ relL2≤1e-6 (FP32)"
SIZES = (480, 960, 1920, 3840)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--frames", type=int, default=16384)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--e2e-steps", type=int, default=0, help="steps of the host-buffer leg (default: steps/10)")
    ap.add_argument("--workload", default="realfft",
                    choices=["realfft", "fp64", "large", "serve", "served", "uneven", "precision", "sizes", "dropin",
                             "uneven_class", "uneven_members"],
                    help="realfft: the batched RealFFT<float> line (default); fp64: FFT<double> N=1024 x256; "
                         "large: single FP32 transforms of 2^24, 3^15, 2^12 3^4 5^2; serve: request serving sweep; "
                         "served: the default line's served block alone; "
                         "sizes: per-size batched FP32 kernel sweep (--sizes, --kinds, --sweep-mb, --plan-options)")
    ap.add_argument("--sizes", default="256,512,1024,2048,4096,8192,16384",
                    help="sizes workload: comma-separated transform lengths")
    ap.add_argument("--kinds", default="complex,real", help="sizes workload: complex and/or real")
    ap.add_argument("--sweep-mb", type=int, default=512, help="sizes workload: MiB of input + output per launch")
    ap.add_argument("--plan-options", default="{}", help="sizes workload: JSON keyword options of fft_gb300.Plan")
    ap.add_argument("--serve-duration", type=float, default=3.0)
    ap.add_argument("--passes", type=int, default=0,
                    help="passes of the workload per timed step (0: enough for a timed region of >= --min-timed-s)")
    ap.add_argument("--min-timed-s", type=float, default=1.5,
                    help="default line: the timed region lasts at least this long (clock samples under load)")
    ap.add_argument("--no-served", action="store_true", help="default line: skip the served block")
    ap.add_argument("--no-uneven", action="store_true", help="default line: skip the uneven-batch block")
    ap.add_argument("--served-duration", type=float, default=1.0,
                    help="default line: seconds of offered load per point of the served sweep")
    ap.add_argument("--queue-mode", default="queue", choices=["queue", "pergraph"],
                    help="uneven_class workload: one queue-class launch or one launch per size")
    ap.add_argument("--members", type=int, default=16, help="uneven_members workload: sizes in the class")
    ap.add_argument("--uneven-reps", type=int, default=0, help="uneven workload: timed submissions (0: auto)")
    ap.add_argument("--serve-waves", type=int, default=8, help="batched server: waves in flight")
    ap.add_argument("--serve-wave-requests", type=int, default=256, help="batched server: requests per wave")
    ap.add_argument("--uneven-fp32-only", action="store_true", help="uneven workload: skip the split-BF16 variant")
    ap.add_argument("--frames-total", type=int, default=4000, help="uneven_members workload: transforms in all")
    ap.add_argument("--cpu-seconds", type=float, default=10.0,
                    help="CPU baseline: seconds of CPU work in the bounded sample")
    ap.add_argument("--tune", type=int, default=2, choices=[0, 1, 2],
                    help="autotune level of the plans (0 planner defaults, 1 CTA shape, 2 also radix order)")
    ap.add_argument("--streams", type=int, default=4,
                    help="run each size's forward->inverse chain on its own stream (1..4)")
    return ap.parse_args()


def frames_for(n: int, frames: int, seed: int) -> np.ndarray:
    """Gaussian N(0,1) noise + 3 sinusoids per frame: frequency U(0, n/2), amplitude U[0.1, 2],
    phase U[0, 2 pi)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    x = rng.standard_normal((frames, n), dtype=np.float32)
    t = np.arange(n, dtype=np.float32)
    for _ in range(3):
        f = rng.uniform(0, n / 2, (frames, 1)).astype(np.float32)
        a = rng.uniform(0.1, 2, (frames, 1)).astype(np.float32)
        ph = rng.uniform(0, 2 * np.pi, (frames, 1)).astype(np.float32)
        x += a * np.sin(2 * np.pi * f * t / n + ph)
    return x


def flops_per_step(frames: int) -> float:
    return sum(2 * frames * 2.5 * n * math.log2(n) for n in SIZES)


class ClockSampler:
    """nvidia-smi samples every 100 ms while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.dev = device_index
        self.proc = None
        self.lines: list[str] = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def parse_cpulist(txt: str) -> set:
    """CPU numbers of a sysfs CPU list ("0-3,8,10-11")."""
    cpus = set()
    for part in txt.strip().split(","):
        if "-" in part:
            a, b = part.split("-")
            cpus.update(range(int(a), int(b) + 1))
        elif part:
            cpus.add(int(part))
    return cpus


def gpu_local_cpus(device_index: int):
    """The CPUs of the host node the GPU is attached to (its PCI function's `local_cpulist` in
    sysfs) that this process may run on, or None when that is unknown or every CPU."""
    try:
        import torch
        pr = torch.cuda.get_device_properties(device_index)
        dev = "%04x:%02x:%02x.0" % (pr.pci_domain_id, pr.pci_bus_id, pr.pci_device_id)
        with open(f"/sys/bus/pci/devices/{dev}/local_cpulist") as f:
            cpus = parse_cpulist(f.read())
    except Exception:
        return None
    mine = os.sched_getaffinity(0)
    usable = cpus & mine
    return usable if usable and usable != mine else None


class HostAffinity:
    """Runs the host-buffer legs (pinned buffers, copy threads, the request server) on the CPUs
    local to the GPU, so that page-locked buffers are allocated in the memory next to it; the
    calling thread's affinity is restored on exit (the CPU baseline keeps every core)."""

    def __init__(self, device_index: int):
        self.cpus = gpu_local_cpus(device_index)
        self.old = None

    def note(self) -> str:
        return f"{len(self.cpus)} CPUs local to the GPU" if self.cpus else "not bound (no local CPU list, or all CPUs)"

    def __enter__(self):
        if self.cpus:
            self.old = os.sched_getaffinity(0)
            os.sched_setaffinity(0, self.cpus)
        return self

    def __exit__(self, *exc):
        if self.old:
            os.sched_setaffinity(0, self.old)
        return False


def measured_peak_hbm() -> tuple[float, str]:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def max_over_ranks(seconds: float, dist=None, device: str = "cpu") -> float:
    """The slowest rank's time (replicas: the job ends when the last rank does)."""
    if dist is None:
        return seconds
    import torch
    t = torch.tensor([seconds], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def traffic_for(kernel: str):
    """DRAM bytes per launch (read + write) of `kernel` from the committed ncu launch-list
    summary (its table's last column), if the kernel is listed there."""
    p = os.path.join(ROOT, "profiles", "realfft_f32_launches_16384frames.md")
    try:
        with open(p) as f:
            for line in f:
                cells = [c.strip() for c in line.strip().strip("|").split("|")]
                if cells and cells[0] == kernel:
                    return float(cells[-1])
    except (OSError, ValueError):
        pass
    return None


CPU_KIND = "port_native"  # the oracle's C restatement built -O3 with the host's vector ISA (timing only)


_CPU_DATA: dict = {}


def cpu_leg(frames: int, threads: int, kind: str = CPU_KIND, seed: int = 7, min_seconds: float = 0.0) -> dict:
    """Time the reference algorithm on the host cores: forward + inverse of every size over
    `frames` frames, one plan instance per thread; repeated until `min_seconds` of work."""
    import oracle
    key = (frames, seed)
    if key not in _CPU_DATA:  # the same frames for every step of a run (generating them costs more than a step)
        _CPU_DATA.clear()
        _CPU_DATA[key] = [(n, frames_for(n, frames, seed + i), np.empty((frames, n // 2), dtype=np.complex64),
                           np.empty((frames, n), dtype=np.float32)) for i, n in enumerate(SIZES)]
    data = _CPU_DATA[key]
    total_t, total_f, reps = 0.0, 0.0, 0
    while True:
        for n, x, spec, back in data:
            t0 = time.perf_counter()
            oracle.batch(x, n, real=True, inverse=False, threads=threads, out=spec, kind=kind)
            oracle.batch(spec, n, real=True, inverse=True, threads=threads, out=back, kind=kind)
            total_t += time.perf_counter() - t0
            total_f += 2 * frames * 2.5 * n * math.log2(n)
        reps += 1
        if total_t >= min_seconds:
            break
    return {"gflops": total_f / total_t / 1e9, "seconds": total_t, "reps": reps}


def cpu_build_note() -> str:
    import oracle
    return f"oracle/ssfft_oracle.c built `{oracle.native_flags()}` (oracle/Makefile target native)"


def run_reference(args, rank: int, world: int):
    """The reference arm: the reference's CPU algorithm on all host threads, rank 0 only."""
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    # frames per step so that warmup + steps stay within ~2 minutes of wall time
    probe = cpu_leg(256, threads)
    per_frame = probe["seconds"] / 256
    budget = 120.0 / max(1, args.steps + args.warmup)
    frames = int(max(16, min(args.frames, budget / max(per_frame, 1e-9))))
    for _ in range(args.warmup):
        cpu_leg(frames, threads)
    t = 0.0
    for _ in range(args.steps):
        t += cpu_leg(frames, threads)["seconds"]
    value = flops_per_step(frames) * args.steps / t / 1e9
    sample = (f"{frames} frames per size per step (of {args.frames}), forward+inverse of N in {list(SIZES)}; "
              f"{cpu_build_note()}; one plan instance per thread")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "GFLOP/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "RealFFT<float> N in {480,960,1920,3840}, 16384 frames each, fwd+inv",
                   "frames": args.frames, "frames_timed_per_step": frames, "host": os.uname().machine},
        "cpu_baseline": {"value": value, "unit": "GFLOP/s", "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "GFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def e2e_leg(F, args, plans, xs, specs, backs, frames: int, world: int, dist) -> dict:
    """The same work through the C ABI's host-buffer entry point: pinned host frames -> bins ->
    host frames per size, four host threads (one per size), H2D / kernel / D2H inside the timing."""
    import torch
    from concurrent.futures import ThreadPoolExecutor
    e2e_steps = args.e2e_steps or max(3, args.steps // 10)
    hin = [torch.from_numpy(x.cpu().numpy()).pin_memory() for x in xs]
    hspec = [torch.empty(s.shape, dtype=s.dtype).pin_memory() for s in specs]
    hback = [torch.empty(b.shape, dtype=b.dtype).pin_memory() for b in backs]
    lib = F.lib()

    def chain(p, a, s, b):
        # one size: host frames -> bins -> host frames, through the C ABI's host-buffer entry point
        F.check(lib.ssfft_exec_host(p.handle, 0, a.data_ptr(), s.data_ptr()), "exec_host")
        F.check(lib.ssfft_exec_host(p.handle, 1, s.data_ptr(), b.data_ptr()), "exec_host")

    with ThreadPoolExecutor(max_workers=len(SIZES)) as pool:
        def e2e_step():
            # the sizes are independent jobs: one host thread each (distinct plans are thread-safe)
            list(pool.map(lambda args: chain(*args), zip(plans, hin, hspec, hback)))

        for _ in range(2):
            e2e_step()
        if dist:
            dist.barrier()
        te = time.perf_counter()
        for _ in range(e2e_steps):
            e2e_step()
        te = max_over_ranks(time.perf_counter() - te, dist, "cuda")
    h2d = sum(a.numel() * 4 for a in hin) + sum(s.numel() * 8 for s in hspec)
    d2h = sum(s.numel() * 8 for s in hspec) + sum(b.numel() * 4 for b in hback)
    return {"value": flops_per_step(frames) * e2e_steps * world / te / 1e9, "unit": "GFLOP/s",
            "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h), "steps": e2e_steps,
            "path": "ssfft_exec_host (pinned host buffers, 3-stream copy/compute pipeline)"}


def run_gpu(args, rank: int, world: int):
    import torch

    from fft_gb300 import build as fb
    fb.build()
    import fft_gb300 as F

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    frames = args.frames
    stream = torch.cuda.current_stream()
    sh = int(stream.cuda_stream)
    # independent size chains may run on side streams (forked from / joined to the main stream)
    nstreams = max(1, min(args.streams, len(SIZES)))
    side = [stream] + [torch.cuda.Stream() for _ in range(nstreams - 1)]
    fork_ev = torch.cuda.Event()
    join_ev = [torch.cuda.Event() for _ in side]

    # buffers and plans (outside the timed region)
    plans, xs, specs, backs = [], [], [], []
    for i, n in enumerate(SIZES):
        x = frames_for(n, frames, 1000 * rank + i)
        xs.append(torch.from_numpy(x).cuda())
        specs.append(torch.empty((frames, n // 2), dtype=torch.complex64, device="cuda"))
        backs.append(torch.empty((frames, n), dtype=torch.float32, device="cuda"))
        plans.append(F.Plan(n, "f32", "real", frames, autotune=args.tune))
    schedules = {f"N{n}": p.tuning()["choice"] for n, p in zip(SIZES, plans)}
    for n, p in zip(SIZES, plans):
        for line in p.tuning()["log"]:
            print(f"tune N={n}: {line}", file=sys.stderr)
    nl = len(SIZES) * 2

    def step():
        ns = nstreams
        if ns > 1:
            fork_ev.record(stream)
            for st in side[1:ns]:
                st.wait_event(fork_ev)
        for i, (p, x, s, b) in enumerate(zip(plans, xs, specs, backs)):
            h = int(side[i % ns].cuda_stream)
            p.exec(False, x.data_ptr(), s.data_ptr(), h)
            p.exec(True, s.data_ptr(), b.data_ptr(), h)
        if ns > 1:
            for st, ev in zip(side[1:ns], join_ev[1:ns]):
                ev.record(st)
                stream.wait_event(ev)

    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize()

    # passes per timed step: each step runs the whole workload `passes` times back to back, so
    # that the timed region lasts >= --min-timed-s and the clock sampler sees it under load
    passes = args.passes
    if passes <= 0:
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(5):
            step()
        b.record(stream)
        torch.cuda.synchronize()
        per = a.elapsed_time(b) / 1e3 / 5
        passes = max(1, math.ceil(args.min_timed_s / (per * max(1, args.steps))))
    if dist:
        pt = torch.tensor([passes], dtype=torch.int64, device="cuda")
        dist.all_reduce(pt, op=dist.ReduceOp.MAX)
        passes = int(pt.item())

    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.25)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    for k in range(args.steps):
        for _ in range(passes):
            step()
    t1.record(stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clk = clocks.stop()
    elapsed = max_over_ranks(t0.elapsed_time(t1) / 1e3, dist, "cuda")
    value = flops_per_step(frames) * passes * args.steps * world / elapsed / 1e9

    # per-kernel durations for the roofline: each kernel timed alone, CUDA events around `reps`
    # back-to-back launches of it (idempotent: same input and output), mean per launch.  The
    # launches are captured in a CUDA graph, so the gaps between them are the device's, not the
    # host's launch rate (a 14 us kernel would otherwise carry ~1 us of launch overhead each);
    # the mean over plain stream launches is reported beside it.
    reps = max(20, args.steps)
    kt = np.zeros(nl)
    kt_stream = np.zeros(nl)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    gstream = torch.cuda.Stream()
    for i, (p, x, s, b) in enumerate(zip(plans, xs, specs, backs)):
        for d, (src, dst) in enumerate(((x, s), (s, b))):
            p.exec(bool(d), src.data_ptr(), dst.data_ptr(), sh)
            ev0.record(stream)
            for _ in range(reps):
                p.exec(bool(d), src.data_ptr(), dst.data_ptr(), sh)
            ev1.record(stream)
            torch.cuda.synchronize()
            kt_stream[2 * i + d] = ev0.elapsed_time(ev1) / 1e3 / reps
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g, stream=gstream):
                gsh = int(torch.cuda.current_stream().cuda_stream)
                for _ in range(reps):
                    p.exec(bool(d), src.data_ptr(), dst.data_ptr(), gsh)
            g.replay()
            torch.cuda.synchronize()
            ev0.record(stream)
            g.replay()
            ev1.record(stream)
            torch.cuda.synchronize()
            kt[2 * i + d] = ev0.elapsed_time(ev1) / 1e3 / reps
            del g
    names, alg = [], []
    for n in SIZES:
        for d in ("r2c", "c2r"):
            names.append(f"realfft_f32_{d}_N{n}")
            alg.append(frames * 8.0 * n)  # 4N bytes in + 4N bytes out (N/2 complex) per frame
    top = int(np.argmax(kt))
    peak, peak_kind = measured_peak_hbm()
    achieved = alg[top] / kt[top] / 1e9
    kernels = {names[j]: {"ms": round(kt[j] * 1e3, 4), "GB_s": round(alg[j] / kt[j] / 1e9, 1),
                          "frac": round(alg[j] / kt[j] / 1e9 / peak, 3),
                          "ms_stream_launches": round(kt_stream[j] * 1e3, 4)} for j in range(nl)}
    agg_bytes = sum(alg)
    agg_gbs = agg_bytes / (elapsed / (args.steps * passes)) / 1e9

    # numerics of what was timed: 64 frames of every size, forward spectrum and inverse output,
    # against the FP64 oracle (relL2, the FP32 bar is 1e-6)
    import oracle
    rel_sizes = {}
    for n, x, s, b in zip(SIZES, xs, specs, backs):
        xh = x[:64].cpu().numpy().astype(np.float64)
        sref = np.stack([oracle.rfft(r) for r in xh])
        rf = float(np.linalg.norm(s[:64].cpu().numpy() - sref) / np.linalg.norm(sref))
        bref = np.stack([oracle.irfft(r.astype(np.complex128), n) for r in s[:64].cpu().numpy()])
        ri = float(np.linalg.norm(b[:64].cpu().numpy() - bref) / np.linalg.norm(bref))
        rel_sizes[f"N{n}"] = {"fwd": rf, "inv": ri}
    rel = max(max(v.values()) for v in rel_sizes.values())

    # end to end through the C ABI with pinned host buffers (on the CPUs local to the GPU)
    with HostAffinity(local) as affinity:
        e2e = e2e_leg(F, args, plans, xs, specs, backs, frames, world, dist)
        e2e["host_cpus"] = affinity.note()

    cpu = None
    if rank == 0 and not args.no_cpu:
        threads = os.cpu_count() or 1
        sample = min(frames, 4096)
        c = cpu_leg(sample, threads, min_seconds=args.cpu_seconds)
        cpu = {"value": c["gflops"], "unit": "GFLOP/s", "cores": threads, "kind": "port",
               "sample": f"{sample} frames per size x {c['reps']} repetitions, forward+inverse of N in "
                         f"{list(SIZES)} ({c['seconds']:.1f} s of CPU work on {threads} threads, one plan "
                         f"instance per thread); {cpu_build_note()}"}

    served = uneven = None
    if rank == 0 and not args.no_served:
        with HostAffinity(local) as aff:
            served = served_block(args)
            served["host_cpus"] = aff.note()
    if rank == 0 and not args.no_uneven:
        uneven = uneven_block(args, steps=50)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "GFLOP/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": elapsed / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "RealFFT<float> N in {480,960,1920,3840}, 16384 frames each, fwd+inv",
                       "frames": frames, "parallelism": f"replicas x{world}", "streams": nstreams,
                       "passes_per_step": passes,
                       "step": f"{passes} back-to-back passes of the workload (forward + inverse of every size)",
                       "timed_region_s": elapsed,
                       "l2": "each pass streams ~1.9 GB (> 129 MB L2), no flush",
                       "autotune": args.tune, "schedules": schedules},
            "gpu_launches": nl * args.steps * passes,
            "relL2_vs_fp64_oracle": rel, "relL2_per_size": rel_sizes,
            "roofline": {"bound": "hbm", "kernel": names[top], "achieved": achieved, "peak": peak,
                         "peak_source": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": traffic_for(names[top]), "alg_bytes_per_launch": alg[top],
                         "timing": "kernel alone: CUDA events around a CUDA graph of back-to-back launches of it, mean",
                         "aggregate_GB_s": agg_gbs, "aggregate_frac": agg_gbs / peak},
            "kernels": kernels,
            "e2e": e2e,
            "gpu_launches_note": "per pass: forward + inverse of each of the 4 sizes, one launch each",
            "cpu_baseline": cpu,
            "clocks": clk,
            "served": served,
            "uneven": uneven,
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def _time_device(fn, steps: int, warmup: int) -> float:
    """Seconds per call of fn() (launches on the current stream), CUDA events, after warm-up."""
    import torch
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(steps):
        fn()
    b.record()
    torch.cuda.synchronize()
    return a.elapsed_time(b) / 1e3 / steps


def run_fp64(args):
    """FFT<double> N=1024, 256 transforms, forward then inverse per step, U[-1,1)."""
    import torch
    import fft_gb300 as F
    import oracle
    n, b = 1024, 256
    rng = np.random.default_rng(1)
    x = rng.uniform(-1, 1, (b, n)) + 1j * rng.uniform(-1, 1, (b, n))
    xi = torch.from_numpy(x).cuda()
    y = torch.empty_like(xi)
    z = torch.empty_like(xi)
    p = F.Plan(n, "f64", "complex", b)
    sh = int(torch.cuda.current_stream().cuda_stream)

    def step():
        p.exec(False, xi.data_ptr(), y.data_ptr(), sh)
        p.exec(True, y.data_ptr(), z.data_ptr(), sh)
    t = _time_device(step, max(args.steps, 200), max(args.warmup, 5))
    flops = 2 * b * 5 * n * math.log2(n)
    ref = np.stack([oracle.fft(r) for r in x])
    rel = float(np.linalg.norm(y.cpu().numpy() - ref) / np.linalg.norm(ref))
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    reps = 20
    for _ in range(reps):
        yy = oracle.batch(x, n, real=False, inverse=False, threads=threads)
        oracle.batch(yy, n, real=False, inverse=True, threads=threads)
    tc = (time.perf_counter() - t0) / reps
    # FP64 roofline: this batch (4 MiB each way) sits in L2 and is bound by FP64 arithmetic, so
    # the reference rate is a measured FP64 GEMM (cuBLAS DGEMM 4096^3, best of 3)
    a64 = torch.randn(4096, 4096, dtype=torch.float64, device="cuda")
    b64 = torch.randn(4096, 4096, dtype=torch.float64, device="cuda")
    dg = min(_time_device(lambda: torch.matmul(a64, b64), 1, 1) for _ in range(3))
    fp64_peak = 2 * 4096 ** 3 / dg / 1e12
    print(json.dumps({"workload": "FFT<double> N=1024 x256, fwd+inv", "value": flops / t / 1e9, "unit": "GFLOP/s",
                      "ms_per_step": t * 1e3, "GB_s": 2 * 2 * b * n * 16 / t / 1e9, "relL2_vs_oracle": rel,
                      "fp64_roofline": {"measured_dgemm_TFLOP_s": fp64_peak,
                                        "frac": flops / t / 1e12 / fp64_peak,
                                        "note": "5N log2 N flops per transform against cuBLAS DGEMM throughput"},
                      "cpu_baseline": {"value": flops / tc / 1e9, "unit": "GFLOP/s", "cores": threads, "kind": "port"},
                      "plan": p.describe()}), flush=True)


def run_large(args):
    """One FP32 complex transform each at 2^24, 3^15, 2^12 3^4 5^2 (forward), U[-1,1)."""
    import torch
    import fft_gb300 as F
    out = []
    sh = int(torch.cuda.current_stream().cuda_stream)
    for n in (2 ** 24, 3 ** 15, 2 ** 12 * 3 ** 4 * 5 ** 2):
        rng = np.random.default_rng(n % 997)
        x = (rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)).astype(np.complex64)
        xi = torch.from_numpy(x).cuda()
        y = torch.empty_like(xi)
        p = F.Plan(n, "f32", "complex", 1)
        t = _time_device(lambda: p.exec(False, xi.data_ptr(), y.data_ptr(), sh), 20, 3)
        alg = 16 * n
        p.exec(False, xi.data_ptr(), y.data_ptr(), sh)
        torch.cuda.synchronize()
        import oracle
        ref = oracle.fft(x.astype(np.complex128))
        rel = float(np.linalg.norm(y.cpu().numpy() - ref) / np.linalg.norm(ref))
        out.append({"n": n, "ms": t * 1e3, "GFLOP_s": 5 * n * math.log2(n) / t / 1e9, "alg_GB_s": alg / t / 1e9,
                    "passes": p.describe()["radices"], "launches": p.describe()["launches"],
                    "relL2_vs_fp64_oracle": rel})
        del xi, y, p
        torch.cuda.empty_cache()
    peak, kind = measured_peak_hbm()
    for o in out:
        o["frac_of_hbm"] = o["alg_GB_s"] / peak
    print(json.dumps({"workload": "single large complex FP32 transforms", "results": out, "peak_GB_s": peak,
                      "peak_source": kind}), flush=True)


SERVE_LOADS = (1e4, 1e5, 5e5, 1e6, 1.25e6, 1.375e6, 1.5e6, 1.75e6, 2e6)
P99_BOUND_US = 2000.0  # a load is "sustained" when the batched p99 stays within this and it keeps up


def _serve_point(srv, rate: float, duration: float, seed: int) -> dict:
    st = srv.loadgen(offered_rate=rate, duration_s=duration, seed=seed)
    span = st["span_seconds"]
    tps = st["frames"] / span if span else 0.0
    return {"p50_us": st["p50_latency_us"], "p99_us": st["p99_latency_us"], "transforms_per_s": tps,
            "GFLOP_s": st["flops"] / span / 1e9 if span else 0.0, "requests": st["completed"],
            "failed": st["failed"], "waves": st["waves"], "launches": st["launches"], "span_s": span,
            "keeps_up": bool(tps >= 0.9 * rate)}


def _serve_relerr(F) -> dict:
    """relL2 of served results against the FP64 oracle: a burst of mixed requests (complex and
    real, both directions, one- and multi-pass sizes) submitted together to the batched server,
    so that they are coalesced into shared waves."""
    import oracle
    rng = np.random.default_rng(321)
    srv = F.Server(hbm_budget_bytes=1 << 30, waves=4, max_requests_per_wave=256, coalesce=True)
    shapes = [(256, "real"), (480, "complex"), (1920, "real"), (3840, "real"), (4096, "complex"),
              (15625, "complex"), (20480, "complex"), (65536, "real"), (62500, "real"), (65536, "complex")]
    jobs = []
    for i in range(40):
        n, kind = shapes[i % len(shapes)]
        inv = bool(i % 2)
        frames = int(rng.integers(1, 5))
        if kind == "complex":
            x = (rng.standard_normal((frames, n)) + 1j * rng.standard_normal((frames, n))).astype(np.complex64)
            y = np.empty_like(x)
        elif not inv:
            x = rng.standard_normal((frames, n)).astype(np.float32)
            y = np.empty((frames, n // 2), dtype=np.complex64)
        else:
            x = (rng.standard_normal((frames, n // 2)) + 1j * rng.standard_normal((frames, n // 2))).astype(np.complex64)
            y = np.empty((frames, n), dtype=np.float32)
        t = srv.submit(n, kind, inv, x, y, frames)
        jobs.append((t, n, kind, inv, x, y))
    worst = 0.0
    for t, n, kind, inv, x, y in jobs:
        srv.wait(t)
        if kind == "complex":
            ref = oracle.batch(x.astype(np.complex128), n, real=False, inverse=inv)
        else:
            ref = oracle.batch(x.astype(np.complex128 if inv else np.float64), n, real=True, inverse=inv)
        worst = max(worst, float(np.linalg.norm(y - ref) / np.linalg.norm(ref)))
    srv.close()
    return {"worst_relL2": worst, "requests": len(jobs),
            "sample": "40 requests (1-4 frames; complex and RealFFT, forward and inverse, N 256-65536) "
                      "submitted together to the batched server, against the FP64 oracle"}


def served_block(args) -> dict:
    """Serving configuration: open-loop Poisson requests of 1-64 frames of one size, log-uniform
    over the 2^a 3^b 5^c sizes in [256, 65536], 70% RealFFT / 30% complex, 50/50 forward/inverse,
    FP32, N(0,1) inputs in pinned host memory, 16 GB HBM budget.  At each offered load: p50/p99
    latency and throughput of the continuous-batching server and of plain per-request execution
    (one synchronous copy-in / launch / copy-out per request) on the same GPU."""
    import fft_gb300 as F
    t0 = time.perf_counter()
    batched = F.Server(hbm_budget_bytes=16 << 30, waves=args.serve_waves,
                       max_requests_per_wave=args.serve_wave_requests, coalesce=True)
    plain = F.Server(hbm_budget_bytes=16 << 30, coalesce=False)
    sweep = []
    for i, rate in enumerate(SERVE_LOADS):
        row = {"offered_transforms_per_s": rate,
               "batched": _serve_point(batched, rate, args.served_duration, 100 + i),
               "plain": _serve_point(plain, rate, args.served_duration, 100 + i)}
        b, p = row["batched"], row["plain"]
        row["throughput_ratio"] = b["transforms_per_s"] / p["transforms_per_s"] if p["transforms_per_s"] else None
        sweep.append(row)
        print(json.dumps({"served_point": row}), file=sys.stderr, flush=True)
    batched.close()
    plain.close()
    ok = [r for r in sweep if r["batched"]["keeps_up"] and r["batched"]["p99_us"] <= P99_BOUND_US]
    best = max(ok, key=lambda r: r["offered_transforms_per_s"]) if ok else None
    sat_b = max(sweep, key=lambda r: r["batched"]["transforms_per_s"])
    sat_p = max(sweep, key=lambda r: r["plain"]["transforms_per_s"])
    out = {
        "workload": "open-loop Poisson, 1-64 frames/request, N log-uniform over 2^a3^b5^c in [256,65536], "
                    "70% real / 30% complex, 50/50 fwd/inv, FP32, pinned host buffers, 16 GB HBM budget",
        "duration_s_per_load": args.served_duration,
        "server": {"waves_in_flight": args.serve_waves, "requests_per_wave": args.serve_wave_requests},
        "p99_bound_us": P99_BOUND_US,
        "max_sustained_load": best["offered_transforms_per_s"] if best else None,
        "at_max_sustained_load": ({"GFLOP_s": best["batched"]["GFLOP_s"],
                                   "transforms_per_s": best["batched"]["transforms_per_s"],
                                   "p50_us": best["batched"]["p50_us"], "p99_us": best["batched"]["p99_us"],
                                   "plain_transforms_per_s": best["plain"]["transforms_per_s"],
                                   "plain_p99_us": best["plain"]["p99_us"],
                                   "throughput_ratio_vs_plain": best["throughput_ratio"]} if best else None),
        "saturation": {"batched_GFLOP_s": sat_b["batched"]["GFLOP_s"],
                       "batched_transforms_per_s": sat_b["batched"]["transforms_per_s"],
                       "plain_GFLOP_s": sat_p["plain"]["GFLOP_s"],
                       "plain_transforms_per_s": sat_p["plain"]["transforms_per_s"],
                       "ratio": (sat_b["batched"]["transforms_per_s"] / sat_p["plain"]["transforms_per_s"]
                                 if sat_p["plain"]["transforms_per_s"] else None)},
        "sweep": sweep,
        "relL2": _serve_relerr(F),
        "wall_s": None,
    }
    out["wall_s"] = time.perf_counter() - t0
    return out


def run_serve(args):
    """Open-loop Poisson request stream (1-64 frames of one size, log-uniform over 2^a 3^b 5^c
    sizes in [256, 65536], 70% real / 30% complex, 50/50 forward/inverse, FP32, 16 GB HBM budget):
    p50/p99 latency and throughput of the batched server against plain per-request execution."""
    import fft_gb300 as F
    loads = [1e4, 1e5, 5e5, 1e6, 2e6]
    sweep = []
    batched = F.Server(hbm_budget_bytes=16 << 30, waves=args.serve_waves,
                       max_requests_per_wave=args.serve_wave_requests, coalesce=True)
    plain = F.Server(hbm_budget_bytes=16 << 30, coalesce=False)
    for i, rate in enumerate(loads):
        row = {"offered_transforms_per_s": rate}
        for name, srv in (("batched", batched), ("plain", plain)):
            st = srv.loadgen(offered_rate=rate, duration_s=args.serve_duration, seed=100 + i)
            row[name] = {"p50_us": st["p50_latency_us"], "p99_us": st["p99_latency_us"],
                         "transforms_per_s": st["frames"] / st["span_seconds"] if st["span_seconds"] else 0,
                         "GFLOP_s": st["flops"] / st["span_seconds"] / 1e9 if st["span_seconds"] else 0,
                         "requests": st["completed"], "waves": st["waves"], "launches": st["launches"]}
        sweep.append(row)
        print(json.dumps(row), flush=True)
    best_b = max(r["batched"]["GFLOP_s"] for r in sweep)
    best_p = max(r["plain"]["GFLOP_s"] for r in sweep)
    print(json.dumps({"workload": "serving sweep", "metric": METRIC, "value": best_b, "unit": "GFLOP/s",
                      "plain_value": best_p, "ratio_vs_plain": best_b / best_p if best_p else None,
                      "p99_us_at_max_load": sweep[-1]["batched"]["p99_us"], "sweep": sweep}), flush=True)
    batched.close()
    plain.close()


def run_uneven(args):
    print(json.dumps(uneven_block(args)), flush=True)


def uneven_block(args, steps: int | None = None) -> dict:
    """One submission of 32768 complex FP32 transforms, sizes log-uniform over the 175 sizes
    2^a 3^b 5^c in [64, 16384], U[-1,1): the CUDA-graph batch against one plain launch per size."""
    import torch
    import fft_gb300 as F
    import oracle
    rng = np.random.default_rng(4)
    pool = np.array(F.fast_sizes(64, 16384))
    lg = rng.uniform(np.log(64), np.log(16384), 32768)
    sizes = pool[np.abs(np.log(pool)[None, :] - lg[:, None]).argmin(axis=1)].tolist()
    total = int(sum(sizes))
    x = torch.empty(total, dtype=torch.complex64, device="cuda")
    x.real.uniform_(-1, 1)
    x.imag.uniform_(-1, 1)
    y = torch.empty_like(x)
    sh = int(torch.cuda.current_stream().cuda_stream)
    flops = sum(5 * n * math.log2(n) for n in sizes)
    alg = 16 * total
    peak, kind = measured_peak_hbm()
    offs = np.concatenate([[0], np.cumsum(sizes)])
    xs = x.cpu().numpy()
    # FP64 oracle of every 128th transform (the relL2 sample), computed once for both variants
    sample = list(range(0, 32768, 128))
    refs = {i: oracle.fft(xs[offs[i]:offs[i + 1]].astype(np.complex128)) for i in sample}

    reps = args.uneven_reps or steps or max(args.steps // 4, 50)

    def variant(precision):
        t0 = time.perf_counter()
        m = F.Multi(sizes, "f32", autotune=min(args.tune, 1), precision=precision)
        build_s = time.perf_counter() - t0
        tg = _time_device(lambda: m.exec(False, x.data_ptr(), y.data_ptr(), sh), reps, 5)
        tp = _time_device(lambda: m.exec_plain(False, x.data_ptr(), y.data_ptr(), sh), reps, 5)
        m.exec(False, x.data_ptr(), y.data_ptr(), sh)
        torch.cuda.synchronize()
        ys = y.cpu().numpy()
        worst = 0.0
        for i in sample:
            got = ys[offs[i]:offs[i + 1]]
            worst = max(worst, float(np.linalg.norm(got - refs[i]) / np.linalg.norm(refs[i])))
        return {"graph": {"ms": tg * 1e3, "GFLOP_s": flops / tg / 1e9, "alg_GB_s": alg / tg / 1e9,
                          "frac_of_hbm": alg / tg / 1e9 / peak},
                "plain_per_size": {"ms": tp * 1e3, "GFLOP_s": flops / tp / 1e9, "alg_GB_s": alg / tp / 1e9,
                                   "frac_of_hbm": alg / tp / 1e9 / peak},
                "speedup_vs_plain": tp / tg, "plan_build_s": build_s, "worst_relL2_sampled": worst,
                "distinct_sizes": m.info()["distinct_sizes"], "launches_per_submission": m.info()["launches"],
                "design": ("work-item queue kernels (one per class of CTA shapes) in one CUDA graph"
                           if precision == "fp32" else "per-size tensor-core kernels in one CUDA graph")}

    t_all = time.perf_counter()
    fp32 = variant("fp32")
    bf16 = None if args.uneven_fp32_only else variant("split_bf16")
    out = {"workload": "32768 complex FP32 transforms, uneven sizes log-uniform over 2^a3^b5^c in [64,16384]",
           "alg_bytes": alg, "autotune": min(args.tune, 1), "peak_GB_s": peak, "peak_source": kind,
           "relL2_sample": f"{len(sample)} transforms (every 128th) against the FP64 oracle",
           "timing": f"CUDA events around {reps} back-to-back submissions, mean",
           "fp32_fma": fp32,
           "split_bf16": (dict(bf16, note="first radix pass (radix <= 16) on tcgen05 tensor cores, "
                                          "three BF16 parts per operand, FP32 accumulation") if bf16 else None),
           "wall_s": time.perf_counter() - t_all}
    del x, y
    torch.cuda.empty_cache()
    return out


# Per-call timing of the drop-in header: the reference's usage pattern (one object, host
# containers, one transform per call).  Compiled by run_dropin against include/signalsmith-fft.h.
DROPIN_CPP = r"""
#include <chrono>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <string>
#include <vector>
#include <algorithm>
#include "signalsmith-fft.h"

template <class F>
static void timed(const char *name, int calls, F &&call) {
	for (int i = 0; i < 50; ++i) call();
	std::vector<double> us(calls);
	for (int i = 0; i < calls; ++i) {
		auto t0 = std::chrono::steady_clock::now();
		call();
		us[i] = std::chrono::duration<double, std::micro>(std::chrono::steady_clock::now() - t0).count();
	}
	double sum = 0;
	for (double u : us) sum += u;
	std::sort(us.begin(), us.end());
	std::printf("{\"case\": \"%s\", \"calls\": %d, \"mean_us\": %.3f, \"p50_us\": %.3f, \"p99_us\": %.3f}\n", name,
	            calls, sum / calls, us[calls / 2], us[(size_t)(calls * 0.99)]);
}

int main(int argc, char **argv) {
	const int calls = argc > 1 ? std::atoi(argv[1]) : 2000;
	std::mt19937_64 rng(7);
	std::uniform_real_distribution<double> u(-1, 1);
	{
		signalsmith::FFT<double> fft(1024);
		std::vector<std::complex<double>> in(1024), out(1024);
		for (auto &v : in) v = {u(rng), u(rng)};
		timed("FFT<double>(1024).fft(vector, vector)", calls, [&] { fft.fft(in, out); });
	}
	{
		signalsmith::RealFFT<float> real(3840);
		std::vector<float> in(3840);
		std::vector<std::complex<float>> out(1920);
		for (auto &v : in) v = (float)u(rng);
		timed("RealFFT<float>(3840).fft(vector, vector)", calls, [&] { real.fft(in, out); });
	}
	{
		signalsmith::RealFFT<float> real(65536);
		std::vector<float> in(65536);
		std::vector<std::complex<float>> out(32768);
		for (auto &v : in) v = (float)u(rng);
		timed("RealFFT<float>(65536).fft(vector, vector)", calls / 4, [&] { real.fft(in, out); });
	}
	return 0;
}
"""


def run_dropin(args):
    """Per-call latency of the drop-in header (host containers in and out, one transform per call,
    synchronous, as the reference is used: benchmark/main.cpp of the reference times the same
    pattern) against the reference algorithm per call on one host core (the oracle's C
    restatement, one plan reused across calls)."""
    import shutil
    import tempfile
    import oracle
    cuda = os.path.dirname(os.path.dirname(os.path.realpath(shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc")))
    lib_dir = os.path.join(ROOT, "fft_gb300")
    d = tempfile.mkdtemp(prefix="ssfft_dropin_")
    src, exe = os.path.join(d, "dropin_bench.cpp"), os.path.join(d, "dropin_bench")
    with open(src, "w") as f:
        f.write(DROPIN_CPP)
    subprocess.run(["g++", "-std=c++14", "-O2", "-I", os.path.join(ROOT, "include"), "-I", os.path.join(cuda, "include"),
                    src, "-L", lib_dir, "-lssfft", "-L", os.path.join(cuda, "lib64"), "-lcudart",
                    f"-Wl,-rpath,{lib_dir}", f"-Wl,-rpath,{os.path.join(cuda, 'lib64')}", "-o", exe], check=True)
    r = subprocess.run([exe, str(max(200, args.steps * 10))], capture_output=True, text=True, check=True)
    gpu = [json.loads(line) for line in r.stdout.splitlines() if line.startswith("{")]
    rng = np.random.default_rng(7)
    cpu = []
    for name, n, real, dt, reps in (("FFT<double>(1024)", 1024, False, np.complex128, 4000),
                                    ("RealFFT<float>(3840)", 3840, True, np.float32, 2000),
                                    ("RealFFT<float>(65536)", 65536, True, np.float32, 100)):
        if real:
            x = rng.standard_normal((1, n)).astype(dt)
        else:
            x = (rng.uniform(-1, 1, (1, n)) + 1j * rng.uniform(-1, 1, (1, n))).astype(dt)
        oracle.batch(x, n, real=real, inverse=False, threads=1, repeats=10, kind=CPU_KIND)
        t0 = time.perf_counter()
        oracle.batch(x, n, real=real, inverse=False, threads=1, repeats=reps, kind=CPU_KIND)
        cpu.append({"case": name, "us_per_call": (time.perf_counter() - t0) / reps * 1e6})
    print(json.dumps({"workload": "drop-in header per call (host containers, synchronous)", "gpu": gpu,
                      "cpu_reference_algorithm_1_core": cpu, "cpu_build": cpu_build_note()}), flush=True)


def run_uneven_class(args):
    """One queue class of long transforms on its own: 300 complex FP32 transforms each of the
    eight sizes 8640-11520 (the 384-thread class), shuffled, U[-1,1); --queue-mode queue runs them
    as one queue-class launch (every size in a class), pergraph as one launch per size in a CUDA
    graph.  Mean time of --steps submissions after one warm-up."""
    import torch
    import fft_gb300 as F
    sizes0 = [11520, 10800, 10240, 10125, 9375, 9216, 9000, 8640]
    rng = np.random.default_rng(9)
    sizes = [n for n in sizes0 for _ in range(300)]
    rng.shuffle(sizes)
    total = int(sum(sizes))
    x = torch.empty(total, dtype=torch.complex64, device="cuda")
    x.real.uniform_(-1, 1)
    x.imag.uniform_(-1, 1)
    y = torch.empty_like(x)
    sh = int(torch.cuda.current_stream().cuda_stream)
    old = os.environ.get("SSFFT_DEBUG")
    os.environ["SSFFT_DEBUG"] = "multi_mode=1" if args.queue_mode == "pergraph" else "queue_max_n=16384"
    m = F.Multi(sizes, "f32")
    if old is None:
        os.environ.pop("SSFFT_DEBUG")
    else:
        os.environ["SSFFT_DEBUG"] = old
    t = _time_device(lambda: m.exec(False, x.data_ptr(), y.data_ptr(), sh), max(1, args.steps), 1)
    peak, kind = measured_peak_hbm()
    print(json.dumps({"workload": "uneven class 8640-11520 x300 each", "mode": args.queue_mode, "ms": t * 1e3,
                      "frac_of_hbm": 16 * total / t / 1e9 / peak, "launches": m.info()["launches"]}), flush=True)


def run_uneven_members(args):
    """The first --members of the 16 sizes 900-2048 (one CTA shape), 4000 // members complex FP32
    transforms each (--frames-total overrides the 4000), shuffled, U[-1,1): as one queue class
    (--queue-mode queue, every size in the class) or one launch per size (pergraph).  Mean time of
    --steps submissions after two warm-ups; the instruction-cache pressure of a class grows with its
    member count."""
    import torch
    import fft_gb300 as F
    pool = [2048, 1920, 1800, 1536, 1440, 1350, 1280, 1200, 1152, 1125, 1080, 1024, 1000, 972, 960, 900]
    k = max(1, min(16, args.members))
    rng = np.random.default_rng(3)
    sizes = [n for n in pool[:k] for _ in range(args.frames_total // k)]
    rng.shuffle(sizes)
    total = int(sum(sizes))
    x = torch.empty(total, dtype=torch.complex64, device="cuda")
    x.real.uniform_(-1, 1)
    x.imag.uniform_(-1, 1)
    y = torch.empty_like(x)
    sh = int(torch.cuda.current_stream().cuda_stream)
    old = os.environ.get("SSFFT_DEBUG")
    os.environ["SSFFT_DEBUG"] = "multi_mode=1" if args.queue_mode == "pergraph" else "queue_max_n=16384,queue_members=16"
    m = F.Multi(sizes, "f32")
    if old is None:
        os.environ.pop("SSFFT_DEBUG")
    else:
        os.environ["SSFFT_DEBUG"] = old
    t = _time_device(lambda: m.exec(False, x.data_ptr(), y.data_ptr(), sh), max(1, args.steps), 2)
    peak, kind = measured_peak_hbm()
    print(json.dumps({"workload": f"uneven sizes 900-2048, {k} members", "mode": args.queue_mode, "ms": t * 1e3,
                      "frac_of_hbm": 16 * total / t / 1e9 / peak, "launches": m.info()["launches"]}), flush=True)


def run_precision(args):
    """Complex FP32 N=1024, 32768 transforms: the FP32-FMA kernel against the split-BF16
    tensor-core first pass, forward + inverse, with relL2 against the FP64 oracle."""
    import torch
    import fft_gb300 as F
    import oracle
    n, b = 1024, 32768
    rng = np.random.default_rng(11)
    x = torch.empty(b, n, dtype=torch.complex64, device="cuda")
    x.real.uniform_(-1, 1)
    x.imag.uniform_(-1, 1)
    y = torch.empty_like(x)
    z = torch.empty_like(x)
    sh = int(torch.cuda.current_stream().cuda_stream)
    xs = x[:64].cpu().numpy()
    ref = oracle.batch(xs.astype(np.complex128), n, real=False, inverse=False)
    peak, kind = measured_peak_hbm()
    out = {}
    for prec in ("fp32", "split_bf16"):
        p = F.Plan(n, "f32", "complex", b, precision=prec)
        t = _time_device(lambda: (p.exec(False, x.data_ptr(), y.data_ptr(), sh),
                                  p.exec(True, y.data_ptr(), z.data_ptr(), sh)), max(args.steps // 8, 20), 3)
        torch.cuda.synchronize()
        rel = float(np.linalg.norm(y[:64].cpu().numpy() - ref) / np.linalg.norm(ref))
        alg = 2 * 16.0 * n * b
        out[prec] = {"ms_fwd_inv": t * 1e3, "GFLOP_s": 2 * 5 * n * math.log2(n) * b / t / 1e9,
                     "alg_GB_s": alg / t / 1e9, "frac_of_hbm": alg / t / 1e9 / peak, "relL2_vs_fp64_oracle": rel,
                     "schedule": p.tuning()["choice"]}
        del p
    print(json.dumps({"workload": "complex FP32 N=1024 x 32768, forward + inverse, FP32-FMA vs split-BF16",
                      "peak_GB_s": peak, "peak_source": kind, **out}), flush=True)


def run_sizes(args):
    """Per-size kernel sweep: batched FP32 transforms (complex and/or real) of each size, sized to
    --sweep-mb MiB of algorithmic traffic per launch (larger than L2), forward and inverse timed
    with CUDA events over 10 back-to-back launches each.  One JSON line per (size, kind)."""
    import torch
    import fft_gb300 as F
    peak, kind_src = measured_peak_hbm()
    opts = json.loads(args.plan_options)
    sh = int(torch.cuda.current_stream().cuda_stream)
    failures = []
    for kind in args.kinds.split(","):
        for n in (int(v) for v in args.sizes.split(",")):
            per = 16 * n if kind == "complex" else 8 * n  # algorithmic bytes per transform / frame
            batch = max(1, (args.sweep_mb << 20) // per)
            try:
                p = F.Plan(n, "f32", kind, batch, **opts)  # planner defaults unless --plan-options says
            except Exception as e:  # a size / option combination the planner refuses
                print(json.dumps({"n": n, "kind": kind, "error": str(e)}), flush=True)
                continue
            if kind == "complex":
                x = torch.randn(batch, n, dtype=torch.complex64, device="cuda")
                y = torch.empty_like(x)
            else:
                x = torch.randn(batch, n, device="cuda")
                y = torch.empty(batch, n // 2, dtype=torch.complex64, device="cuda")
            res = {}
            try:
                for inv, (a, b) in ((False, (x, y)), (True, (y, x))):
                    t = _time_device(lambda: p.exec(inv, a.data_ptr(), b.data_ptr(), sh), 10, 3)
                    res["inverse" if inv else "forward"] = {"us": round(t * 1e6, 1),
                                                            "GB_s": round(batch * per / t / 1e9),
                                                            "frac": round(batch * per / t / 1e9 / peak, 3)}
            except Exception as e:  # reported with the plan's kernels; the sweep goes on, exit status 1
                failures.append(n)
                print(json.dumps({"n": n, "kind": kind, "batch": batch, "error": str(e),
                                  "schedule": p.tuning()["choice"], "kernel": p.kernel(False),
                                  "kernel_inverse": p.kernel(True), "tune_log": p.tuning()["log"][-4:]}), flush=True)
                del x, y, p
                torch.cuda.empty_cache()
                continue
            d = p.describe()
            print(json.dumps({"n": n, "kind": kind, "batch": batch, **res, "peak_GB_s": peak, "peak_source": kind_src,
                              "radices": d["radices"], "threads": d["threads"], "per_cta": d["per_cta"],
                              "schedule": p.tuning()["choice"], "kernel": p.kernel(False)}), flush=True)
            del x, y, p
            torch.cuda.empty_cache()
    if failures:
        sys.exit(1)


def main():
    args = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", str(args.gpus)))
    if args.impl == "reference":
        run_reference(args, rank, world)
    elif args.workload != "realfft":
        import torch
        from fft_gb300 import build as fb
        fb.build()
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        {"fp64": run_fp64, "large": run_large, "serve": run_serve, "uneven": run_uneven,
         "served": lambda a: print(json.dumps(served_block(a)), flush=True),
         "precision": run_precision, "sizes": run_sizes, "dropin": run_dropin,
         "uneven_class": run_uneven_class, "uneven_members": run_uneven_members}[args.workload](args)
    else:
        run_gpu(args, rank, world if "WORLD_SIZE" in os.environ else 1)


if __name__ == "__main__":
    main()
