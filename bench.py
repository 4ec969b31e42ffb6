#!/usr/bin/env python
"""Benchmark of the design-matrix (A-matrix) assembly of ChIMES-lsq on GB300.

Workload: 128 rigid H2O (384 atoms, cubic 15.65 A, Gaussian 0.1 A displacements),
200 frames, Chebyshev 2-body order 16 (5.0 A) + 3-body order 8 (4.0 A), force,
full-stress and energy rows: A is 232,800 x 820.  Synthetic and seeded.

A step assembles the whole A matrix of the 200 frames in FP64 (the plain form,
parity-exact with the reference).  ``value`` is rows/s with the frames already
resident in HBM and A written to HBM; ``e2e`` is the same through the C ABI's
host-buffer call (coordinates host->device, A device->host into pinned memory).
Each step writes 1.5 GB of A, far above the 129 MB L2, so no L2 flush is needed.

``--impl reference`` times the reference algorithm on the host cores: the CPU
oracle port (the reference's own loops restated in C++, OpenMP over frames, the
reference's MPI frame split) on a bounded sample of the same frames.
"""
import argparse
import importlib
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
METRIC = "A-matrix rows/s & MD atom-steps/s at 1 GB300 vs plain FP64; p50/p99 force latency"
WORKLOAD = "water-3b"
WORKLOAD_DESC = ("128 H2O (384 atoms, cubic 15.65 A, +0.1 A Gaussian), 200 frames, Chebyshev 2B16@5.0 + 3B8@4.0, "
                 "force + full stress + energy rows, A 232800 x 820")


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi sampling of SM clock and throttle reasons during the timed region."""

    def __init__(self, gpu=0):
        self.gpu = gpu
        self.proc = None
        self.out = tempfile.NamedTemporaryFile(delete=False, suffix=".csv").name

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.out, "w"), stderr=subprocess.DEVNULL)
        except FileNotFoundError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.out):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.out)
        if not sm:
            return None
        load = [s for s in sm if s > 0.5 * mx] or sm
        return {"sm_mhz": statistics.median(load), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def time_oracle(fm, nframes_sample, threads):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build() if not os.path.exists(oracle.LIB) else None
    t = time.perf_counter()
    A, _ = oracle.assemble(fm, nframes=nframes_sample, first=0, count=nframes_sample, nthreads=threads)
    dt = time.perf_counter() - t
    return A.shape[0] / dt, A.shape[0], dt


def reference_arm(args, rank, world):
    if rank != 0:
        return
    synth = importlib.import_module("chimes_lsq-myllfork_gb300.synth")
    tmp = tempfile.mkdtemp(prefix="chimes_ref_")
    fm = synth.make_workload(WORKLOAD, tmp, seed=1000)
    threads = cpu_threads()
    sample = 32
    for _ in range(args.warmup):
        time_oracle(fm, sample, threads)
    rates, rows, secs = [], 0, 0.0
    for _ in range(args.steps):
        r, n, dt = time_oracle(fm, sample, threads)
        rows += n
        secs += dt
    value = rows / secs
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "rows/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * secs / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "desc": WORKLOAD_DESC, "sample_frames_per_step": sample},
        "cpu_baseline": {"value": value, "unit": "rows/s", "cores": threads, "kind": "port",
                         "sample": f"first {sample} of the 200 frames per step (OpenMP over frames)"},
        "e2e": {"value": value, "unit": "rows/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "fp32"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--frames", type=int, default=200, help="frames per rank (200 = the full workload)")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return reference_arm(args, rank, world)

    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    cg = importlib.import_module("chimes_lsq-myllfork_gb300")
    synth = importlib.import_module("chimes_lsq-myllfork_gb300.synth")
    tmp = tempfile.mkdtemp(prefix="chimes_bench_")
    fm = synth.make_workload(WORKLOAD, tmp, nframes=args.frames, seed=1000 + rank)   # weak scaling: own frames per rank
    model = cg.Model(fm)
    frames = cg.Frames.read(model)
    sess = cg.Session(model, local)
    prec = cg.CG_FP64 if args.precision == "fp64" else cg.CG_FP32
    esz = 8 if prec == cg.CG_FP64 else 4
    nrows, natoms = frames.rows()
    ncols = model.ncols
    dfr = sess.upload(frames)
    A = torch.empty((nrows, ncols), dtype=torch.float64 if esz == 8 else torch.float32, device="cuda")
    stream = torch.cuda.ExternalStream(sess.stream)

    def step():
        sess.assemble_device(dfr, prec, A.data_ptr(), ncols)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    ms = e0.elapsed_time(e1)
    clk = clocks.stop()
    launches = sess.last_launches() * args.steps
    counts = sess.last_counts()
    if dist:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = world * nrows * args.steps / (ms / 1000.0)

    # live per-stage timing (same stream, CUDA events) for the roofline of the dominant kernel
    sess.profile(True)
    for _ in range(3):
        step()
    stages = sess.stage_times()
    sess.profile(False)
    dom = max(stages, key=lambda k: stages[k][0])
    dom_ms = stages[dom][0] / max(1, stages[dom][1])
    cols = model.columns()
    frames_n = args.frames
    force_rows = 3 * natoms
    vir_rows = nrows - force_rows
    # algorithmic bytes written per launch (A entries the kernel owns) and FP64 work
    bytes_by_stage = {
        "force_3b": force_rows * cols["n3b"] * esz, "virial_3b": vir_rows * cols["n3b"] * esz,
        "force_2b": force_rows * cols["n2b"] * esz, "virial_2b": vir_rows * cols["n2b"] * esz,
    }
    flops_by_stage = {"force_3b": counts["evals3"] * 3 * 3 * 2, "virial_3b": counts["evals3"] * 13 * 2}
    hbm_peak, peak_kind = peaks()
    algo_bytes = bytes_by_stage.get(dom, nrows * ncols * esz)
    achieved = algo_bytes / (dom_ms / 1000.0) / 1e9
    roofline = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                "frac": achieved / hbm_peak, "traffic": None, "peak_source": peak_kind,
                "note": "FP64 kernels are FP64-pipe bound; see fp64 below"}
    fp64 = None
    if dom in flops_by_stage:
        tf = flops_by_stage[dom] / (dom_ms / 1000.0) / 1e12
        fp64 = {"kernel": dom, "achieved_tflops": tf, "nominal_peak_tflops": 1.25, "frac_nominal": tf / 1.25,
                "flops_per_launch": flops_by_stage[dom]}

    # end to end through the C ABI with host buffers
    host = torch.empty((nrows, ncols), dtype=A.dtype, pin_memory=True)
    out = host.numpy()
    sess.assemble(frames, prec, out=out)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        sess.assemble(frames, prec, out=out)
    e2e_s = time.perf_counter() - t0
    e2e = {"value": world * nrows * args.steps / e2e_s, "unit": "rows/s",
           "h2d_bytes_per_step": int(natoms * (3 * 8 + 4) + frames_n * (4 + 3 * 8 + 2 * 4 + 208) + 3 * 8),
           "d2h_bytes_per_step": int(nrows * ncols * esz)}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        th = cpu_threads()
        r, n, dt = time_oracle(fm, 48, th)
        cpu = {"value": r, "unit": "rows/s", "cores": th, "kind": "port",
               "sample": f"first 48 of the 200 frames ({n} rows, {dt:.1f} s wall, OpenMP over frames)"}
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "rows/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if esz == 8 else "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "desc": WORKLOAD_DESC, "rows_per_step": nrows, "cols": ncols,
                       "l2": "each step writes 1.5 GB of A (> 129 MB L2); no flush needed",
                       "parallelism": f"frames sharded, {world} rank(s), no collective"},
            "clocks": clk, "e2e": e2e, "gpu_launches": launches, "roofline": roofline, "fp64": fp64,
            "stages_ms_per_step": {k: v[0] / max(1, v[1]) for k, v in stages.items() if v[1]},
            "work": counts, "cpu_baseline": cpu,
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
