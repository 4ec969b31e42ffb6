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


def bf16_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("bf16_tflops", 1900.0), "measured"
    return 1900.0, "fallback"


def gram_bench(cg, sess, model, A64, b, steps, torch):
    """Normal equations of the step's A: the plain form (FP64 A, FP64 library Gram)
    against the mixed form (FP32 A, split-BF16 tcgen05 Gram, FP32 accumulate), and
    the FP64 solve of both against each other."""
    nrows, ncols = A64.shape
    stream = torch.cuda.ExternalStream(sess.stream)
    A32 = A64.float()
    G = torch.zeros((ncols, ncols), dtype=torch.float64, device="cuda")
    h = torch.zeros(ncols, dtype=torch.float64, device="cuda")
    flops = nrows * ncols * (ncols + 1) + 2 * nrows * ncols   # SYRK lower triangle + A^T b
    out = {}
    for name, prec, src, mode in (("fp64", 0, A64, 0), ("bf16x3", 1, A32, 1)):
        def one():
            G.zero_(); h.zero_()
            sess.gram(prec, src.data_ptr(), ncols, nrows, ncols, b.data_ptr(), mode, G.data_ptr(), h.data_ptr())
        for _ in range(3):
            one()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            one()
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        sess.gram_finish(G.data_ptr(), ncols)
        torch.cuda.synchronize()
        out[name] = {"ms": ms, "tflops": flops / (ms / 1e3) / 1e12, "G": G.clone()}
        # per-kernel split of the call (CUDA events on the session stream)
        sess.profile(True)
        for _ in range(3):
            one()
        st = sess.stage_times()
        sess.profile(False)
        out[name]["stages_ms"] = {k: v[0] / v[1] for k, v in st.items() if k.startswith("gram") and v[1]}
    pk, kind = bf16_peak()
    tc = out["bf16x3"]
    tc_ms = tc["stages_ms"].get("gram_tensor", tc["ms"])
    tc_tf = flops / (tc_ms / 1e3) / 1e12
    roof = {"bound": "tensor", "kernel": "k_gram_tc (split-BF16 3-term, tcgen05)", "achieved": tc_tf,
            "peak": pk / 3.0, "unit": "TFLOP/s", "frac": tc_tf / (pk / 3.0), "traffic": None,
            "peak_source": f"{kind} bf16 dense burst / 3 (three BF16 products per FP32-accurate product)",
            "flops_per_launch": flops, "kernel_ms": tc_ms,
            "note": "achieved = algorithmic SYRK flops R*C*(C+1) / k_gram_tc time; the three BF16 products run "
                    "3x these flops on the tensor pipe"}
    # the solve of both forms on one ridge system (coefficients and RMSE agreement)
    Gd = torch.diagonal(out["fp64"]["G"])
    lam = 1e-6 * float(Gd.abs().max())
    h64 = (A64.T @ b).contiguous()
    res = {}
    for name, it in (("fp64", 20), ("bf16x3", 400)):
        x = torch.zeros(ncols, dtype=torch.float64, device="cuda")
        t0 = time.perf_counter()
        info = sess.solve(out[name]["G"].data_ptr(), h64.data_ptr(), ncols, lam, A64.data_ptr(), ncols, nrows,
                          b.data_ptr(), it, x.data_ptr())
        torch.cuda.synchronize()
        res[name] = (x, time.perf_counter() - t0, info)
    xf, xm = res["fp64"][0], res["bf16x3"][0]
    rel = float(torch.linalg.norm(xm - xf) / torch.linalg.norm(xf))
    rm = lambda x: float(torch.sqrt(torch.mean((A64 @ x - b) ** 2)))
    return {
        "rows": nrows, "cols": ncols, "fp64_ms": out["fp64"]["ms"], "fp64_tflops": out["fp64"]["tflops"],
        "bf16x3_ms": tc["ms"], "bf16x3_tflops": tc["tflops"], "speedup_mixed_vs_fp64": out["fp64"]["ms"] / tc["ms"],
        "stages_ms": {"fp64": out["fp64"]["stages_ms"], "bf16x3": tc["stages_ms"]},
        "solve": {"ridge": lam, "fp64_s": res["fp64"][1], "mixed_s": res["bf16x3"][1],
                  "coef_rel_diff_mixed_vs_fp64": rel, "rmse_fp64": rm(xf), "rmse_mixed": rm(xm),
                  "unit_rmse": "kcal/mol/A over all rows"},
    }, roof


def md_bench(cg, local):
    """MD serving on the Poisson-arrival, 64-4096-atom, 4-species, 4-body workload:
    a bounded arrival window, 100 NVE steps per request, batched FP64 and
    FP32-contraction serving against one request at a time in FP64."""
    synth = importlib.import_module("chimes_lsq-myllfork_gb300.synth")
    import numpy as np
    KB = 0.0019872067
    window, nsteps, rate = 0.02, 100, 2000.0
    rng = np.random.default_rng(7)
    arr = np.cumsum(rng.exponential(1 / rate, size=10000))
    arr = arr[arr < window]
    nreq = len(arr)
    sizes = np.exp(rng.uniform(np.log(64), np.log(4096), size=nreq)).astype(int)
    tmp = tempfile.mkdtemp(prefix="chimes_md_")
    fm = synth.make_workload("chno-4b", tmp, nframes=nreq, seed=9, sizes=list(sizes), triclinic=False, density=0.1,
                             labels=False)
    model = cg.Model(fm)
    nat, types, xyz, cell = synth.frames_arrays(os.path.join(tmp, "traj.xyzf"), nreq, ["C", "H", "N", "O"])[:4]
    masses = np.array([12.011, 1.0079, 14.007, 15.9994])
    x = np.random.default_rng(1).standard_normal(model.ncols) * 1e-4
    ofs = np.concatenate([[0], np.cumsum(nat)])
    reqs = []
    for k in range(nreq):
        a, b = ofs[k], ofs[k + 1]
        v = rng.standard_normal((b - a, 3)) * np.sqrt(KB * 300.0 / masses[types[a:b]])[:, None]
        reqs.append(dict(types=types[a:b], xyz=xyz[a:b], cell=cell[k], v=v, nsteps=nsteps, arrival=float(arr[k])))
    out = {"workload": f"{nreq} Poisson arrivals at {rate:.0f}/s over {window} s, N log-uniform in [64, 4096] "
                       f"(mean {sizes.mean():.0f}), 4 species, density 0.1/A^3, 2B16@5.0 / 3B8@4.0 / 4B4@3.5 "
                       f"({model.ncols} coefficients, seeded), {nsteps} NVE steps at 0.2 fs each",
           "unit": "atom-steps/s"}
    sel = (sizes >= 768) & (sizes <= 1280)
    # throughput-oriented batches (16k atoms), a latency-oriented FP32 batch cap, and the
    # plain one-request-at-a-time FP64 loop
    for name, prec, cap, frames_cap, sub in (("batched_fp64", 0, 16384, 1024, None),
                                             ("batched_fp32", 1, 16384, 1024, None),
                                             ("batched_fp32_cap4096", 1, 4096, 1024, None),
                                             ("one_at_a_time_fp64", 0, 1 << 16, 1, 6)):
        sess = cg.Session(model, local)
        sess.md_setup(x, precision=prec)
        rq = reqs if sub is None else [dict(r, arrival=0.0) for r in reqs[:sub]]
        sz = sizes if sub is None else sizes[:sub]
        outs, res, step_ms, nb = sess.md_serve(rq, masses, dt_fs=0.2, max_batch_atoms=cap,
                                               max_batch_frames=frames_cap)
        t_first = min(r["arrival"] for r in rq)
        span = float(res["finished"].max() - t_first)
        sm = step_ms.reshape(-1)
        d = {"value": float(sz.sum() * nsteps / span), "batched_steps": int(nb), "requests": len(rq),
             "max_batch_atoms": cap if frames_cap > 1 else "one request",
             "step_ms_p50": float(np.percentile(sm, 50)), "step_ms_p99": float(np.percentile(sm, 99)),
             "request_latency_s_p50": float(np.percentile(res["finished"] - np.array([r["arrival"] for r in rq]), 50)),
             "request_latency_s_p99": float(np.percentile(res["finished"] - np.array([r["arrival"] for r in rq]), 99))}
        s1 = sel[: len(rq)]
        if s1.any():
            d["step_ms_p50_1024atom"] = float(np.percentile(step_ms[s1].reshape(-1), 50))
            d["step_ms_p99_1024atom"] = float(np.percentile(step_ms[s1].reshape(-1), 99))
        out[name] = d
    # one 1024-atom request alone: per-step latency of the plain and the FP32 form
    for name, prec in (("single_1024_fp64", 0), ("single_1024_fp32", 1)):
        tmp2 = tempfile.mkdtemp(prefix="chimes_md1_")
        fm2 = synth.make_workload("chno-4b", tmp2, nframes=1, seed=21, sizes=[1024], triclinic=False, density=0.1,
                                  labels=False)
        m2 = cg.Model(fm2)
        n2, t2, x2, c2 = synth.frames_arrays(os.path.join(tmp2, "traj.xyzf"), 1, ["C", "H", "N", "O"])[:4]
        v2 = rng.standard_normal((1024, 3)) * np.sqrt(KB * 300.0 / masses[t2])[:, None]
        sess = cg.Session(m2, local)
        sess.md_setup(x, precision=prec)
        _, res, step_ms, _ = sess.md_serve([dict(types=t2, xyz=x2, cell=c2[0], v=v2, nsteps=nsteps, arrival=0.0)],
                                           masses, dt_fs=0.2)
        sm = step_ms.reshape(-1)[1:]
        out[name] = {"step_ms_p50": float(np.percentile(sm, 50)), "step_ms_p99": float(np.percentile(sm, 99)),
                     "value": float(1024 / (np.mean(sm) / 1e3))}
    return out


def fit4b_bench(cg, local, nframes, block, solve):
    """The 4-body fit (256-atom C/H/N/O triclinic frames, 2B16 / 3B8 / 4B4, force +
    stress + energy rows, 51,209 columns) in blocks of frames: the plain form (FP64
    assembly + FP64 library Gram) against the mixed form (FP32 assembly + split-BF16
    tcgen05 Gram).  The FP64 Gram runs about 0.4 TFLOP/s on this GPU, so it is timed
    on one frame's rows and scaled per row (linear in rows)."""
    import numpy as np
    import torch
    synth = importlib.import_module("chimes_lsq-myllfork_gb300.synth")
    tmp = tempfile.mkdtemp(prefix="chimes_4b_")
    fm = synth.make_workload("chno-4b", tmp, nframes=nframes, seed=2024)
    model = cg.Model(fm)
    C = model.ncols
    nat, types, xyz, cell, frc, st, en = synth.frames_arrays(os.path.join(tmp, "traj.xyzf"), nframes,
                                                             ["C", "H", "N", "O"])
    sess = cg.Session(model, local)
    stream = torch.cuda.ExternalStream(sess.stream)
    ofs = np.concatenate([[0], np.cumsum(nat)])
    blocks = []
    for f0 in range(0, nframes, block):
        f1 = min(nframes, f0 + block)
        a, b = ofs[f0], ofs[f1]
        fr = cg.Frames.from_arrays(model, nat[f0:f1], types[a:b], xyz[a:b], cell[f0:f1], forces=frc[a:b],
                                   stress=st[f0:f1], energy=en[f0:f1], first_index=f0)
        blocks.append((fr, sess.upload(fr), torch.from_numpy(fr.labels()).cuda()))
    rows = sum(bl[0].nrows for bl in blocks)
    maxr = max(bl[0].nrows for bl in blocks)
    G = torch.zeros((C, C), dtype=torch.float64, device="cuda")
    h = torch.zeros(C, dtype=torch.float64, device="cuda")

    def timed(fn):
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / 1e3

    out = {"workload": f"chno-4b: {nframes} frames x 256 atoms (triclinic, Morse + Axilrod-Teller labels), "
                       f"2B16@5.0 / 3B8@4.0 / 4B4@3.5, {rows} rows x {C} columns, blocks of {block} frames"}
    for name, prec in (("fp64", cg.CG_FP64), ("fp32", cg.CG_FP32)):
        A = torch.empty((maxr, C), dtype=torch.float64 if prec == cg.CG_FP64 else torch.float32, device="cuda")
        sess.assemble_device(blocks[0][1], prec, A.data_ptr(), C)   # warm-up
        t_asm, t_gram = 0.0, 0.0
        G.zero_(); h.zero_()
        for fr, dfr, bvec in blocks:
            t_asm += timed(lambda: sess.assemble_device(dfr, prec, A.data_ptr(), C))
            if prec == cg.CG_FP32:
                t_gram += timed(lambda: sess.gram(1, A.data_ptr(), C, fr.nrows, C, bvec.data_ptr(), 1, G.data_ptr(),
                                                  h.data_ptr()))
        if prec == cg.CG_FP64:
            # FP64 Gram on the first frame's rows, scaled per row
            r1 = 780
            Gs = torch.zeros((C, C), dtype=torch.float64, device="cuda")
            hs = torch.zeros(C, dtype=torch.float64, device="cuda")
            fr0, dfr0, b0 = blocks[0]
            sess.assemble_device(dfr0, prec, A.data_ptr(), C)
            t1 = timed(lambda: sess.gram(0, A.data_ptr(), C, r1, C, b0.data_ptr(), 0, Gs.data_ptr(), hs.data_ptr()))
            t_gram = t1 * rows / r1
            del Gs, hs
        out[name] = {"assembly_rows_per_s": rows / t_asm, "assembly_s": t_asm, "gram_s": t_gram,
                     "gram_timing": "measured over all rows" if prec == cg.CG_FP32 else
                     "measured on 780 rows, scaled per row",
                     "assembly_plus_gram_rows_per_s": rows / (t_asm + t_gram)}
        del A
        torch.cuda.empty_cache()
    out["speedup_mixed_vs_plain"] = (out["fp64"]["assembly_s"] + out["fp64"]["gram_s"]) / (
        out["fp32"]["assembly_s"] + out["fp32"]["gram_s"])
    out["speedup_assembly_fp32_vs_fp64"] = out["fp64"]["assembly_s"] / out["fp32"]["assembly_s"]
    if solve:
        sess.gram_finish(G.data_ptr(), C)
        lam = 1e-6 * float(torch.diagonal(G).abs().max())
        x = torch.zeros(C, dtype=torch.float64, device="cuda")
        t = time.perf_counter()
        info = sess.solve(G.data_ptr(), h.data_ptr(), C, lam, 0, C, 0, 0, 0, x.data_ptr())
        torch.cuda.synchronize()
        out["solve_fp64_cholesky_s"] = time.perf_counter() - t
        out["solve_ridge"] = info[2]
    return out


def batched_bench(cg, local, nframes, per_frame_sample=24):
    """Batched assembly streamed into the FP32-accumulated tensor-core Gram: frames
    with log-uniform 32-1024 atoms, 4 species, cubic boxes at 0.1 atoms/A^3, the
    4-body basis (2B16 / 3B8 / 4B4, 51,209 columns).  One CUDA graph replays every
    block's assembly (FP32) and Gram; block size from the autotuner.  Against: the
    same frames one at a time (per-frame assembly + Gram calls, host-synchronised)."""
    import numpy as np
    import torch
    synth = importlib.import_module("chimes_lsq-myllfork_gb300.synth")
    autotune = importlib.import_module("chimes_lsq-myllfork_gb300.autotune")
    rng = np.random.default_rng(33)
    sizes = np.exp(rng.uniform(np.log(32), np.log(1024), size=nframes)).astype(int)
    tmp = tempfile.mkdtemp(prefix="chimes_batch_")
    fm = synth.make_workload("chno-4b", tmp, nframes=nframes, seed=34, sizes=list(sizes), triclinic=False,
                             density=0.1, labels=False)
    model = cg.Model(fm)
    frames = cg.Frames.read(model)
    sess = cg.Session(model, local)
    C = model.ncols
    stream = torch.cuda.ExternalStream(sess.stream)
    t0 = time.perf_counter()
    choice, trials = autotune.tune_batch(cg, sess, frames, sizes, block_candidates=(16, 32, 64), sample_frames=64,
                                         repeats=1, torch=torch)
    tune_s = time.perf_counter() - t0
    sess.tune("gram_ctas_per_sm", choice["gram_ctas_per_sm"])
    bf = choice["block_frames"]
    blocks = [frames.slice(f0, min(bf, nframes - f0)) for f0 in range(0, nframes, bf)]
    rows = sum(b.nrows for b in blocks)
    maxrows = max(b.nrows for b in blocks)
    A = torch.empty((maxrows, C), dtype=torch.float32, device="cuda")
    G = torch.zeros((C, C), dtype=torch.float64, device="cuda")
    h = torch.zeros(C, dtype=torch.float64, device="cuda")
    dfs = [sess.upload(b) for b in blocks]
    labels = [torch.from_numpy(b.labels()).cuda() for b in blocks]
    t0 = time.perf_counter()
    g = sess.batch_fit(dfs, [l.data_ptr() for l in labels], cg.CG_FP32, A.data_ptr(), C, G.data_ptr(), h.data_ptr())
    build_s = time.perf_counter() - t0
    torch.cuda.synchronize()
    G.zero_(); h.zero_()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    g.launch()
    e1.record(stream)
    torch.cuda.synchronize()
    graph_s = e0.elapsed_time(e1) / 1e3
    # per-frame launches on a sample of the same frames
    nper = min(per_frame_sample, nframes)
    single = [frames.slice(f, 1) for f in range(nper)]
    A1 = torch.empty((max(x.nrows for x in single), C), dtype=torch.float32, device="cuda")
    d1 = [sess.upload(x) for x in single]
    l1 = [torch.from_numpy(x.labels()).cuda() for x in single]
    sess.assemble_device(d1[0], cg.CG_FP32, A1.data_ptr(), C)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for x, dfx, lx in zip(single, d1, l1):
        sess.assemble_device(dfx, cg.CG_FP32, A1.data_ptr(), C)
        sess.gram(1, A1.data_ptr(), C, x.nrows, C, lx.data_ptr(), 1, G.data_ptr(), h.data_ptr())
    torch.cuda.synchronize()
    per_s = time.perf_counter() - t0
    rows_per = sum(x.nrows for x in single)
    hbm, kind = peaks()
    cpad = (C + 127) // 128 * 128
    bytes_per_row = 4 * C + 4 * C + 4 * cpad + 4 * cpad   # A write, A read by the split, planes write + read
    flops = rows * C * (C + 1)
    pk, bkind = bf16_peak()
    return {
        "workload": f"{nframes} frames, N log-uniform in [32, 1024] (mean {sizes.mean():.0f}), 4 species, cubic "
                    f"0.1/A^3, 2B16@5.0 / 3B8@4.0 / 4B4@3.5, {rows} rows x {C} columns",
        "graph": {"rows_per_s": rows / graph_s, "seconds": graph_s, "blocks": len(blocks), "block_frames": bf,
                  "graph_nodes": g.nodes, "capture_and_sizing_s": build_s,
                  "hbm_gbs_algorithmic": rows * bytes_per_row / graph_s / 1e9, "hbm_peak_gbs": hbm,
                  "gram_tflops_algorithmic": flops / graph_s / 1e12, "bf16_peak_over_3": pk / 3.0},
        "per_frame": {"rows_per_s": rows_per / per_s, "frames": nper, "seconds": per_s},
        "speedup_graph_vs_per_frame": (rows / graph_s) / (rows_per / per_s),
        "autotune": {"choice": choice, "seconds": tune_s, "trials": trials},
        "note": "bytes per row: FP32 A write + read by the BF16 split + BF16 hi/lo planes write + read",
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "fp32"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--frames", type=int, default=200, help="frames per rank (200 = the full workload)")
    ap.add_argument("--no-gram", action="store_true")
    ap.add_argument("--no-md", action="store_true")
    ap.add_argument("--fit4b", type=int, default=0, metavar="FRAMES",
                    help="also measure the 4-body fit (assembly + Gram, plain vs mixed) on FRAMES frames")
    ap.add_argument("--fit4b-solve", action="store_true", help="with --fit4b: time the FP64 Cholesky of its Gram")
    ap.add_argument("--batched", type=int, default=0, metavar="FRAMES",
                    help="also measure the batched graph fit on FRAMES uneven 4-body frames")
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
    # the 3-body force stage (k_cluster_basis + k_force_mb) writes 99% of A's bytes; the
    # stress/energy stage of similar length writes 1%, so the HBM roofline is the force
    # stage's (both are FP64-pipe bound in the FP64 form: see fp64 / fp64_virial)
    dom = "force_3b" if "force_3b" in stages else max(stages, key=lambda k: stages[k][0])
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
    # DRAM bytes (read + write) of the stage's kernels per frame, from one ncu capture of
    # `profile_cases.py assemble 40` (FP64; profiles/k_force_mb_traffic_water3b_40frames.md),
    # scaled to this launch's frames
    traffic_per_frame = {("force_3b", 8): (406343168 + 218856704 + 18518272 + 327047680) / 40.0,
                         ("virial_3b", 8): (410388736 + 14920704) / 40.0}
    tpf = traffic_per_frame.get((dom, esz)) if WORKLOAD == "water-3b" else None
    roofline = {"bound": "hbm", "kernel": dom + (" (k_cluster_basis + k_force_mb<3>)" if dom == "force_3b" else ""),
                "achieved": achieved, "peak": hbm_peak, "unit": "GB/s", "frac": achieved / hbm_peak,
                "traffic": None if tpf is None else tpf * frames_n,
                "traffic_note": None if tpf is None else "ncu dram bytes of a 40-frame capture scaled per frame",
                "peak_source": peak_kind,
                "note": "the FP64 kernels are FP64-pipe bound (89% of the FP64 pipe in k_force_mb); see fp64"}
    fp64 = None
    if dom in flops_by_stage:
        tf = flops_by_stage[dom] / (dom_ms / 1000.0) / 1e12
        fp64 = {"kernel": dom, "achieved_tflops": tf, "nominal_peak_tflops": 1.25, "frac_nominal": tf / 1.25,
                "flops_per_launch": flops_by_stage[dom]}
    fp64_virial = None
    if "virial_3b" in stages:
        vms = stages["virial_3b"][0] / max(1, stages["virial_3b"][1])
        tf = flops_by_stage["virial_3b"] / (vms / 1000.0) / 1e12
        fp64_virial = {"kernel": "virial_3b (k_virial_mb<3>)", "ms": vms, "achieved_tflops": tf,
                       "frac_nominal": tf / 1.25, "flops_per_launch": flops_by_stage["virial_3b"]}

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

    gram, gram_roof = None, None
    if rank == 0 and not args.no_gram:
        b = torch.from_numpy(frames.labels()).cuda()
        A64 = A if esz == 8 else A.double()
        sess.assemble_device(dfr, cg.CG_FP64, A64.data_ptr(), ncols) if esz != 8 else None
        torch.cuda.synchronize()
        gram, gram_roof = gram_bench(cg, sess, model, A64, b, max(3, args.steps // 2), torch)
    # the mixed-precision form of the same step: FP32 assembly + split-BF16 Gram, against
    # the plain FP64 assembly + FP64 Gram (the spec comparison on this workload)
    mixed = None
    if rank == 0 and not args.no_gram and esz == 8 and gram is not None:
        A32 = torch.empty((nrows, ncols), dtype=torch.float32, device="cuda")
        for _ in range(3):
            sess.assemble_device(dfr, cg.CG_FP32, A32.data_ptr(), ncols)
        torch.cuda.synchronize()
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        for _ in range(args.steps):
            sess.assemble_device(dfr, cg.CG_FP32, A32.data_ptr(), ncols)
        f1.record(stream)
        torch.cuda.synchronize()
        ms32 = f0.elapsed_time(f1) / args.steps
        plain = ms / args.steps + gram["fp64_ms"]
        mix = ms32 + gram["bf16x3_ms"]
        mixed = {"assembly_fp32_rows_per_s": nrows / (ms32 / 1000.0), "assembly_fp32_ms": ms32,
                 "plain_assembly_plus_gram_ms": plain, "mixed_assembly_plus_gram_ms": mix,
                 "speedup_mixed_vs_plain": plain / mix,
                 "note": "FP32 A within 2e-5 of each column's scale; ridge coefficients of the mixed Gram "
                         "(FP64-refined) vs FP64 in gram.solve"}
        del A32
    md = None
    if rank == 0 and not args.no_md:
        del A
        torch.cuda.empty_cache()
        md = md_bench(cg, local)

    fit4b = None
    if rank == 0 and args.fit4b > 0:
        fit4b = fit4b_bench(cg, local, args.fit4b, 8, args.fit4b_solve)

    batched = None
    if rank == 0 and args.batched > 0:
        batched = batched_bench(cg, local, args.batched)

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
            "clocks": clk, "e2e": e2e, "gpu_launches": launches, "roofline": roofline, "fp64": fp64, "fp64_virial": fp64_virial, "mixed_form": mixed,
            "stages_ms_per_step": {k: v[0] / max(1, v[1]) for k, v in stages.items() if v[1]},
            "work": counts, "cpu_baseline": cpu, "gram": gram, "roofline_gram": gram_roof, "md": md, "fit4b": fit4b, "batched": batched,
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
