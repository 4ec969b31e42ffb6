#!/usr/bin/env python
"""Benchmark of the ChIMES-lsq design-matrix path on one GB300.

Workload (the 4-body fit): 1000 frames of 256 C/H/N/O atoms in triclinic cells
(a, b, c in [12, 16] A, angles in [80, 100] deg, minimum separation 0.9 A), labels
from a Morse pair + Axilrod-Teller triple potential; Chebyshev 2-body order 16
(5.0 A), 3-body order 8 (4.0 A), 4-body order 4 (3.5 A); force, full-stress and
energy rows.  A is 780,000 x 51,209.  Synthetic and seeded.

A step assembles every row of A in FP64 (the plain form, parity-exact with the
reference) in row blocks of 50 frames.  ``value`` is rows/s with the frames already
resident in HBM; ``e2e`` is the same metric through the C ABI's streamed host call
(cg_assemble_stream: coordinates host->device, every A block device->host into
pinned memory while the next block assembles).  Each step writes 320 GB of A, far
above the 129 MB L2, so no L2 flush is needed.

Beside the headline the line carries the spec comparison on the same
workload (``fit4b``): the mixed form (FP32 assembly, split-BF16 tensor-core Gram,
FP64 Cholesky, FP64 conjugate-gradient passes over re-assembled row blocks) against
the plain FP64 form (FP64 assembly, FP64 SYRK Gram, FP64 Cholesky), with the
coefficient error and the force-row RMS difference against the FP64-converged
solution; the batched form on 4096 uneven frames (``batched``); and MD serving
(``md``).

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
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
METRIC = "A-matrix rows/s & MD atom-steps/s at 1 GB300 vs plain FP64; p50/p99 force latency"
WORKLOAD = "chno-4b"
NFRAMES = 1000
BLOCK_FRAMES = 50
E2E_BLOCK_FRAMES = 25   # streamed host call: 8 GB of FP64 A per block, two pinned host buffers
EV = 23.0605   # kcal/mol per eV


def workload_desc(nframes):
    return (f"{nframes} frames x 256 C/H/N/O atoms, triclinic a,b,c in [12,16] A, angles in [80,100] deg, "
            f"Morse + Axilrod-Teller labels; Chebyshev 2B16@5.0 / 3B8@4.0 / 4B4@3.5, force + full stress + "
            f"energy rows, A {780 * nframes} x 51209")


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs", 6800.0), d.get("bf16_tflops", 1900.0), "measured"
    return 6800.0, 1900.0, "fallback"


class ClockSampler:
    """nvidia-smi sampling of SM clock and throttle reasons during a timed region."""

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
        return self

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


def make_fit_workload(tmp, nframes, seed):
    synth = importlib.import_module("chimes_lsq-myllfork_gb300.synth")
    return synth.make_workload(WORKLOAD, tmp, nframes=nframes, seed=seed, workers=min(16, cpu_threads()))


def time_oracle(fm, nframes_sample, threads):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build() if not os.path.exists(oracle.LIB) else None
    t = time.perf_counter()
    A, _ = oracle.assemble(fm, nframes=nframes_sample, first=0, count=nframes_sample, nthreads=threads)
    dt = time.perf_counter() - t
    return A.shape[0] / dt, A.shape[0], dt


def reference_arm(args, rank, world):
    """The reference algorithm on the host cores: the oracle port, every thread one
    frame of a bounded sample per step."""
    if rank != 0:
        return
    tmp = tempfile.mkdtemp(prefix="chimes_ref_")
    threads = cpu_threads()
    sample = max(1, min(threads, 16))
    synth = importlib.import_module("chimes_lsq-myllfork_gb300.synth")
    fm = synth.make_workload(WORKLOAD, tmp, nframes=sample, seed=2024, labels=False)
    for _ in range(args.warmup):
        time_oracle(fm, sample, threads)
    rows, secs = 0, 0.0
    for _ in range(args.steps):
        _, n, dt = time_oracle(fm, sample, threads)
        rows += n
        secs += dt
    value = rows / secs
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "rows/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * secs / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "desc": workload_desc(NFRAMES), "sample_frames_per_step": sample},
        "cpu_baseline": {"value": value, "unit": "rows/s", "cores": threads, "kind": "port",
                         "sample": f"{sample} frames of the workload per step (OpenMP over frames, one per thread)"},
        "e2e": {"value": value, "unit": "rows/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


class Timer:
    """CUDA events on the session stream."""

    def __init__(self, torch, stream):
        self.torch, self.stream = torch, stream

    def __call__(self, fn):
        t = self.torch
        t.cuda.synchronize()
        e0, e1 = t.cuda.Event(enable_timing=True), t.cuda.Event(enable_timing=True)
        e0.record(self.stream)
        fn()
        e1.record(self.stream)
        t.cuda.synchronize()
        return e0.elapsed_time(e1) / 1e3


def traffic_per_frame(kernel_stage):
    """DRAM bytes per frame of a stage's kernels from the committed ncu summary data
    (profiles/traffic.json: one capture of a few frames of this workload)."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(p):
        return None, None
    d = json.load(open(p)).get(WORKLOAD, {}).get(kernel_stage)
    if not d:
        return None, None
    return d["dram_bytes"] / d["frames"], d["source"]


def fit_bench(cg, sess, model, blocks, dblocks, asm64_s, timer, torch, args):
    """The spec comparison on the 4-body workload, every row of it.
    mixed: FP32 assembly + split-BF16 Gram (one pass over the row blocks), FP64
    Cholesky of G + ridge I, FP64 CG passes over re-assembled row blocks until the
    relative update is below 1e-10.  plain: FP64 assembly (the headline step) + FP64
    SYRK Gram (timed on a slice of all 51,209 columns and 8,192 rows, scaled per row)
    + the same FP64 Cholesky.  The FP64-converged solution (CG continued to a
    relative update of 1e-14) is the reference of the coefficient and force errors."""
    import numpy as np
    C = model.ncols
    R = sum(b.nrows for b in blocks)
    maxrows = max(b.nrows for b in blocks)
    labels = [torch.from_numpy(b.labels()).cuda() for b in blocks]
    clocks = ClockSampler(torch.cuda.current_device()).start()
    G = torch.zeros((C, C), dtype=torch.float64, device="cuda")
    h = torch.zeros(C, dtype=torch.float64, device="cuda")
    A32 = torch.empty((maxrows, C), dtype=torch.float32, device="cuda")
    sess.assemble_device(dblocks[0], cg.CG_FP32, A32.data_ptr(), C)   # warm
    sess.profile(True)
    t_asm32 = t_gram = 0.0
    for b, d, lab in zip(blocks, dblocks, labels):
        t_asm32 += timer(lambda: sess.assemble_device(d, cg.CG_FP32, A32.data_ptr(), C))
        t_gram += timer(lambda: sess.gram(1, A32.data_ptr(), C, b.nrows, C, lab.data_ptr(), 1, G.data_ptr(),
                                          h.data_ptr()))
    st = sess.stage_times()
    sess.profile(False)
    del A32
    torch.cuda.empty_cache()
    t_gram += timer(lambda: sess.gram_finish(G.data_ptr(), C))
    lam = 1e-6 * float(torch.diagonal(G).abs().max())
    L = torch.empty((C, C), dtype=torch.float64, device="cuda")
    x = torch.zeros(C, dtype=torch.float64, device="cuda")
    t0 = time.perf_counter()
    used = sess.cholesky(G.data_ptr(), C, lam, L.data_ptr())
    t_chol = time.perf_counter() - t0
    del G
    torch.cuda.empty_cache()
    t_cs = timer(lambda: sess.cholesky_solve(L.data_ptr(), C, h.data_ptr(), x.data_ptr()))
    x_direct = x.clone()
    lab_ptrs = [l.data_ptr() for l in labels]
    sess.profile(True)
    t0 = time.perf_counter()
    info = sess.refine_streamed(L.data_ptr(), C, lam, dblocks, lab_ptrs, x.data_ptr(), max_iters=40, tol=1e-10)
    t_ref = time.perf_counter() - t0
    rst = sess.stage_times()
    sess.profile(False)
    ref_stages = {k: v[0] / 1e3 for k, v in rst.items() if v[1]}
    x_mixed = x.clone()
    info_c = sess.refine_streamed(L.data_ptr(), C, lam, dblocks, lab_ptrs, x.data_ptr(), max_iters=30, tol=1e-14)
    x_conv = x.clone()
    del L
    torch.cuda.empty_cache()
    rel = lambda u, v: float(torch.linalg.norm(u - v) / torch.linalg.norm(v))
    # force rows: 768 of every frame's 780 rows (256 atoms x 3, then 9 stress + 3 energy rows)
    y = torch.empty(R, dtype=torch.float64, device="cuda")
    sess.predict_streamed(dblocks, (x_mixed - x_conv).data_ptr(), y.data_ptr())
    force = torch.zeros(R, dtype=torch.bool, device="cuda")
    r0 = 0
    for b in blocks:
        for f in range(b.nframes):
            force[r0 + 780 * f: r0 + 780 * f + 768] = True
        r0 += b.nrows
    dF = float(torch.sqrt(torch.mean(y[force] ** 2))) / EV
    del y
    # plain form: FP64 SYRK on a slice of all columns, scaled per row
    Abuf = torch.empty((maxrows, C), dtype=torch.float64, device="cuda")
    sess.assemble_device(dblocks[0], cg.CG_FP64, Abuf.data_ptr(), C)
    K = min(8192, blocks[0].nrows)
    Gs = torch.zeros((C, C), dtype=torch.float64, device="cuda")
    hs = torch.zeros(C, dtype=torch.float64, device="cuda")
    reps = [timer(lambda: sess.gram(0, Abuf.data_ptr(), C, K, C, labels[0].data_ptr(), 0, Gs.data_ptr(),
                                    hs.data_ptr())) for _ in range(2)]
    del Gs, hs, Abuf
    torch.cuda.empty_cache()
    clk = clocks.stop()
    t_gram64 = statistics.mean(reps) / K * R
    flops = R * C * (C + 1)
    _, bf16, kind = measured_peaks()
    tc_ms = st.get("gram_tensor", (0.0, 0))[0]
    plain = asm64_s + t_gram64 + t_chol + t_cs
    mixed = t_asm32 + t_gram + t_chol + t_cs + t_ref
    out = {
        "workload": f"{WORKLOAD}: " + workload_desc(sum(b.nframes for b in blocks)),
        "rows": R, "cols": C, "ridge": lam, "ridge_rule": "1e-6 * max_i (A^T A)_ii",
        "mixed": {"assembly_fp32_s": t_asm32, "gram_bf16x3_s": t_gram, "cholesky_fp64_s": t_chol,
                  "cholesky_solve_s": t_cs, "refine_fp64_s": t_ref, "refine_passes": info["iters"],
                  "refine_last_rel_update": info["rel_update"], "refine_stages_s": ref_stages, "total_s": mixed,
                  "rows_per_s_assembly_plus_gram": R / (t_asm32 + t_gram)},
        "plain": {"assembly_fp64_s": asm64_s, "gram_fp64_s": t_gram64,
                  "gram_fp64_timing": f"FP64 SYRK of {K} rows x all {C} columns, {len(reps)} repeats "
                                      f"({', '.join('%.2f s' % r for r in reps)}), scaled per row (extrapolated)",
                  "gram_fp64_tflops": K * C * (C + 1) / statistics.mean(reps) / 1e12,
                  "cholesky_fp64_s": t_chol, "cholesky_solve_s": t_cs, "total_s": plain,
                  "rows_per_s_assembly_plus_gram": R / (asm64_s + t_gram64)},
        "speedup_assembly_plus_gram_mixed_vs_plain": (asm64_s + t_gram64) / (t_asm32 + t_gram),
        "speedup_fit_mixed_vs_plain": plain / mixed,
        "coef_rel_err": rel(x_mixed, x_conv),
        "coef_rel_err_without_refinement": rel(x_direct, x_conv),
        "force_rmse_diff_eVA": dF,
        "force_rmse_note": "RMS over the 768,000 force rows of A (x_mixed - x_fp64) in eV/A, which bounds the "
                           "difference of the two fits' force RMSE",
        "fp64_reference": f"the same ridge system solved by FP64 CG passes to a relative update of "
                          f"{info_c['rel_update']:.1e} ({info['iters'] + info_c['iters']} passes in all)",
        "cholesky_ridge_used": used,
        "roofline_gram": {"bound": "tensor", "kernel": "k_gram_tc (split-BF16 3-term, tcgen05)",
                          "achieved": flops / (tc_ms / 1e3) / 1e12 if tc_ms else None, "peak": bf16 / 3.0,
                          "unit": "TFLOP/s", "frac": (flops / (tc_ms / 1e3) / 1e12) / (bf16 / 3.0) if tc_ms else None,
                          "kernel_s": tc_ms / 1e3, "flops": flops,
                          "peak_source": f"{kind} bf16 dense burst / 3 (three BF16 products per FP32-accurate one)"},
        "gram_stages_s": {k: v[0] / 1e3 for k, v in st.items() if k.startswith("gram") and v[1]},
        "clocks": clk,
    }
    return out


def batched_bench(cg, local, nframes, timer, torch, eager_blocks=4, per_frame_sample=24):
    """Batched form: frames with log-uniform 32-1024 atoms, 4 species, cubic boxes at
    0.1 atoms/A^3, the 4-body basis (51,209 columns).  One CUDA graph replays every
    block's FP32 assembly and split-BF16 Gram; block size from the autotuner.  Against:
    the same blocks launched eagerly (no graph) and the frames one at a time."""
    import numpy as np
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
    t0 = time.perf_counter()
    choice, trials = autotune.tune_batch(cg, sess, frames, sizes, block_candidates=(16, 32, 64), sample_frames=64,
                                         repeats=1, torch=torch)
    tune_s = time.perf_counter() - t0
    for k in ("gram_ctas_per_sm", "force4_threads", "gram_rows_per_launch"):
        sess.tune(k, choice[k])
    bf = choice["block_frames"]
    blocks = [frames.slice(f0, min(bf, nframes - f0)) for f0 in range(0, nframes, bf)]
    rows = sum(b.nrows for b in blocks)
    maxrows = max(b.nrows for b in blocks)
    A = torch.empty((maxrows, C), dtype=torch.float32, device="cuda")
    G = torch.zeros((C, C), dtype=torch.float64, device="cuda")
    h = torch.zeros(C, dtype=torch.float64, device="cuda")
    dfs = [sess.upload(b) for b in blocks]
    labels = [torch.from_numpy(b.labels()).cuda() for b in blocks]
    clocks = ClockSampler(local).start()
    t0 = time.perf_counter()
    g = sess.batch_fit(dfs, [l.data_ptr() for l in labels], cg.CG_FP32, A.data_ptr(), C, G.data_ptr(), h.data_ptr())
    build_s = time.perf_counter() - t0
    G.zero_()
    h.zero_()
    graph_s = timer(g.launch)
    del g
    # the first blocks launched eagerly (same kernels, no graph)
    ne = min(eager_blocks, len(blocks))
    eager_s = timer(lambda: [(sess.assemble_device(dfs[k], cg.CG_FP32, A.data_ptr(), C),
                              sess.gram(1, A.data_ptr(), C, blocks[k].nrows, C, labels[k].data_ptr(), 1,
                                        G.data_ptr(), h.data_ptr())) for k in range(ne)])
    eager_rows = sum(blocks[k].nrows for k in range(ne))
    # frames one at a time on a sample
    nper = min(per_frame_sample, nframes)
    single = [frames.slice(f, 1) for f in range(nper)]
    d1 = [sess.upload(x) for x in single]
    l1 = [torch.from_numpy(x.labels()).cuda() for x in single]
    per_s = timer(lambda: [(sess.assemble_device(d, cg.CG_FP32, A.data_ptr(), C),
                            sess.gram(1, A.data_ptr(), C, x.nrows, C, l.data_ptr(), 1, G.data_ptr(), h.data_ptr()))
                           for x, d, l in zip(single, d1, l1)])
    rows_per = sum(x.nrows for x in single)
    clk = clocks.stop()
    hbm, bf16, kind = measured_peaks()
    cpad = (C + 127) // 128 * 128
    bytes_per_row = 4 * C + 4 * C + 4 * cpad + 4 * cpad   # A write, A read by the split, planes write + read
    flops = rows * C * (C + 1)
    return {
        "workload": f"{nframes} frames, N log-uniform in [32, 1024] (mean {sizes.mean():.0f}), 4 species, cubic "
                    f"0.1/A^3, 2B16@5.0 / 3B8@4.0 / 4B4@3.5, {rows} rows x {C} columns",
        "graph": {"rows_per_s": rows / graph_s, "seconds": graph_s, "blocks": len(blocks), "block_frames": bf,
                  "capture_and_sizing_s": build_s,
                  "hbm_gbs_algorithmic": rows * bytes_per_row / graph_s / 1e9, "hbm_peak_gbs": hbm,
                  "gram_tflops_algorithmic": flops / graph_s / 1e12, "bf16_peak_over_3": bf16 / 3.0},
        "eager_blocks": {"rows_per_s": eager_rows / eager_s, "blocks": ne, "seconds": eager_s},
        "per_frame": {"rows_per_s": rows_per / per_s, "frames": nper, "seconds": per_s},
        "speedup_graph_vs_eager_blocks": (rows / graph_s) / (eager_rows / eager_s),
        "speedup_graph_vs_per_frame": (rows / graph_s) / (rows_per / per_s),
        "autotune": {"choice": choice, "seconds": tune_s, "trials": trials},
        "clocks": clk,
        "note": "bytes per row: FP32 A write + read by the BF16 split + BF16 hi/lo planes write + read",
    }


def md_bench(cg, local):
    """MD serving on the Poisson-arrival, 64-4096-atom, 4-species, 4-body workload:
    a bounded arrival window, 100 NVE steps per request, batched FP64 and
    FP32-contraction serving against the same requests served one at a time in FP64."""
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
    for name, prec, cap, frames_cap in (("batched_fp64", 0, 16384, 1024), ("batched_fp32", 1, 16384, 1024),
                                        ("batched_fp32_cap4096", 1, 4096, 1024), ("one_at_a_time_fp64", 0, 1 << 16, 1)):
        sess = cg.Session(model, local)
        sess.md_setup(x, precision=prec)
        outs, res, step_ms, nb = sess.md_serve(reqs, masses, dt_fs=0.2, max_batch_atoms=cap,
                                               max_batch_frames=frames_cap)
        t_first = min(r["arrival"] for r in reqs)
        span = float(res["finished"].max() - t_first)
        sm = step_ms.reshape(-1)
        lat = res["finished"] - np.array([r["arrival"] for r in reqs])
        d = {"value": float(sizes.sum() * nsteps / span), "batched_steps": int(nb), "requests": nreq,
             "max_batch_atoms": cap if frames_cap > 1 else "one request",
             "step_ms_p50": float(np.percentile(sm, 50)), "step_ms_p99": float(np.percentile(sm, 99)),
             "request_latency_s_p50": float(np.percentile(lat, 50)),
             "request_latency_s_p99": float(np.percentile(lat, 99)),
             "reserved_gb_max": float(res["reserved_bytes"].max() / 1e9)}
        if sel.any():
            d["step_ms_p50_1024atom"] = float(np.percentile(step_ms[sel].reshape(-1), 50))
            d["step_ms_p99_1024atom"] = float(np.percentile(step_ms[sel].reshape(-1), 99))
        out[name] = d
    out["speedup_batched_fp32_cap4096_vs_one_at_a_time_fp64"] = (out["batched_fp32_cap4096"]["value"] /
                                                                  out["one_at_a_time_fp64"]["value"])
    # the same requests through the live server: a client thread submits each one at its
    # arrival time while the server's thread runs the batches (FP32 form, 4096-atom cap)
    import threading
    sess = cg.Session(model, local)
    sess.md_setup(x, precision=1)
    srv = sess.md_server(masses, dt_fs=0.2, max_batch_atoms=4096, max_batch_frames=1024)
    submitted, tickets = [], []
    t0 = time.perf_counter()

    def client():
        for q in reqs:
            w = q["arrival"] - (time.perf_counter() - t0)
            if w > 0:
                time.sleep(w)
            submitted.append(time.perf_counter() - t0)
            tickets.append(srv.submit(q["types"], q["xyz"], q["cell"], q["v"], q["nsteps"]))

    th = threading.Thread(target=client)
    th.start()
    done = [None] * nreq
    left = nreq
    while left:   # non-blocking polls of every submitted ticket: completion seen within ~0.2 ms
        for k in range(len(tickets)):
            if done[k] is None and srv.poll(tickets[k]) is not None:
                done[k] = time.perf_counter() - t0
                left -= 1
        time.sleep(0.0002)
    th.join()
    nb = srv.stop()
    lat = np.array(done) - np.array(submitted)
    out["live_server_fp32_cap4096"] = {
        "value": float(sizes.sum() * nsteps / (max(done) - min(submitted))), "batched_steps": int(nb),
        "requests": nreq, "request_latency_s_p50": float(np.percentile(lat, 50)),
        "request_latency_s_p99": float(np.percentile(lat, 99)),
        "note": "cg_md_server_*: submissions from a client thread at the arrival times while the server thread "
                "runs; latency = completion seen by non-blocking polls - submission"}
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


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--frames", type=int, default=NFRAMES, help="frames per rank (1000 = the full workload)")
    ap.add_argument("--block-frames", type=int, default=BLOCK_FRAMES)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fit", action="store_true", help="skip the mixed-vs-plain fit comparison")
    ap.add_argument("--no-md", action="store_true")
    ap.add_argument("--batched", type=int, default=4096, metavar="FRAMES",
                    help="frames of the batched form (0 skips it)")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return reference_arm(args, rank, world)

    # inputs first (label generation in spawned processes), then the GPU
    tmp = tempfile.mkdtemp(prefix="chimes_bench_")
    fm = make_fit_workload(tmp, args.frames, 2024 + rank)   # weak scaling: own frames per rank
    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    cg = importlib.import_module("chimes_lsq-myllfork_gb300")
    model = cg.Model(fm)
    frames = cg.Frames.read(model)
    sess = cg.Session(model, local)
    stream = torch.cuda.ExternalStream(sess.stream)
    timer = Timer(torch, stream)
    C = model.ncols
    nrows, natoms = frames.rows()
    bf = args.block_frames
    blocks = [frames.slice(f0, min(bf, args.frames - f0)) for f0 in range(0, args.frames, bf)]
    dblocks = [sess.upload(b) for b in blocks]
    maxrows = max(b.nrows for b in blocks)
    A = torch.empty((maxrows, C), dtype=torch.float64, device="cuda")

    def step():
        for d in dblocks:
            sess.assemble_device(d, cg.CG_FP64, A.data_ptr(), C)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    clocks = ClockSampler(local).start()
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
    launches = sess.last_launches() * len(dblocks) * args.steps
    if dist:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = world * nrows * args.steps / (ms / 1000.0)
    asm64_s = ms / 1000.0 / args.steps

    # per-stage device time of one step (CUDA events on the session stream) and the
    # work counters of the whole step
    sess.profile(True)
    counts = {}
    for d in dblocks:
        sess.assemble_device(d, cg.CG_FP64, A.data_ptr(), C)
        for k, v in sess.last_counts().items():
            counts[k] = counts.get(k, 0) + v
    stages = sess.stage_times()
    sess.profile(False)
    del A
    torch.cuda.empty_cache()
    fp64_peak = sess.fp64_fma_rate()
    cols = model.columns()
    force_rows = 3 * natoms
    vir_rows = nrows - force_rows
    hbm_peak, _, peak_kind = measured_peaks()
    stage_ms = {k: v[0] for k, v in stages.items() if v[1]}
    dom = max(stage_ms, key=stage_ms.get)
    dom_s = stage_ms[dom] / 1e3
    # algorithmic bytes: the A entries each stage owns (FP64); FP64 work: 3 FMAs per
    # (cluster, member, power) in the force rows, 13 per (cluster, power) in the
    # stress / energy rows (factorised basis products)
    bytes_by_stage = {"force_4b": force_rows * cols["n4b"] * 8, "virial_4b": vir_rows * cols["n4b"] * 8,
                      "force_3b": force_rows * cols["n3b"] * 8, "virial_3b": vir_rows * cols["n3b"] * 8,
                      "force_2b": force_rows * cols["n2b"] * 8, "virial_2b": vir_rows * cols["n2b"] * 8}
    flops_by_stage = {"force_4b": counts["evals4"] * 4 * 3 * 2, "virial_4b": counts["evals4"] * 13 * 2,
                      "force_3b": counts["evals3"] * 3 * 3 * 2, "virial_3b": counts["evals3"] * 13 * 2}
    algo = bytes_by_stage.get(dom, nrows * C * 8)
    tpf, tsrc = traffic_per_frame(dom)
    roofline = {"bound": "hbm", "kernel": dom, "achieved": algo / dom_s / 1e9, "peak": hbm_peak, "unit": "GB/s",
                "frac": algo / dom_s / 1e9 / hbm_peak, "traffic": None if tpf is None else tpf * args.frames,
                "traffic_source": tsrc, "bytes_per_launch": algo, "peak_source": peak_kind,
                "note": "the FP64 assembly kernels are FP64-pipe bound: see fp64"}
    # the bound that holds for the dominant kernel: its FP64 work against the FP64 rate
    # measured in this run (the better of an FMA-chain kernel and the FP64 SYRK)
    roofline_fp64 = None
    if dom in flops_by_stage:
        ach = flops_by_stage[dom] / dom_s / 1e12
        roofline_fp64 = {"bound": "fp64", "kernel": dom, "achieved": ach, "peak": fp64_peak, "unit": "TFLOP/s",
                         "frac": ach / fp64_peak, "flops_per_step": flops_by_stage[dom],
                         "peak_source": "measured in this run (cg_fp64_fma_rate)"}
    fp64 = {"measured_fma_peak_tflops": fp64_peak,
            "stages": {k: {"s": stage_ms[k] / 1e3, "tflops": flops_by_stage[k] / (stage_ms[k] / 1e3) / 1e12,
                           "frac_of_measured_peak": flops_by_stage[k] / (stage_ms[k] / 1e3) / 1e12 / fp64_peak}
                       for k in flops_by_stage if k in stage_ms}}

    # end to end through the C ABI: host frames in, every A block to pinned host memory
    e2e_steps = min(args.steps, 2)
    sink_rows = [0]

    def sink(first, blk):
        sink_rows[0] += blk.shape[0]
        return False
    # two untimed calls: the first allocates the pinned staging (two cudaMallocHost
    # buffers of one block each) and the device blocks
    for _ in range(2):
        sess.assemble_stream(frames, cg.CG_FP64, sink, block_frames=E2E_BLOCK_FRAMES)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        sess.assemble_stream(frames, cg.CG_FP64, sink, block_frames=E2E_BLOCK_FRAMES)
    e2e_s = time.perf_counter() - t0
    # one more streamed call with stage timing: the device time of the block copies
    # (copy stream) beside the assembly stages, against the call's wall time
    sess.profile(True)
    t1 = time.perf_counter()
    sess.assemble_stream(frames, cg.CG_FP64, sink, block_frames=E2E_BLOCK_FRAMES)
    diag_wall = time.perf_counter() - t1
    diag = {k: v[0] for k, v in sess.stage_times().items() if v[1]}
    sess.profile(False)
    # the host link's device-to-host rate in this run (pinned destination), the
    # ceiling of the streamed call
    link = torch.empty(1 << 29, dtype=torch.float64, device="cuda")
    pin = torch.empty(1 << 29, dtype=torch.float64, pin_memory=True)
    pin.copy_(link, non_blocking=True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(3):
        pin.copy_(link, non_blocking=True)
    torch.cuda.synchronize()
    link_gbs = 3 * link.numel() * 8 / (time.perf_counter() - t0) / 1e9
    del link, pin
    e2e = {"value": world * nrows * e2e_steps / e2e_s, "unit": "rows/s", "steps": e2e_steps,
           "d2h_link_gbs_measured": link_gbs, "d2h_gbs_achieved": nrows * C * 8 * e2e_steps / e2e_s / 1e9,
           "h2d_bytes_per_step": int(natoms * (3 * 8 + 4) + args.frames * (4 + 3 * 8 + 2 * 4 + 208)),
           "d2h_bytes_per_step": int(nrows * C * 8),
           "call": f"cg_assemble_stream (FP64, blocks of {E2E_BLOCK_FRAMES} frames, pinned double buffer, no-op sink)",
           "profiled_call": {"wall_s": diag_wall, "host_copies_s": diag.get("host_copies", 0.0) / 1e3,
                             "copy_gbs_device": nrows * C * 8 / (diag["host_copies"] / 1e3) / 1e9
                             if diag.get("host_copies") else None,
                             "assembly_stages_s": sum(v for k, v in diag.items() if k != "host_copies") / 1e3}}

    fit = None
    if rank == 0 and not args.no_fit:
        fit = fit_bench(cg, sess, model, blocks, dblocks, asm64_s, timer, torch, args)
    del dblocks
    torch.cuda.empty_cache()
    batched = None
    if rank == 0 and args.batched > 0:
        batched = batched_bench(cg, local, args.batched, timer, torch)
        torch.cuda.empty_cache()
    md = None
    if rank == 0 and not args.no_md:
        md = md_bench(cg, local)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        th = cpu_threads()
        sample = max(1, min(th, 16))
        r, n, dt = time_oracle(fm, sample, th)
        cpu = {"value": r, "unit": "rows/s", "cores": th, "kind": "port",
               "sample": f"first {sample} of the {args.frames} frames ({n} rows, {dt:.1f} s wall, OpenMP over frames)"}
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "rows/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "desc": workload_desc(args.frames), "rows_per_step": nrows, "cols": C,
                       "block_frames": bf, "l2": "each step writes 320 GB of A (> 129 MB L2); no flush needed",
                       "parallelism": f"frames sharded, {world} rank(s), no collective"},
            "clocks": clk, "e2e": e2e, "gpu_launches": launches, "roofline": roofline, "roofline_fp64": roofline_fp64,
            "fp64": fp64,
            "stages_s_per_step": {k: v / 1e3 for k, v in stage_ms.items()}, "work": counts,
            "cpu_baseline": cpu, "fit4b": fit, "batched": batched, "md": md,
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
