"""Autotuner of the batched fit's launch shapes.

Tunes, on a sample of the batch's own frames, (a) the frames per row block (the
A buffer a block is assembled into and the K extent of each tensor-core Gram
launch), (b) the CTAs per SM the Gram aims for when it slices K (which only
matters when the column count is small), (c) the threads per CTA of the per-power
4-body force-row kernel (512 or 1024: one CTA per SM either way, shared memory
bound; it runs only when the session's "force_range" tunable is 0 -- by default the
4-body rows use the range form, whose thread count the library picks itself) and
(d) the rows of A each tensor-core Gram launch sums in FP32 (longer is faster, but
the FP32 sums lose accuracy; only lengths up to the accuracy limit are offered).
Each candidate is built as the real graph (sizing pass, capture) and timed with
CUDA events on the session stream over repeated launches; the fastest rows/s wins.
Choices are cached in a JSON file keyed by the column count and the sample's mean
frame size.
"""
import json
import os
import time


def _key(ncols, mean_atoms):
    return f"C{ncols}_N{int(round(mean_atoms / 16.0)) * 16}"


def tune_batch(cg, sess, frames, natoms, a_precision=1, block_candidates=(16, 32, 64), ctas_candidates=(4,),
               sample_frames=64, repeats=2, cache=None, torch=None, force4_candidates=(512, 1024),
               gram_rows_candidates=(0,)):
    """Returns (best dict, all trials).  frames: a cg.Frames batch; natoms: its
    per-frame atom counts (for the cache key)."""
    import numpy as np
    if torch is None:
        import torch
    ncols = frames.model.ncols
    nf = min(sample_frames, frames.nframes)
    key = _key(ncols, float(np.mean(natoms[:nf])))
    if cache and os.path.exists(cache):
        data = json.load(open(cache))
        if key in data:
            return data[key], []
    stream = torch.cuda.ExternalStream(sess.stream)
    sample = frames.slice(0, nf)
    esz = 4 if a_precision == 1 else 8
    trials = []
    for bf in block_candidates:
        blocks = [sample.slice(f0, min(bf, nf - f0)) for f0 in range(0, nf, bf)]
        maxrows = max(b.nrows for b in blocks)
        rows = sum(b.nrows for b in blocks)
        A = torch.empty((maxrows, ncols), dtype=torch.float32 if esz == 4 else torch.float64, device="cuda")
        G = torch.zeros((ncols, ncols), dtype=torch.float64, device="cuda")
        h = torch.zeros(ncols, dtype=torch.float64, device="cuda")
        dfs = [sess.upload(b) for b in blocks]
        labels = [torch.from_numpy(b.labels()).cuda() for b in blocks]
        for ctas in ctas_candidates:
            for nt4 in force4_candidates:
                for grl in gram_rows_candidates:
                    sess.tune("gram_ctas_per_sm", ctas)
                    sess.tune("force4_threads", nt4)
                    sess.tune("gram_rows_per_launch", grl)
                    t0 = time.perf_counter()
                    g = sess.batch_fit(dfs, [l.data_ptr() for l in labels], a_precision, A.data_ptr(), ncols,
                                       G.data_ptr(), h.data_ptr())
                    build_s = time.perf_counter() - t0
                    g.launch()   # warm
                    torch.cuda.synchronize()
                    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    e0.record(stream)
                    for _ in range(repeats):
                        g.launch()
                    e1.record(stream)
                    torch.cuda.synchronize()
                    ms = e0.elapsed_time(e1) / repeats
                    trials.append({"block_frames": bf, "gram_ctas_per_sm": ctas, "force4_threads": nt4,
                                   "gram_rows_per_launch": grl, "rows_per_s": rows / (ms / 1e3), "ms": ms,
                                   "graph_nodes": g.nodes, "build_s": build_s})
                    del g
        del A, G, h, dfs, labels
        torch.cuda.empty_cache()
    best = max(trials, key=lambda t: t["rows_per_s"])
    choice = {k: best[k] for k in ("block_frames", "gram_ctas_per_sm", "force4_threads", "gram_rows_per_launch")}
    if cache:
        data = json.load(open(cache)) if os.path.exists(cache) else {}
        data[key] = choice
        os.makedirs(os.path.dirname(os.path.abspath(cache)), exist_ok=True)
        json.dump(data, open(cache, "w"), indent=1)
    return choice, trials
