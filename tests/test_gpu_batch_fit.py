"""Batched fit captured as one CUDA graph (cg_batch_fit_*): uneven frames in row
blocks, assembled in FP32 and folded into the split-BF16 tensor-core Gram, replayed
by one launch.  Checked against the FP64 A^T A / A^T b of the same frames
(tolerance of the split-BF16 Gram: 1e-4 sqrt(G_ii G_jj); h from the FP32 A: 1e-6
relative), and a second launch adds the same amounts again (1e-12).  The FP64
normal equations come from the CPU oracle's A (the reference's loops restated), so the
batched form is pinned to the oracle, not to the device's own FP64 assembly."""
import importlib
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_batch_fit_graph_matches_fp64_normal_equations(cg, oracle, tmp_path):
    torch = pytest.importorskip("torch")
    synth = importlib.import_module("chimes_lsq-myllfork_gb300.synth")
    autotune = importlib.import_module("chimes_lsq-myllfork_gb300.autotune")
    sizes = [20, 48, 33, 64, 25, 40, 57, 30, 44, 36, 61, 28]
    fm = synth.make_workload("chno-4b", str(tmp_path), nframes=len(sizes), seed=77, order=(8, 4, 3), sizes=sizes,
                             triclinic=False, density=0.1)
    model = cg.Model(fm)
    frames = cg.Frames.read(model)
    sess = cg.Session(model, 0)
    C = model.ncols
    blocks = [frames.slice(f0, 4) for f0 in range(0, len(sizes), 4)]
    dfs = [sess.upload(b) for b in blocks]
    labels = [torch.from_numpy(b.labels()).cuda() for b in blocks]
    maxrows = max(b.nrows for b in blocks)
    A = torch.empty((maxrows, C), dtype=torch.float32, device="cuda")
    G = torch.zeros((C, C), dtype=torch.float64, device="cuda")
    h = torch.zeros(C, dtype=torch.float64, device="cuda")
    g = sess.batch_fit(dfs, [l.data_ptr() for l in labels], cg.CG_FP32, A.data_ptr(), C, G.data_ptr(), h.data_ptr())
    assert g.nodes > 10 * len(blocks)
    g.launch()
    torch.cuda.synchronize()
    sess.gram_finish(G.data_ptr(), C)
    G1, h1 = G.cpu().numpy().copy(), h.cpu().numpy().copy()
    A64, b64 = oracle.assemble(fm, nthreads=8)   # every frame, in order: the blocks' rows
    Gr, hr = A64.T @ A64, A64.T @ b64
    d = np.sqrt(np.maximum(np.diag(Gr), 1e-300))
    assert np.all(np.abs(G1 - Gr) <= 1e-4 * np.outer(d, d) + 1e-300)
    assert np.allclose(h1, hr, rtol=1e-6, atol=1e-6 * np.abs(hr).max())
    # replay: the same work again (G holds twice the upper triangle plus the mirror)
    G.zero_(); h.zero_()
    g.launch()
    g.launch()
    torch.cuda.synchronize()
    sess.gram_finish(G.data_ptr(), C)
    assert np.allclose(G.cpu().numpy(), 2 * G1, rtol=1e-12, atol=1e-12 * np.abs(G1).max())
    # the autotuner runs the same graphs and picks one of its candidates
    choice, trials = autotune.tune_batch(cg, sess, frames, np.array(sizes), block_candidates=(4, 6),
                                         sample_frames=12, repeats=1, torch=torch)
    assert choice["block_frames"] in (4, 6) and choice["force4_threads"] in (512, 1024) and len(trials) == 4
