"""Small, fixed workloads for profiling single kernels under ncu.

    python profile_cases.py gram [nframes]        # split-BF16 Gram of water-3b A
    python profile_cases.py md NATOMS PRECISION   # MD force of one 4-body system
    python profile_cases.py assemble [nframes] [fp32] [form=N]  # A of water-3b frames
    python profile_cases.py assemble4b [nframes] [fp32] [form=N]  # A of 256-atom C/H/N/O 4-body frames
    python profile_cases.py gram4b [rows]         # split-BF16 Gram of a 4-body FP32 A (51,209 columns)
    python profile_cases.py syrk [rows] [cols]    # FP64 SYRK Gram of a random A
    python profile_cases.py gramrand [rows] [cols]  # split-BF16 Gram of a random FP32 A
    python profile_cases.py cholesky [n] [tensor]   # blocked Cholesky of a random SPD matrix
    python profile_cases.py serve NATOMS PRECISION NSTEPS  # one NVE request, stage times
    python profile_cases.py forms4b [nframes]     # both force-row forms: stage times, agreement

Each case runs its launch twice after the set-up, so `ncu -k regex:<kernel> -c 1`
captures a warm launch; the synthetic inputs are seeded.  form=N sets the session's
force_range tunable (0: the per-power force kernel k_force_mb, 2: the range form
k_force_rg everywhere; default 1).
"""
import importlib
import os
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)


def main(argv):
    cg = importlib.import_module("chimes_lsq-myllfork_gb300")
    synth = importlib.import_module("chimes_lsq-myllfork_gb300.synth")
    import numpy as np
    import torch
    form = [int(a.split("=", 1)[1]) for a in argv if a.startswith("form=")]
    argv = [a for a in argv if not a.startswith("form=")]
    case = argv[0] if argv else "md"
    tmp = tempfile.mkdtemp(prefix="chimes_prof_")
    if case in ("gram", "assemble"):
        nframes = int(argv[1]) if len(argv) > 1 else 200
        fm = synth.make_workload("water-3b", tmp, nframes=nframes, seed=1000)
        model = cg.Model(fm)
        fr = cg.Frames.read(model)
        sess = cg.Session(model, 0)
        if form:
            sess.tune("force_range", form[0])
        nrows, _ = fr.rows()
        ncols = model.ncols
        dfr = sess.upload(fr)
        fp32 = case == "gram" or (len(argv) > 2 and argv[2] == "fp32")
        prec = cg.CG_FP32 if fp32 else cg.CG_FP64
        A = torch.empty((nrows, ncols), dtype=torch.float32 if fp32 else torch.float64, device="cuda")
        for _ in range(1 if case == "gram" else 2):
            sess.assemble_device(dfr, prec, A.data_ptr(), ncols)
        if case == "gram":
            b = torch.from_numpy(fr.labels()).cuda()
            G = torch.zeros((ncols, ncols), dtype=torch.float64, device="cuda")
            h = torch.zeros(ncols, dtype=torch.float64, device="cuda")
            for _ in range(2):
                sess.gram(1, A.data_ptr(), ncols, nrows, ncols, b.data_ptr(), 1, G.data_ptr(), h.data_ptr())
        torch.cuda.synchronize()
        print("ok", case, nrows, ncols)
        return
    if case == "forms4b":   # the range and per-power forms of the force rows, FP64 and FP32
        nframes = int(argv[1]) if len(argv) > 1 else 50
        fm = synth.make_workload("chno-4b", tmp, nframes=nframes, seed=2024, labels=False)
        model = cg.Model(fm)
        fr = cg.Frames.read(model)
        sess = cg.Session(model, 0)
        nrows, _ = fr.rows()
        ncols = model.ncols
        dfr = sess.upload(fr)
        for prec, dt in ((cg.CG_FP64, torch.float64), (cg.CG_FP32, torch.float32)):
            outs = {}
            for form in (2, 0):
                sess.tune("force_range", form)
                A = torch.empty((nrows, ncols), dtype=dt, device="cuda")
                sess.assemble_device(dfr, prec, A.data_ptr(), ncols)
                sess.profile(True)
                for _ in range(3):
                    sess.assemble_device(dfr, prec, A.data_ptr(), ncols)
                torch.cuda.synchronize()
                st = sess.stage_times()
                sess.profile(False)
                outs[form] = A
                ms = {k: round(v[0] / 3, 2) for k, v in st.items() if k.startswith(("force", "virial"))}
                print(f"prec {prec} force_range {form} ms per assembly of {nframes} frames: {ms}", flush=True)
            d = (outs[2].double() - outs[0].double()).abs().max().item()
            print(f"prec {prec}: max |range - per-power| / max |A| = {d / outs[0].double().abs().max().item():.3e}",
                  flush=True)
            del outs
        print("ok", case, nrows, ncols)
        return
    if case in ("assemble4b", "gram4b"):
        nframes = int(argv[1]) if len(argv) > 1 and case == "assemble4b" else 4
        fm = synth.make_workload("chno-4b", tmp, nframes=nframes, seed=2024, labels=case == "gram4b")
        model = cg.Model(fm)
        fr = cg.Frames.read(model)
        sess = cg.Session(model, 0)
        if form:
            sess.tune("force_range", form[0])
        nrows, _ = fr.rows()
        ncols = model.ncols
        dfr = sess.upload(fr)
        fp32 = case == "gram4b" or (len(argv) > 2 and argv[2] == "fp32")
        prec = cg.CG_FP32 if fp32 else cg.CG_FP64
        A = torch.empty((nrows, ncols), dtype=torch.float32 if fp32 else torch.float64, device="cuda")
        for _ in range(1 if case == "gram4b" else 2):
            sess.assemble_device(dfr, prec, A.data_ptr(), ncols)
        if case == "gram4b":   # rows: repeat the frames' rows up to the requested K
            rows = int(argv[1]) if len(argv) > 1 else 8192
            reps = (rows + nrows - 1) // nrows
            Ar = A.repeat(reps, 1)[:rows].contiguous()
            b = torch.from_numpy(np.tile(fr.labels(), reps)[:rows].copy()).cuda()
            G = torch.zeros((ncols, ncols), dtype=torch.float64, device="cuda")
            h = torch.zeros(ncols, dtype=torch.float64, device="cuda")
            for _ in range(2):
                sess.gram(1, Ar.data_ptr(), ncols, rows, ncols, b.data_ptr(), 1, G.data_ptr(), h.data_ptr())
        torch.cuda.synchronize()
        print("ok", case, nrows, ncols)
        return
    if case == "gramrand":
        rows = int(argv[1]) if len(argv) > 1 else 16384
        cols = int(argv[2]) if len(argv) > 2 else 8192
        fm = synth.make_workload("water-2b", tmp, nframes=1, seed=3)
        sess = cg.Session(cg.Model(fm), 0)
        A = torch.randn(rows, cols, dtype=torch.float32, device="cuda")
        b = torch.randn(rows, dtype=torch.float64, device="cuda")
        G = torch.zeros((cols, cols), dtype=torch.float64, device="cuda")
        h = torch.zeros(cols, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        for _ in range(2):
            sess.gram(1, A.data_ptr(), cols, rows, cols, b.data_ptr(), 1, G.data_ptr(), h.data_ptr())
        torch.cuda.synchronize()
        print("ok", case, rows, cols)
        return
    if case == "cholesky":   # one factorisation; tensor = 1: tensor-core trailing updates
        n = int(argv[1]) if len(argv) > 1 else 8192
        tensor = int(argv[2]) if len(argv) > 2 else 1
        fm = synth.make_workload("water-2b", tmp, nframes=1, seed=3)
        sess = cg.Session(cg.Model(fm), 0)
        gen = torch.Generator(device="cuda").manual_seed(11)
        X = torch.randn(n + 256, n, dtype=torch.float64, device="cuda", generator=gen)
        G = X.T @ X
        del X
        G += 1e-3 * torch.diag(torch.diagonal(G))
        L = torch.empty_like(G)
        sess.tune("cholesky_tensor_updates", tensor)
        sess.cholesky(G.data_ptr(), n, 0.0, L.data_ptr())
        torch.cuda.synchronize()
        print("ok", case, n, tensor)
        return
    if case == "syrk":
        rows = int(argv[1]) if len(argv) > 1 else 8192
        cols = int(argv[2]) if len(argv) > 2 else 8192
        fm = synth.make_workload("water-2b", tmp, nframes=1, seed=3)
        sess = cg.Session(cg.Model(fm), 0)
        A = torch.randn(rows, cols, dtype=torch.float64, device="cuda")
        b = torch.randn(rows, dtype=torch.float64, device="cuda")
        G = torch.zeros((cols, cols), dtype=torch.float64, device="cuda")
        h = torch.zeros(cols, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        for _ in range(2):
            sess.gram(0, A.data_ptr(), cols, rows, cols, b.data_ptr(), 0, G.data_ptr(), h.data_ptr())
        torch.cuda.synchronize()
        print("ok", case, rows, cols)
        return
    n = int(argv[1]) if len(argv) > 1 else 1024
    prec = int(argv[2]) if len(argv) > 2 else 0
    if case == "serve":   # one request through the serving loop (list reuse, rebuilds)
        return serve_case(cg, synth, np, torch, tmp, n, prec, int(argv[3]) if len(argv) > 3 else 100)
    fm = synth.make_workload("chno-4b", tmp, nframes=1, seed=5, sizes=[n], triclinic=False, density=0.1, labels=False)
    model = cg.Model(fm)
    nat, types, xyz, cell = synth.frames_arrays(os.path.join(tmp, "traj.xyzf"), 1, ["C", "H", "N", "O"])[:4]
    x = np.random.default_rng(1).standard_normal(model.ncols) * 1e-3
    fr = cg.Frames.from_arrays(model, nat, types, xyz, cell).independent()
    sess = cg.Session(model, 0)
    sess.md_setup(x, precision=prec)
    dfr = sess.upload(fr)
    F = torch.zeros(3 * n, dtype=torch.float64, device="cuda")
    S = torch.zeros(11, dtype=torch.float64, device="cuda")
    for _ in range(2):
        sess.md_force_device(dfr, F.data_ptr(), S.data_ptr())
    torch.cuda.synchronize()
    print("ok", case, sess.md_last_counts())


def serve_case(cg, synth, np, torch, tmp, n, prec, nsteps):
    KB = 0.0019872067
    masses = np.array([12.011, 1.008, 14.007, 15.999])
    fm = synth.make_workload("chno-4b", tmp, nframes=1, seed=21, sizes=[n], triclinic=False, density=0.1, labels=False)
    model = cg.Model(fm)
    nat, types, xyz, cell = synth.frames_arrays(os.path.join(tmp, "traj.xyzf"), 1, ["C", "H", "N", "O"])[:4]
    rng = np.random.default_rng(3)
    x = rng.standard_normal(model.ncols) * 1e-3
    v = rng.standard_normal((n, 3)) * np.sqrt(KB * 300.0 / masses[types])[:, None]
    sess = cg.Session(model, 0)
    sess.md_setup(x, precision=prec)
    req = [dict(types=types, xyz=xyz, cell=cell[0], v=v, nsteps=nsteps, arrival=0.0)]
    sess.md_serve(req, masses, dt_fs=0.2)   # warm (allocations, attributes)
    sess.profile(True)
    _, _, step_ms, _ = sess.md_serve(req, masses, dt_fs=0.2)
    st = sess.stage_times()
    sess.profile(False)
    sm = step_ms.reshape(-1)
    torch.cuda.synchronize()
    print("ok serve", n, prec, "steps", nsteps, "p50 %.3f p90 %.3f p99 %.3f max %.3f ms" % (
        np.percentile(sm, 50), np.percentile(sm, 90), np.percentile(sm, 99), sm.max()))
    print("slowest steps (index, ms):", sorted(enumerate(np.round(sm, 3).tolist()), key=lambda t: -t[1])[:12])
    for k, (ms, calls) in st.items():
        if calls:
            print(f"  {k:16s} {ms:9.3f} ms  {calls:5d} calls  {ms / calls * 1e3:8.1f} us/call")


if __name__ == "__main__":
    main(sys.argv[1:])
