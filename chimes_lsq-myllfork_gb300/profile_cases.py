"""Small, fixed workloads for profiling single kernels under ncu.

    python chimes_lsq-myllfork_gb300/profile_cases.py gram [nframes]        # split-BF16 Gram of water-3b A
    python chimes_lsq-myllfork_gb300/profile_cases.py md NATOMS PRECISION   # MD force of one 4-body system
    python chimes_lsq-myllfork_gb300/profile_cases.py assemble [nframes]    # FP64 A of water-3b frames

Each case runs its launch twice after the set-up, so `ncu -k regex:<kernel> -c 1`
captures a warm launch; the synthetic inputs are seeded.
"""
import importlib
import os
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))


def main(argv):
    cg = importlib.import_module("chimes_lsq-myllfork_gb300")
    synth = importlib.import_module("chimes_lsq-myllfork_gb300.synth")
    import numpy as np
    import torch
    case = argv[0] if argv else "md"
    tmp = tempfile.mkdtemp(prefix="chimes_prof_")
    if case in ("gram", "assemble"):
        nframes = int(argv[1]) if len(argv) > 1 else 200
        fm = synth.make_workload("water-3b", tmp, nframes=nframes, seed=1000)
        model = cg.Model(fm)
        fr = cg.Frames.read(model)
        sess = cg.Session(model, 0)
        nrows, _ = fr.rows()
        ncols = model.ncols
        dfr = sess.upload(fr)
        prec = cg.CG_FP32 if case == "gram" else cg.CG_FP64
        A = torch.empty((nrows, ncols), dtype=torch.float32 if case == "gram" else torch.float64, device="cuda")
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
    n = int(argv[1]) if len(argv) > 1 else 1024
    prec = int(argv[2]) if len(argv) > 2 else 0
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


if __name__ == "__main__":
    main(sys.argv[1:])
