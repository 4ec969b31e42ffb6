"""Fit a ChIMES force field on the GPU: the drop-in for `chimes_lsq fm_setup.in`
followed by `python chimes_lsq.py --algorithm ...` (src/chimes_lsq.C:108-424,
src/chimes_lsq.py:1-675).

    python chimes_lsq-myllfork_gb300/fit.py fm_setup.in [--algorithm ridge|lassolars|dlars|dlasso]
        [--alpha A] [--precision fp64|mixed] [--block-frames K] [--refine N] [--write-a] [--out DIR]

Writes params.header, ff_groups.map, params.txt and force.txt (and, with
--write-a, A.txt / b.txt / b-labeled.txt / natoms.txt / dim.txt) in the reference's
formats.  The design matrix is assembled on the GPU in blocks of frames and folded
into the normal equations G = A^T A, h = A^T b:
  fp64   FP64 assembly, FP64 SYRK Gram, FP64 Cholesky (ridge) or LARS;
  mixed  FP32 assembly, split-BF16 tensor-core Gram; ridge is then refined by
         preconditioned conjugate gradients on the FP64 system, each pass
         assembling the row blocks again in FP64 (no FP64 A is stored; at most
         --refine passes, stopping once the relative update is below --tol).
ridge solves (A^T A + alpha I) x = A^T b (scikit-learn Ridge(alpha,
fit_intercept=False), the reference's --algorithm ridge); lassolars follows the
LARS-lasso path to (1/2n)||b - A x||^2 + alpha ||x||_1 (the reference's
--algorithm lassolars); dlars / dlasso follow the reference's DLARS solver
(contrib/dlars, --algorithm dlars / dlasso, --normalize as its --normalize=y):
LARS or LASSO steps stopped at the first vertex where the objective with
lambda = alpha rises.
The reference's default truncated SVD is not offered: ridge with a small alpha
replaces it.
"""
import argparse
import datetime
import importlib
import math
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("fm_setup")
    ap.add_argument("--algorithm", default="ridge", choices=["ridge", "lassolars", "dlars", "dlasso"])
    ap.add_argument("--alpha", type=float, default=1.0e-3)
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    ap.add_argument("--block-frames", type=int, default=64)
    ap.add_argument("--refine", type=int, default=50, help="most CG passes of the mixed ridge solve")
    ap.add_argument("--tol", type=float, default=1e-11,
                    help="mixed ridge solve: stop once the relative size of a CG update is below this")
    ap.add_argument("--normalize", action="store_true",
                    help="dlars / dlasso: centre and scale the columns and centre b (DLARS --normalize=y)")
    ap.add_argument("--write-a", action="store_true", help="also write A.txt, b.txt, ... (slow for large A)")
    ap.add_argument("--out", default=None, help="output directory (default: the fm_setup.in directory)")
    ap.add_argument("--device", type=int, default=0)
    ap.add_argument("--weights", default=None,
                    help="row weights, one per A row (chimes_lsq.py --weights): rows of A and b are multiplied by them")
    ap.add_argument("--ranks", type=int, default=1,
                    help="order the frames and text files as `srun -n RANKS chimes_lsq` would (SKPFRMS, SPLITFI)")
    args = ap.parse_args(argv)

    import numpy as np
    import torch
    cg = importlib.import_module("chimes_lsq-myllfork_gb300")
    out = args.out or os.path.dirname(os.path.abspath(args.fm_setup))
    os.makedirs(out, exist_ok=True)
    model = cg.Model(args.fm_setup)
    open(os.path.join(out, "params.header"), "w").write(model.params_header())
    open(os.path.join(out, "ff_groups.map"), "w").write(model.ff_groups_map())
    frames = cg.Frames.read(model, nprocs=args.ranks)
    torch.cuda.set_device(args.device)
    sess = cg.Session(model, args.device)
    C = model.ncols
    nf = frames.nframes
    mixed = args.precision == "mixed"
    G = torch.zeros((C, C), dtype=torch.float64, device="cuda")
    h = torch.zeros(C, dtype=torch.float64, device="cuda")
    blocks = [frames.slice(f0, min(args.block_frames, nf - f0)) for f0 in range(0, nf, args.block_frames)]
    Acon, bcon = model.constraint_rows()   # FITCOUL charge constraints, after the last frame
    nfr_rows = sum(b.nrows for b in blocks)
    nrows = nfr_rows + Acon.shape[0]
    fits = nrows * C * 8 < 0.5 * torch.cuda.mem_get_info()[0]
    keep64 = fits and not mixed   # the plain form keeps its FP64 A for force.txt when it fits
    A64_all = torch.empty((nrows, C), dtype=torch.float64, device="cuda") if keep64 else None
    b_all = torch.empty(nrows, dtype=torch.float64, device="cuda")
    w_all = None   # row weights (src/chimes_lsq.py:71-149)
    if args.weights:
        wh = np.atleast_1d(np.loadtxt(args.weights, dtype=np.float64))
        if wh.shape[0] != nrows:
            raise SystemExit("Wrong number of lines in WEIGHTS file")
        w_all = torch.from_numpy(wh).cuda()
    wp = (lambda r: w_all[r:].data_ptr()) if w_all is not None else (lambda r: 0)
    wcol = (lambda r, n: w_all[r:r + n, None]) if w_all is not None else (lambda r, n: 1.0)
    colsum = torch.zeros(C, dtype=torch.float64, device="cuda")   # A^T 1 (DLARS --normalize)
    dfrs, lab_ptrs, w_ptrs = [], [], []   # the blocks on the device (FP64 refinement, force.txt)
    r0 = 0
    for blk in blocks:
        dfr = sess.upload(blk)
        n = blk.nrows
        dfrs.append(dfr)
        lab_ptrs.append(b_all[r0:].data_ptr())
        w_ptrs.append(w_all[r0:].data_ptr() if w_all is not None else 0)
        b_all[r0:r0 + n] = torch.from_numpy(blk.labels())
        if mixed:
            A32 = torch.empty((n, C), dtype=torch.float32, device="cuda")
            sess.assemble_device(dfr, cg.CG_FP32, A32.data_ptr(), C)
            sess.gram(1, A32.data_ptr(), C, n, C, b_all[r0:].data_ptr(), 1, G.data_ptr(), h.data_ptr(), wp(r0))
            colsum += (A32.double() * wcol(r0, n)).sum(0)
            del A32
        else:
            dst = A64_all[r0:r0 + n] if keep64 else torch.empty((n, C), dtype=torch.float64, device="cuda")
            sess.assemble_device(dfr, cg.CG_FP64, dst.data_ptr(), C)
            sess.gram(0, dst.data_ptr(), C, n, C, b_all[r0:].data_ptr(), 0, G.data_ptr(), h.data_ptr(), wp(r0))
            colsum += (dst * wcol(r0, n)).sum(0)
            del dst
        r0 += n
    dAc = None
    if Acon.shape[0]:   # the constraint rows join the normal equations like any row block
        dAc = torch.from_numpy(Acon).cuda()
        b_all[r0:] = torch.from_numpy(bcon)
        sess.gram(0, dAc.data_ptr(), C, Acon.shape[0], C, b_all[r0:].data_ptr(), 0, G.data_ptr(), h.data_ptr(),
                  wp(r0))
        colsum += (dAc * wcol(r0, Acon.shape[0])).sum(0)
        if keep64:
            A64_all[r0:] = dAc
    sess.gram_finish(G.data_ptr(), C)
    x = torch.zeros(C, dtype=torch.float64, device="cuda")
    lines = [f"! Date  {datetime.date.today()}", "!", f"! Number of variables            =  {C}",
             f"! Number of equations            =  {nrows}"]
    if args.algorithm == "ridge":
        if mixed and args.refine > 0:
            extra = None
            if dAc is not None:
                extra = (dAc.data_ptr(), Acon.shape[0], b_all[r0:].data_ptr(),
                         w_all[r0:].data_ptr() if w_all is not None else 0)
            info = sess.solve_streamed(G.data_ptr(), h.data_ptr(), C, args.alpha, dfrs, lab_ptrs, x.data_ptr(),
                                       weight_ptrs=w_ptrs if w_all is not None else None, extra=extra,
                                       max_iters=args.refine, tol=args.tol)
            iters = info["iters"]
        else:
            sess.solve(G.data_ptr(), h.data_ptr(), C, args.alpha, 0, C, 0, 0, 0, x.data_ptr())
            iters = 0
        lines += ["! ridge regression used", "! Ridge alpha = %11.4e" % args.alpha]
        if mixed:
            lines += [f"! split-BF16 tensor-core Gram, FP64 Cholesky, {iters} FP64 CG passes "
                      f"over FP64 row blocks assembled again"]
    elif args.algorithm == "lassolars":
        sess.lars(G.data_ptr(), h.data_ptr(), C, nrows, args.alpha, x.data_ptr())
        lines += ["! LARS implementation of LASSO used", "! LASSO alpha = %11.4e" % args.alpha]
    else:   # fit_dlars src/chimes_lsq.py:714-790
        lasso = args.algorithm == "dlasso"
        bw = b_all * w_all if w_all is not None else b_all
        btb = float(bw @ bw)
        bsum = float(bw.sum())
        sess.dlars(G.data_ptr(), h.data_ptr(), C, nrows, btb, args.alpha, lasso, x.data_ptr(),
                   colsum_ptr=colsum.data_ptr() if args.normalize else 0, bsum=bsum)
        lines += ["! DLARS code for %s used" % ("LASSO" if lasso else "LARS"), "! DLARS alpha = %10.4e" % args.alpha,
                  "! DLARS run: cg_dlars (device, normal equations) --lambda=%s --algorithm=%s --normalize=%s"
                  % (args.alpha, "lasso" if lasso else "lars", "y" if args.normalize else "n"), ""]
    torch.cuda.synchronize()
    xh = x.cpu().numpy()
    # predicted labels y = A x (force.txt) and the fit statistics
    if keep64:
        y = (A64_all @ x).cpu().numpy()
    else:   # FP64 rows assembled block by block (no stored A)
        yd = torch.empty(max(nfr_rows, 1), dtype=torch.float64, device="cuda")
        sess.predict_streamed(dfrs, x.data_ptr(), yd.data_ptr())
        y = np.concatenate([yd[:nfr_rows].cpu().numpy(), Acon @ xh])
    b = b_all.cpu().numpy()
    if args.normalize and args.algorithm in ("dlars", "dlasso"):   # print_unshifted_mu: the centring comes back
        y = y - float((colsum @ x).item()) / nrows + float(b.sum()) / nrows
    Z = float(((y - b) ** 2).sum())
    nvars = C if args.algorithm == "ridge" else int(np.count_nonzero(xh))
    bic = nrows * math.log(Z / nrows) + nvars * math.log(nrows)
    lines += ["! RMS force error                = %11.4e" % math.sqrt(Z / nrows),
              "! max abs variable               = %11.4e" % float(np.abs(xh).max()),
              f"! number of fitting vars         =  {nvars}",
              "! Bayesian Information Criterion = %11.4e" % bic]
    if args.weights:
        lines += ["! Using weighting file:             " + args.weights]
    lines += ["!"]
    with open(os.path.join(out, "force.txt"), "w") as f:
        f.write("".join("%13.6e\n" % v for v in y))
    open(os.path.join(out, "params.txt"), "w").write(model.params_txt(xh, "\n".join(lines) + "\n"))
    if args.write_a:
        A = A64_all[:nfr_rows].cpu().numpy() if keep64 else None
        if A is None:
            A = np.concatenate([sess.assemble(blk, cg.CG_FP64) for blk in blocks])
        frames.write_lsq_files(A, out)   # (appends the constraint rows)
    print(f"fit: {nrows} rows x {C} columns, {args.algorithm} alpha {args.alpha:g}, {args.precision}; "
          f"RMS {math.sqrt(Z / nrows):.4e}; wrote {out}/params.txt")
    return xh, y


if __name__ == "__main__":
    main()
