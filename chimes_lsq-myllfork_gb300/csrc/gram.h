// Normal equations and their FP64 solve (see gram.cu, solve.cu and dense64.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <functional>

namespace cg {

// Bytes of the two BF16 planes for an A block of nrows_block rows.
size_t gram_plane_bytes(int64_t nrows_block, int ncols);

// G (row-major ncols x ncols FP64, upper triangle) += A^T A and h += A^T b for the
// device A block (row-major, lda; prec_in 0 = FP64, 1 = FP32).  mode 0: FP64 SYRK
// (dense64.cu); mode 1: split-BF16 3-product Gram on tcgen05 (planes: scratch of at
// least gram_plane_bytes(64, ncols) bytes; larger buffers take larger row blocks).
// mark(stage, begin) brackets the A^T b, split, tensor and FP64 SYRK launches
// (stage ids of session.h) for the optional CUDA-event timing.
// ctas_per_sm: target CTAs per SM when the K dimension is sliced (tunable).
void gram_accumulate(int prec_in, const void* A, int64_t lda, int64_t nrows, int ncols, const double* b, int mode,
                     double* G, double* h, void* planes, size_t planes_bytes, int* d_err, cudaStream_t st,
                     const std::function<void(int, bool)>& mark, int ctas_per_sm = 4);
// C (row-major ldc, upper triangle) += alpha X^T X for X of K <= 128 rows x m columns
// (row-major ldx), with FP64 accuracy from exact BF16 digit products on the tensor
// cores (gram.cu).  scratch: ozaki_scratch_bytes(m) bytes (its first int is the
// kernel's error word, zeroed by the caller before the first call).
size_t ozaki_scratch_bytes(int m_max);
void syrk_update_ozaki(const double* X, int64_t ldx, int K, int m, double alpha, double* C, int64_t ldc,
                       void* scratch, cudaStream_t st);
// Copy the upper triangle of G to the lower one.
void gram_symmetrize(double* G, int n, bool from_upper, cudaStream_t st);

// L = Cholesky factor of G + r I (n x n, L: device n*n doubles, column-major lower in
// the symmetric storage) with r = ridge, grown tenfold at most 8 times while G + r I
// is not positive definite.  Returns the r used, or -1 when every attempt failed.
// tensor_updates: trailing updates by syrk_update_ozaki (else the FP64 SYRK).
double factor_ridge(const double* G, int n, double ridge, double* L, int* d_info, cudaStream_t st,
                    bool tensor_updates = true);

// The FP64 products of a least-squares problem with rows A (never stored whole by
// the streamed form): apply(p, q): q = A^T (A p); residual(x, r): r = A^T (b - A x).
// Row weights, when present, enter both as A^T W^2 (...).
struct Fp64Operator {
    std::function<void(const double* p, double* q)> apply;
    std::function<void(const double* x, double* r)> residual;
    std::function<void(bool begin)> mark;   // brackets the preconditioner solves (optional timing)
};
struct PcgStats {
    int iters = 0;
    double rel_update = 0.0;   // |alpha| ||p|| / ||x|| of the last step
    double rnorm0 = 0.0, rnorm = 0.0;   // ||A^T (b - A x) - ridge x|| before and after (recursive)
};
// Preconditioned CG on (A^T A + ridge I) x = A^T b from x (device, updated), with
// M = L L^T (factor_ridge); stops after max_iters steps or when the relative update
// falls to tol.
PcgStats pcg_ridge(const double* L, int n, double ridge, const Fp64Operator& op, double* x, int max_iters,
                   double tol, cudaStream_t st);

// LARS with the lasso modification on G (full symmetric, FP64, device) and h:
// coefficients into x (device); info: [steps, active variables, final C / n].
// mode 0: scikit-learn LassoLars; mode 1 / 2: the reference's DLARS `lars` /
// `lasso` (needs btb = b^T b; info[2] is then the objective of the last vertex).
// DLARS only (mode 1 / 2): max_norm stops once ||x||_1 after a step exceeds it and
// returns the vertex before that step (the driver's --max_norm); restart_out (may be
// null) receives the walk's state every ten iterations and restart_in (may be null)
// resumes a walk from such a file (the driver's --restart).
void lars_lasso(const double* G, const double* h, int n, int64_t nsamples, double alpha, int max_iter, double* x,
                double* info, cudaStream_t st, int mode = 0, double btb = 0.0, double max_norm = 1.0e50,
                const char* restart_in = nullptr, const char* restart_out = nullptr);
// DLARS with --normalize: columns centred and scaled, b centred (colsum = A^T 1 on
// the device, bsum = sum b), coefficients returned in unscaled units.
void dlars_normalized(const double* G, const double* h, const double* colsum, double bsum, int n, int64_t nsamples,
                      double btb, double lambda, int lasso, int max_iter, double* x, double* info, cudaStream_t st,
                      double max_norm = 1.0e50, const char* restart_in = nullptr,
                      const char* restart_out = nullptr);

}  // namespace cg
