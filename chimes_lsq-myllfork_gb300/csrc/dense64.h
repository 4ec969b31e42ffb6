// FP64 dense kernels of the normal-equations solve (dense64.cu): the plain form's
// Gram, the blocked Cholesky factorisation, triangular solves and the matrix-vector
// products of the refinement.  All launches go to the given stream; no library BLAS.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace cg {

// Upper-triangle tiles of C (row-major, ldc) += alpha * X^T X, X = K rows of m
// contiguous values (row-major, ldx): C[i][j] += alpha * sum_k X[k][i] X[k][j] for
// j >= i.  K is split across CTAs (FP64 atomics) only when the m x m triangle has too
// few tiles to fill the GPU; otherwise every C entry is updated by one CTA in a
// fixed order (bit-reproducible).
void syrk_tn(const double* X, int64_t ldx, int64_t K, int m, double alpha, double* C, int64_t ldc, cudaStream_t st);

// In-place right-looking blocked Cholesky of a symmetric n x n matrix held in full
// (row-major == column-major) storage: on return its column-major lower triangle
// holds L (G = L L^T); the strict upper triangle of each diagonal block is zeroed and
// the rest of the upper triangle keeps G's values.  128 x 128 diagonal
// blocks are factorised in shared memory, the panel below by substitution against
// the block, the trailing matrix by syrk_tn.  Returns false when a pivot is not
// positive (d_info: device int, first bad column + 1).
bool cholesky64(double* G, int n, int* d_info, cudaStream_t st, bool tensor_updates = false);

// In-place triangular solve T x = b (x holds b on entry) with T(i, j) = M[i*si + j*sj]
// lower (forward substitution) or upper (backward substitution), n x n.
void trsv64(const double* M, int64_t si, int64_t sj, int n, bool lower, double* x, cudaStream_t st);

// x = (L L^T)^-1 h with L from cholesky64 (x and h may alias).
void cholesky_solve64(const double* L, int n, const double* h, double* x, cudaStream_t st);

// t[r] = sum_c A[r][c] v[c] (row-major A, lda), then t[r] = b[r] - t[r] when b is not
// null; when w is not null t[r] *= w[r]^2 afterwards (row weights of a weighted fit).
void gemv_rows64(const double* A, int64_t lda, int64_t nrows, int ncols, const double* v, const double* b,
                 const double* w, double* t, cudaStream_t st);

// g[c] += sum_r A[r][c] t[r] (row-major A, lda): row slices summed into partials
// (scratch, at least atb_partial_doubles(nrows, ncols) doubles), then an ordered sum,
// so the result is reproducible.
int64_t atb_partial_doubles(int64_t nrows, int ncols);
void gemv_cols64(const double* A, int64_t lda, int64_t nrows, int ncols, const double* t, double* g,
                 double* partial, cudaStream_t st);

// Vector helpers (n doubles, device).  dot64 writes sum_i x[i] y[i] to *out (device)
// in a fixed order.
void dot64(const double* x, const double* y, int n, double* out, cudaStream_t st);
// y = a*x + b*y
void axpby64(int n, double a, const double* x, double b, double* y, cudaStream_t st);
// G[i][i] += v
void add_diag64(double* G, int n, double v, cudaStream_t st);

// Measured FP64 FMA rate of the current device (TFLOP/s, 2 flops per FMA): the
// better of a kernel of independent FMA chains on every SM and this file's
// register-blocked SYRK on a 2048 x 4096 operand, timed with CUDA events.  Changes
// no device setting.
double fp64_fma_tflops(cudaStream_t st);

}  // namespace cg
