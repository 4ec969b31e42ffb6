// FP64 solve of the normal equations G x = h.
//
// The reference solves the least-squares problem by truncated SVD in numpy
// (src/chimes_lsq.py:169-214).  Here G (from gram.cu) is factorised by a right-
// looking blocked Cholesky: a hand-written kernel factors each 128x128 diagonal
// block in shared memory; the panel solve and the trailing update are plain BLAS-3
// library calls (cuBLAS TRSM / SYRK).  Iterative refinement uses the FP64 residual
// r = b - A x, g = A^T r, d = G^-1 g, x += d.
#include <cublas_v2.h>
#include <cuda_runtime.h>

#include <stdexcept>
#include <string>

#include "gram.h"

namespace cgd {

constexpr int CH_NB = 128;

// Factor the kb x kb diagonal block at (k, k) of the column-major lower matrix
// (leading dimension n) in place; info <- first non-positive pivot + 1.
__global__ void k_potrf_block(double* __restrict__ G, int n, int k, int kb, int* info) {
    extern __shared__ double a[];   // kb x kb, column-major
    for (int idx = threadIdx.x; idx < kb * kb; idx += blockDim.x) {
        const int i = idx % kb, j = idx / kb;
        a[idx] = G[(int64_t)(k + j) * n + (k + i)];
    }
    __syncthreads();
    __shared__ int bad;
    if (threadIdx.x == 0) bad = 0;
    __syncthreads();
    for (int j = 0; j < kb; ++j) {
        if (threadIdx.x == 0) {
            const double d = a[j * kb + j];
            if (!(d > 0.0)) { bad = 1; if (atomicCAS(info, 0, k + j + 1) == 0) {} }
            a[j * kb + j] = d > 0.0 ? sqrt(d) : 1.0;
        }
        __syncthreads();
        const double djj = a[j * kb + j];
        for (int i = j + 1 + threadIdx.x; i < kb; i += blockDim.x) a[j * kb + i] /= djj;
        __syncthreads();
        const int m = kb - j - 1;
        for (int idx = threadIdx.x; idx < m * m; idx += blockDim.x) {
            const int i = j + 1 + idx % m, l = j + 1 + idx / m;
            if (i >= l) a[l * kb + i] -= a[j * kb + i] * a[j * kb + l];
        }
        __syncthreads();
    }
    for (int idx = threadIdx.x; idx < kb * kb; idx += blockDim.x) {
        const int i = idx % kb, j = idx / kb;
        G[(int64_t)(k + j) * n + (k + i)] = i >= j ? a[idx] : 0.0;
    }
}

__global__ void k_axpy_neg(const double* x, double* y, int64_t n) {   // y = x - y
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = x[i] - y[i];
}

}  // namespace cgd

namespace cg {

static void cb(cublasStatus_t s, const char* w) {
    if (s != CUBLAS_STATUS_SUCCESS) throw std::runtime_error(std::string("cuBLAS failure in ") + w);
}

bool cholesky(double* G, int n, int* d_info, void* handle, cudaStream_t st) {
    cublasHandle_t h = (cublasHandle_t)handle;
    cb(cublasSetStream(h, st), "setStream");
    cudaMemsetAsync(d_info, 0, sizeof(int), st);
    const size_t smem = (size_t)cgd::CH_NB * cgd::CH_NB * sizeof(double);
    cudaFuncSetAttribute(cgd::k_potrf_block, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    const double one = 1.0, mone = -1.0;
    // G is symmetric: its row-major storage is also the column-major matrix.
    for (int k = 0; k < n; k += cgd::CH_NB) {
        const int kb = std::min(cgd::CH_NB, n - k);
        cgd::k_potrf_block<<<1, 512, (size_t)kb * kb * sizeof(double), st>>>(G, n, k, kb, d_info);
        const int m = n - k - kb;
        if (m > 0) {
            double* Lkk = G + (int64_t)k * n + k;
            double* P = G + (int64_t)k * n + (k + kb);          // rows k+kb.., columns k..k+kb
            double* A22 = G + (int64_t)(k + kb) * n + (k + kb);
            cb(cublasDtrsm(h, CUBLAS_SIDE_RIGHT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_T, CUBLAS_DIAG_NON_UNIT, m, kb,
                           &one, Lkk, n, P, n),
               "trsm");
            cb(cublasDsyrk(h, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_N, m, kb, &mone, P, n, &one, A22, n), "syrk");
        }
    }
    int info = 0;
    cudaMemcpyAsync(&info, d_info, sizeof(int), cudaMemcpyDeviceToHost, st);
    cudaStreamSynchronize(st);
    return info == 0;
}

void cholesky_solve(const double* L, int n, const double* hvec, double* x, void* handle, cudaStream_t st) {
    cublasHandle_t h = (cublasHandle_t)handle;
    cb(cublasSetStream(h, st), "setStream");
    cudaMemcpyAsync(x, hvec, sizeof(double) * n, cudaMemcpyDeviceToDevice, st);
    cb(cublasDtrsv(h, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_N, CUBLAS_DIAG_NON_UNIT, n, L, n, x, 1), "trsv");
    cb(cublasDtrsv(h, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_T, CUBLAS_DIAG_NON_UNIT, n, L, n, x, 1), "trsv^T");
}

void residual(const double* A, int64_t lda, int64_t nrows, int ncols, const double* b, const double* x, double* r,
              double* g, double* rnorm, double* gnorm, void* handle, cudaStream_t st) {
    cublasHandle_t h = (cublasHandle_t)handle;
    cb(cublasSetStream(h, st), "setStream");
    const double one = 1.0, zero = 0.0;
    // row-major A is column-major X = A^T (ncols x nrows, ld lda): A x = X^T x
    cb(cublasDgemv(h, CUBLAS_OP_T, ncols, (int)nrows, &one, A, (int)lda, x, 1, &zero, r, 1), "gemv A x");
    cgd::k_axpy_neg<<<(unsigned)((nrows + 255) / 256), 256, 0, st>>>(b, r, nrows);
    cb(cublasDgemv(h, CUBLAS_OP_N, ncols, (int)nrows, &one, A, (int)lda, r, 1, &zero, g, 1), "gemv A^T r");
    cb(cublasSetPointerMode(h, CUBLAS_POINTER_MODE_HOST), "ptrmode");
    cb(cublasDnrm2(h, (int)nrows, r, 1, rnorm), "nrm2 r");
    cb(cublasDnrm2(h, ncols, g, 1, gnorm), "nrm2 g");
}

}  // namespace cg
