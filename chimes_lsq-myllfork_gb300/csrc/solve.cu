// Ridge solve of the normal equations (A^T A + ridge I) x = A^T b.
//
// The reference solves the least-squares problem by a truncated SVD in numpy
// (src/chimes_lsq.py:169-214).  Here the Gram G (gram.cu, FP64 or split-BF16) is
// factorised by the FP64 blocked Cholesky of dense64.cu, and the solution is refined
// by preconditioned conjugate gradients on the FP64 system, whose products A^T (A p)
// and residuals A^T (b - A x) come from an FP64 operator: a device-resident FP64 A,
// or FP64 row blocks assembled again block by block (the mixed form, which never
// stores an FP64 A).  The preconditioner is the Cholesky factor, so a mixed-precision
// G converges to the FP64 solution of the same ridge system.
#include <cuda_runtime.h>

#include <cmath>
#include <stdexcept>
#include <string>
#include <vector>

#include "dense64.h"
#include "gram.h"

namespace cg {

static void cks(cudaError_t e, const char* w) {
    if (e != cudaSuccess) throw std::runtime_error(std::string("CUDA error in ") + w + ": " + cudaGetErrorString(e));
}

namespace {
struct DevVec {
    double* p = nullptr;
    cudaStream_t st;
    DevVec(size_t n, cudaStream_t s) : st(s) {
        cks(cudaMallocAsync((void**)&p, sizeof(double) * std::max<size_t>(n, 1), s), "solve scratch");
    }
    ~DevVec() { cudaFreeAsync(p, st); }
};
double host_dot(const double* x, const double* y, int n, double* dscal, cudaStream_t st) {
    dot64(x, y, n, dscal, st);
    double v = 0.0;
    cks(cudaMemcpyAsync(&v, dscal, sizeof(double), cudaMemcpyDeviceToHost, st), "dot");
    cks(cudaStreamSynchronize(st), "dot");
    return v;
}
}  // namespace

double factor_ridge(const double* G, int n, double ridge, double* L, int* d_info, cudaStream_t st,
                    bool tensor_updates) {
    // The ridge grows tenfold (at most 8 times) until the factorisation succeeds: a
    // mixed-precision G can be indefinite at tiny ridges.
    double used = ridge;
    for (int attempt = 0; attempt < 9; ++attempt) {
        cks(cudaMemcpyAsync(L, G, sizeof(double) * (size_t)n * n, cudaMemcpyDeviceToDevice, st), "L = G");
        add_diag64(L, n, used, st);
        if (cholesky64(L, n, d_info, st, tensor_updates)) return used;
        used = used > 0.0 ? used * 10.0 : 1e-12;
    }
    return -1.0;
}

PcgStats pcg_ridge(const double* L, int n, double ridge, const Fp64Operator& op, double* x, int max_iters,
                   double tol, cudaStream_t st) {
    auto precond = [&](const double* r, double* z) {
        if (op.mark) op.mark(true);
        cholesky_solve64(L, n, r, z, st);
        if (op.mark) op.mark(false);
    };
    PcgStats out;
    DevVec r(n, st), z(n, st), p(n, st), q(n, st), sc(1, st);
    // r = A^T (b - A x) - ridge x
    op.residual(x, r.p);
    axpby64(n, -ridge, x, 1.0, r.p, st);
    out.rnorm0 = std::sqrt(host_dot(r.p, r.p, n, sc.p, st));
    out.rnorm = out.rnorm0;
    if (max_iters <= 0 || out.rnorm0 == 0.0) return out;
    precond(r.p, z.p);
    cks(cudaMemcpyAsync(p.p, z.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, st), "p = z");
    double rz = host_dot(r.p, z.p, n, sc.p, st);
    for (int it = 0; it < max_iters && rz > 0.0; ++it) {
        op.apply(p.p, q.p);                       // q = A^T (A p)
        axpby64(n, ridge, p.p, 1.0, q.p, st);     //   + ridge p
        const double pq = host_dot(p.p, q.p, n, sc.p, st);
        if (!(pq > 0.0)) break;
        const double alpha = rz / pq;
        axpby64(n, alpha, p.p, 1.0, x, st);
        axpby64(n, -alpha, q.p, 1.0, r.p, st);
        ++out.iters;
        // relative size of this update: |alpha| ||p|| / ||x||
        const double pp = host_dot(p.p, p.p, n, sc.p, st), xx = host_dot(x, x, n, sc.p, st);
        out.rel_update = xx > 0.0 ? std::fabs(alpha) * std::sqrt(pp / xx) : 0.0;
        precond(r.p, z.p);
        const double rz_new = host_dot(r.p, z.p, n, sc.p, st);
        if (out.rel_update <= tol) { rz = rz_new; break; }
        axpby64(n, 1.0, z.p, rz_new / rz, p.p, st);   // p = z + beta p
        rz = rz_new;
    }
    out.rnorm = std::sqrt(std::max(0.0, host_dot(r.p, r.p, n, sc.p, st)));
    return out;
}

}  // namespace cg
