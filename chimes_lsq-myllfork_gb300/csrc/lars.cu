// LARS with the lasso modification on the normal equations, FP64 on the device.
//
// Reference: `chimes_lsq.py --algorithm lassolars` (scikit-learn LassoLars,
// src/chimes_lsq.py:248-263) and the DLARS code's active-set Cholesky updates
// (contrib/dlars/src/dlars.C:1101-1329, Matrix::cholesky_add_row /
// cholesky_remove_row contrib/dlars/src/Matrix.C:152, 215).  Published algorithm:
// Efron, Hastie, Johnstone, Tibshirani, "Least angle regression" (2004), sec. 2-3.
// Objective (1 / 2n) ||y - X w||^2 + alpha ||w||_1 with G = X^T X, h = X^T y.
//
// Device state: correlations c = h - G w, coefficients, the active list and the
// lower Cholesky factor of G_AA (row-major, leading dimension kmax).  Per step:
// the largest inactive |c| (block reduction), the factor's new row (a triangular
// solve on the stored factor, dense64.cu, then one small kernel), the equiangular
// direction (two triangular solves), a = sum_k w_k G[active_k, :] over contiguous rows of G, the step length
// (block reductions over inactive crossings and active zero crossings), and on a
// zero crossing the deletion of the variable from the factor by Givens rotations.

#include <algorithm>
#include <cstdio>
#include <fstream>
#include <cmath>
#include <stdexcept>
#include <string>
#include <vector>

#include "dense64.h"
#include "gram.h"

namespace cgd {

constexpr int LARS_THREADS = 1024;

struct ArgMax {
    double v;
    int i;
};

__device__ __forceinline__ ArgMax amax(ArgMax a, ArgMax b) { return (b.v > a.v || (b.v == a.v && b.i < a.i)) ? b : a; }

// max |c_j| over j with flag <= maxflag (0: inactive only, 1: inactive and
// active); single block, lowest index wins ties
__global__ void k_lars_argmax(const double* c, const int* flag, int n, ArgMax* out, int maxflag = 0) {
    __shared__ ArgMax sm[32];
    ArgMax best{-1.0, -1};
    for (int j = threadIdx.x; j < n; j += blockDim.x)
        if (flag[j] <= maxflag) best = amax(best, ArgMax{fabs(c[j]), j});
    for (int o = 16; o > 0; o >>= 1) {
        ArgMax other{__shfl_down_sync(0xffffffffu, best.v, o), __shfl_down_sync(0xffffffffu, best.i, o)};
        best = amax(best, other);
    }
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = best;
    __syncthreads();
    if (threadIdx.x == 0) {
        ArgMax b = sm[0];
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) b = amax(b, sm[w]);
        *out = b;
    }
}

// v[k] = G[active_k, j]
__global__ void k_lars_gather(const double* G, int n, const int* active, int na, int j, double* v) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < na) v[k] = G[(size_t)active[k] * n + j];
}

// d2 = G_jj - l.l (single block); out[0] = d2
__global__ void k_lars_dot_rest(const double* l, int na, double gjj, double* out) {
    __shared__ double sm[32];
    double s = 0.0;
    for (int k = threadIdx.x; k < na; k += blockDim.x) s += l[k] * l[k];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sm[w];
        out[0] = gjj - t;
    }
}

// row na of L: l (na entries) then sqrt(d2)
__global__ void k_lars_put_row(double* L, int ld, int na, const double* l, double d2) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < na) L[(size_t)na * ld + k] = l[k];
    if (k == na) L[(size_t)na * ld + na] = sqrt(d2);
}

// s_k = sign(c[active_k])
__global__ void k_lars_signs(const double* c, const int* active, int na, double* s) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < na) s[k] = c[active[k]] >= 0.0 ? 1.0 : -1.0;
}

// w <- w * AA with AA = (s.w)^-1/2 (single block); out[0] = AA
__global__ void k_lars_scale(const double* s, double* w, int na, double* out) {
    __shared__ double sm[32];
    __shared__ double aa;
    double t = 0.0;
    for (int k = threadIdx.x; k < na; k += blockDim.x) t += s[k] * w[k];
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = t;
    __syncthreads();
    if (threadIdx.x == 0) {
        double u = 0.0;
        for (int q = 0; q < (int)(blockDim.x >> 5); ++q) u += sm[q];
        aa = 1.0 / sqrt(u);
        out[0] = aa;
    }
    __syncthreads();
    for (int k = threadIdx.x; k < na; k += blockDim.x) w[k] *= aa;
}

// a_j = sum_k w_k G[active_k, j]  (rows of the symmetric G: coalesced over j)
__global__ void k_lars_direction(const double* G, int n, const int* active, const double* w, int na, double* a) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    double s = 0.0;
    for (int k = 0; k < na; ++k) s = fma(w[k], G[(size_t)active[k] * n + j], s);
    a[j] = s;
}

struct MinPos {
    double v;
    int i;
};
__device__ __forceinline__ MinPos mmin(MinPos a, MinPos b) { return (b.v < a.v || (b.v == a.v && b.i < a.i)) ? b : a; }

// out[0]: smallest positive inactive crossing (g1 or g2), out[1]: smallest positive
// zero crossing -beta_k / w_k over the active list (index k).  `dropped`: the
// variable that just left (its same-sign root is the current point).
__global__ void k_lars_steps(const double* c, const double* a, const int* flag, int n, double C, double AA,
                             int dropped, const double* beta, const int* active, const double* w, int na,
                             MinPos* out, double zmin = 0.0) {
    __shared__ MinPos s1[32], s2[32];
    MinPos b1{INFINITY, -1}, b2{INFINITY, -1};
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
        if (flag[j] != 0) continue;
        const double g1 = (C - c[j]) / (AA - a[j]);
        const double g2 = (C + c[j]) / (AA + a[j]);
        const bool skip1 = j == dropped && c[j] > 0.0, skip2 = j == dropped && c[j] <= 0.0;
        if (!skip1 && g1 > 0.0 && isfinite(g1)) b1 = mmin(b1, MinPos{g1, j});
        if (!skip2 && g2 > 0.0 && isfinite(g2)) b1 = mmin(b1, MinPos{g2, j});
    }
    for (int k = threadIdx.x; k < na; k += blockDim.x) {
        const double z = -beta[active[k]] / w[k];
        if (z > zmin && isfinite(z)) b2 = mmin(b2, MinPos{z, k});
    }
    for (int o = 16; o > 0; o >>= 1) {
        MinPos t1{__shfl_down_sync(0xffffffffu, b1.v, o), __shfl_down_sync(0xffffffffu, b1.i, o)};
        MinPos t2{__shfl_down_sync(0xffffffffu, b2.v, o), __shfl_down_sync(0xffffffffu, b2.i, o)};
        b1 = mmin(b1, t1);
        b2 = mmin(b2, t2);
    }
    if ((threadIdx.x & 31) == 0) { s1[threadIdx.x >> 5] = b1; s2[threadIdx.x >> 5] = b2; }
    __syncthreads();
    if (threadIdx.x == 0) {
        MinPos r1 = s1[0], r2 = s2[0];
        for (int q = 1; q < (int)(blockDim.x >> 5); ++q) { r1 = mmin(r1, s1[q]); r2 = mmin(r2, s2[q]); }
        out[0] = r1;
        out[1] = r2;
    }
}

// DLARS objective 0.5 ||b - A x||^2 / n + lambda ||x||_1 from the normal equations:
// ||b - A x||^2 = b^T b - x^T h - x^T c with c = h - G x (single block; out[0])
__global__ void k_lars_objective(const double* x, const double* h, const double* c, int n, double btb,
                                 double nsamples, double lambda, double* out) {
    __shared__ double s1[32], s2[32];
    double q = 0.0, l1 = 0.0;
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
        q += x[j] * (h[j] + c[j]);
        l1 += fabs(x[j]);
    }
    for (int o = 16; o > 0; o >>= 1) {
        q += __shfl_down_sync(0xffffffffu, q, o);
        l1 += __shfl_down_sync(0xffffffffu, l1, o);
    }
    if ((threadIdx.x & 31) == 0) { s1[threadIdx.x >> 5] = q; s2[threadIdx.x >> 5] = l1; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double Q = 0.0, L1 = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) { Q += s1[w]; L1 += s2[w]; }
        out[0] = 0.5 * (btb - Q) / nsamples + lambda * L1;
    }
}

// ||x||_1 (single block; out[0])
__global__ void k_lars_l1(const double* x, int n, double* out) {
    __shared__ double s1[32];
    double l1 = 0.0;
    for (int j = threadIdx.x; j < n; j += blockDim.x) l1 += fabs(x[j]);
    for (int o = 16; o > 0; o >>= 1) l1 += __shfl_down_sync(0xffffffffu, l1, o);
    if ((threadIdx.x & 31) == 0) s1[threadIdx.x >> 5] = l1;
    __syncthreads();
    if (threadIdx.x == 0) {
        double L1 = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) L1 += s1[w];
        out[0] = L1;
    }
}

// c = h - G x (a warp per row of the symmetric G): the correlations of a restarted path
__global__ void k_lars_corr(const double* G, const double* h, const double* x, int n, double* c) {
    const int lane = threadIdx.x & 31;
    const int64_t i = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (i >= n) return;
    double sacc = 0.0;
    for (int j = lane; j < n; j += 32) sacc = fma(G[i * n + j], x[j], sacc);
    for (int o = 16; o > 0; o >>= 1) sacc += __shfl_xor_sync(0xffffffffu, sacc, o);
    if (lane == 0) c[i] = h[i] - sacc;
}

// DLARS --normalize on the normal equations (Matrix::normalize, Vector::normalize
// contrib/dlars/src/Matrix.h:614-660, Vector.h:140-150): columns centred on their
// means mu = colsum / n and scaled to unit norm sigma_j = sqrt(G_jj - n mu_j^2), b
// centred on its mean ybar:  Gc = (G - n mu mu^T) / (sigma sigma^T),
// hc = (h - ybar colsum) / sigma.
__global__ void k_dlars_sigma(const double* G, const double* colsum, int n, double nsamples, double* sigma, int* bad) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const double mu = colsum[j] / nsamples;
    const double s2 = G[(size_t)j * n + j] - nsamples * mu * mu;
    sigma[j] = s2 > 0.0 ? sqrt(s2) : 0.0;
    if (!(s2 > 0.0)) atomicExch(bad, 1);
}
__global__ void k_dlars_center(const double* G, const double* h, const double* colsum, const double* sigma, int n,
                               double nsamples, double ybar, double* Gc, double* hc) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)n * n) return;
    const int i = (int)(idx / n), j = (int)(idx % n);
    const double mi = colsum[i] / nsamples, mj = colsum[j] / nsamples;
    Gc[idx] = (G[idx] - nsamples * mi * mj) / (sigma[i] * sigma[j]);
    if (j == 0) hc[i] = (h[i] - ybar * colsum[i]) / sigma[i];
}
__global__ void k_dlars_unscale(double* x, const double* sigma, int n) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < n) x[j] /= sigma[j];   // DLARS::print_unscaled (dlars.C:2073-2097)
}

// beta[active] += gamma w; c -= gamma a
__global__ void k_lars_update(double* beta, double* c, const double* a, const int* active, const double* w, int na,
                              int n, double gamma) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < na) beta[active[j]] += gamma * w[j];
    if (j < n) c[j] -= gamma * a[j];
}

// Delete variable k from the lower factor L (na x na, row-major, leading dim ld):
// rows k+1.. move up one, then Givens rotations on columns (j, j+1), j = k..na-2,
// restore the lower triangle (single block).
__global__ void k_lars_chol_delete(double* L, int ld, int na, int k) {
    for (int i = k; i < na - 1; ++i) {
        for (int q = threadIdx.x; q <= i + 1; q += blockDim.x) L[(size_t)i * ld + q] = L[(size_t)(i + 1) * ld + q];
        __syncthreads();
    }
    for (int q = threadIdx.x; q < na; q += blockDim.x) L[(size_t)(na - 1) * ld + q] = 0.0;
    __syncthreads();
    __shared__ double cs, sn;
    for (int j = k; j < na - 1; ++j) {
        if (threadIdx.x == 0) {
            const double a = L[(size_t)j * ld + j], b = L[(size_t)j * ld + j + 1];
            const double r = hypot(a, b);
            cs = a / r;
            sn = b / r;
        }
        __syncthreads();
        for (int i = j + threadIdx.x; i < na - 1; i += blockDim.x) {
            const double x = L[(size_t)i * ld + j], y = L[(size_t)i * ld + j + 1];
            L[(size_t)i * ld + j] = cs * x + sn * y;
            L[(size_t)i * ld + j + 1] = -sn * x + cs * y;
        }
        __syncthreads();
    }
}

}  // namespace cgd

namespace cg {

static void ckl(cudaError_t e, const char* w) {
    if (e != cudaSuccess) throw std::runtime_error(std::string("CUDA error in ") + w + ": " + cudaGetErrorString(e));
}

namespace {
// The walk's state at the top of an iteration (the DLARS restart file).
struct LarsState {
    int steps = 0, next_add = -1;
    bool drop = false;
    double last_obj = 1.0e50;
    std::vector<double> x;        // n coefficients
    std::vector<int> active;      // in entry order
    std::vector<int> exclude;     // left out as dependent on the active set
};

void write_state(const std::string& path, const LarsState& S, double lambda, int mode) {
    FILE* f = std::fopen(path.c_str(), "w");
    if (!f) throw std::runtime_error("cannot write the DLARS restart file " + path);
    std::fprintf(f, "DLARS restart\nIteration %d\nObjective %.17e\nLambda %.17e\nLasso %d\nNextAdd %d\nDrop %d\n",
                 S.steps, S.last_obj, lambda, mode == 2 ? 1 : 0, S.next_add, S.drop ? 1 : 0);
    int nz = 0;
    for (double v : S.x) nz += v != 0.0;
    std::fprintf(f, "Beta %zu %d\n", S.x.size(), nz);
    for (size_t j = 0; j < S.x.size(); ++j)
        if (S.x[j] != 0.0) std::fprintf(f, "%zu %.17e\n", j, S.x[j]);
    std::fprintf(f, "Active %zu\n", S.active.size());
    for (int j : S.active) std::fprintf(f, "%d\n", j);
    std::fprintf(f, "Exclude %zu\n", S.exclude.size());
    for (int j : S.exclude) std::fprintf(f, "%d\n", j);
    std::fclose(f);
}

LarsState read_state(const std::string& path, int n, double lambda, int mode) {
    std::ifstream in(path);
    if (!in) throw std::runtime_error("cannot open the DLARS restart file " + path);
    LarsState S;
    std::string tag, w;
    double lam = 0.0;
    int lasso = 0, drop = 0;
    size_t dim = 0, nz = 0, na = 0, ne = 0;
    in >> w >> w;   // "DLARS restart"
    in >> tag >> S.steps >> tag >> S.last_obj >> tag >> lam >> tag >> lasso >> tag >> S.next_add >> tag >> drop;
    S.drop = drop != 0;
    in >> tag >> dim >> nz;
    if (!in || tag != "Beta" || (int)dim != n) throw std::runtime_error("DLARS restart file does not match the problem");
    if (lasso != (mode == 2 ? 1 : 0) || lam != lambda)
        throw std::runtime_error("DLARS restart file was written for another algorithm or lambda");
    S.x.assign(n, 0.0);
    for (size_t k = 0; k < nz; ++k) {
        size_t j;
        double v;
        in >> j >> v;
        if (j >= (size_t)n) throw std::runtime_error("DLARS restart file: coefficient index out of range");
        S.x[j] = v;
    }
    in >> tag >> na;
    for (size_t k = 0; k < na; ++k) { int j; in >> j; S.active.push_back(j); }
    in >> tag >> ne;
    for (size_t k = 0; k < ne; ++k) { int j; in >> j; S.exclude.push_back(j); }
    if (!in) throw std::runtime_error("DLARS restart file is truncated");
    for (int j : S.active) if (j < 0 || j >= n) throw std::runtime_error("DLARS restart file: bad active index");
    for (int j : S.exclude) if (j < 0 || j >= n) throw std::runtime_error("DLARS restart file: bad excluded index");
    return S;
}
}  // namespace

// Returns [steps, active variables, final C / n]; x (device, n values) receives
// the coefficients.  G: full symmetric FP64 (row-major), h: X^T y (device).
void lars_lasso(const double* G, const double* h, int n, int64_t nsamples, double alpha, int max_iter, double* x,
                double* info, cudaStream_t st, int mode, double btb, double max_norm, const char* restart_in,
                const char* restart_out) {
    // mode 0: scikit-learn LassoLars (exact landing on C/n = alpha).  mode 1 / 2: the
    // reference's DLARS `lars` / `lasso` (contrib/dlars/src/dlars.C): the variable
    // named by the last step enters, C = max |c| over every variable, lasso
    // crossings above 1e-12, no re-entry bar, and the walk stops at the first
    // vertex whose objective 0.5 ||b - A x||^2 / n + alpha ||x||_1 exceeds the
    // previous vertex's by more than 1e-10, returning that vertex (the driver,
    // :376-420).
    const bool dl = mode != 0, dlasso = mode == 2;
    const int kmax = (int)std::min<int64_t>(n, std::max<int64_t>(nsamples, 1));
    std::vector<void*> mem;
    auto get = [&](size_t bytes) {
        void* p = nullptr;
        ckl(cudaMallocAsync(&p, std::max<size_t>(bytes, 8), st), "lars scratch");
        mem.push_back(p);
        return p;
    };
    try {
        double* c = (double*)get(sizeof(double) * n);
        double* a = (double*)get(sizeof(double) * n);
        int* flag = (int*)get(sizeof(int) * n);
        int* dact = (int*)get(sizeof(int) * kmax);
        double* L = (double*)get(sizeof(double) * (size_t)kmax * kmax);
        double* w = (double*)get(sizeof(double) * kmax);
        double* sv = (double*)get(sizeof(double) * kmax);
        double* scal = (double*)get(sizeof(double) * 4);
        double* xprev = (double*)get(sizeof(double) * n);   // the vertex before a step (max_norm)
        cgd::ArgMax* am = (cgd::ArgMax*)get(sizeof(cgd::ArgMax));
        cgd::MinPos* mp = (cgd::MinPos*)get(sizeof(cgd::MinPos) * 2);
        ckl(cudaMemcpyAsync(c, h, sizeof(double) * n, cudaMemcpyDeviceToDevice, st), "c = h");
        ckl(cudaMemsetAsync(x, 0, sizeof(double) * n, st), "x = 0");
        ckl(cudaMemsetAsync(flag, 0, sizeof(int) * n, st), "flags");
        std::vector<int> active;
        std::vector<int> hflag(n, 0);
        const double target = (double)nsamples * alpha;
        double C = 0.0;
        bool drop = false;
        int dropped = -1, steps = 0, next_add = -1;
        bool resumed = false, stopped_max_norm = false, stopped_objective = false;
        double last_obj = 1.0e50, obj = 0.0;
        // C = max |h|
        cgd::k_lars_argmax<<<1, cgd::LARS_THREADS, 0, st>>>(c, flag, n, am);
        cgd::ArgMax hm{};
        ckl(cudaMemcpyAsync(&hm, am, sizeof(hm), cudaMemcpyDeviceToHost, st), "argmax");
        ckl(cudaStreamSynchronize(st), "sync");
        C = hm.v;
        const int tb = 256;
        // the active-set factor's new row for variable j (entering as number na);
        // returns d2, the new diagonal squared (dependent when below 1e-13 G_jj)
        auto factor_row = [&](int j, int na, double& gjj) {
            ckl(cudaMemcpyAsync(&gjj, G + (size_t)j * n + j, sizeof(double), cudaMemcpyDeviceToHost, st), "Gjj");
            double d2 = 0.0;
            if (na == 0) {
                ckl(cudaStreamSynchronize(st), "sync");
                d2 = gjj;
            } else {
                // L l = G[A, j] with the row-major lower factor L(i, j) = L[i * kmax + j]
                cgd::k_lars_gather<<<(na + tb - 1) / tb, tb, 0, st>>>(G, n, dact, na, j, sv);
                trsv64(L, kmax, 1, na, true, sv, st);
                cgd::k_lars_dot_rest<<<1, cgd::LARS_THREADS, 0, st>>>(sv, na, gjj, scal);
                ckl(cudaMemcpyAsync(&d2, scal, sizeof(double), cudaMemcpyDeviceToHost, st), "d2");
                ckl(cudaStreamSynchronize(st), "sync");
            }
            return d2;
        };
        if (dl && restart_in && *restart_in) {   // resume a walk from its restart file
            LarsState R = read_state(restart_in, n, alpha, mode);
            ckl(cudaMemcpyAsync(x, R.x.data(), sizeof(double) * n, cudaMemcpyHostToDevice, st), "restart x");
            cgd::k_lars_corr<<<(n + 7) / 8, 256, 0, st>>>(G, h, x, n, c);
            const int one = 1, two = 2;
            for (int j : R.exclude) {
                hflag[j] = 2;
                ckl(cudaMemcpyAsync(flag + j, &two, sizeof(int), cudaMemcpyHostToDevice, st), "flag");
            }
            for (int j : R.active) {   // the factor of G_AA, one row per active variable in entry order
                const int na = (int)active.size();
                if (na >= kmax) throw std::runtime_error("DLARS restart file: more active variables than rows");
                double gjj = 0.0;
                const double d2 = factor_row(j, na, gjj);
                if (!(d2 > 0.0)) throw std::runtime_error("DLARS restart file: active set is not independent");
                cgd::k_lars_put_row<<<(na + 1 + tb - 1) / tb, tb, 0, st>>>(L, kmax, na, sv, d2);
                active.push_back(j);
                hflag[j] = 1;
                ckl(cudaMemcpyAsync(flag + j, &one, sizeof(int), cudaMemcpyHostToDevice, st), "flag");
                ckl(cudaMemcpyAsync(dact + na, &active.back(), sizeof(int), cudaMemcpyHostToDevice, st), "active");
                ckl(cudaStreamSynchronize(st), "sync");
            }
            steps = R.steps;
            next_add = R.next_add;
            drop = R.drop;
            last_obj = R.last_obj;
            resumed = true;
        }
        while (steps < max_iter && (dl || C > target)) {
            if (dl) {
                if ((int)active.size() >= n) break;   // no more iterations possible
                cgd::k_lars_objective<<<1, cgd::LARS_THREADS, 0, st>>>(x, h, c, n, btb, (double)nsamples, alpha,
                                                                      scal + 2);
                cgd::k_lars_argmax<<<1, cgd::LARS_THREADS, 0, st>>>(c, flag, n, am, 1);   // C over every variable
                ckl(cudaMemcpyAsync(&obj, scal + 2, sizeof(double), cudaMemcpyDeviceToHost, st), "objective");
                ckl(cudaMemcpyAsync(&hm, am, sizeof(hm), cudaMemcpyDeviceToHost, st), "C");
                ckl(cudaStreamSynchronize(st), "sync");
                if (resumed) {   // the restart file holds this vertex's objective already
                    resumed = false;
                } else {
                    if (obj > last_obj + 1.0e-10) { stopped_objective = true; break; }   // this vertex is the answer
                    last_obj = obj;
                }
                C = hm.v;
                if (restart_out && *restart_out && steps > 0 && steps % 10 == 0) {
                    // the state every ten iterations, as the reference's DLARS::print_restart
                    LarsState W;
                    W.steps = steps; W.next_add = next_add; W.drop = drop; W.last_obj = last_obj;
                    W.x.resize(n);
                    ckl(cudaMemcpyAsync(W.x.data(), x, sizeof(double) * n, cudaMemcpyDeviceToHost, st), "x");
                    ckl(cudaStreamSynchronize(st), "sync");
                    W.active = active;
                    for (int j = 0; j < n; ++j) if (hflag[j] == 2) W.exclude.push_back(j);
                    write_state(restart_out, W, alpha, mode);
                }
            }
            if (!drop) {
                if (dl && next_add >= 0) {
                    hm.i = next_add;
                } else {
                    cgd::k_lars_argmax<<<1, cgd::LARS_THREADS, 0, st>>>(c, flag, n, am);
                    ckl(cudaMemcpyAsync(&hm, am, sizeof(hm), cudaMemcpyDeviceToHost, st), "argmax");
                    ckl(cudaStreamSynchronize(st), "sync");
                }
                if (hm.i < 0) break;
                const int j = hm.i;
                const int na = (int)active.size();
                double gjj = 0.0;
                const double d2 = factor_row(j, na, gjj);
                const int one = 1, two = 2;
                if (!(d2 > 1e-13 * gjj) || na >= kmax) {   // dependent on the active set: leave it out
                    hflag[j] = 2;
                    ckl(cudaMemcpyAsync(flag + j, &two, sizeof(int), cudaMemcpyHostToDevice, st), "flag");
                    ckl(cudaStreamSynchronize(st), "sync");
                    next_add = -1;
                    if (dl) last_obj = 1.0e50;   // re-evaluate at the same vertex
                    continue;
                }
                cgd::k_lars_put_row<<<(na + 1 + tb - 1) / tb, tb, 0, st>>>(L, kmax, na, sv, d2);
                active.push_back(j);
                hflag[j] = 1;
                ckl(cudaMemcpyAsync(flag + j, &one, sizeof(int), cudaMemcpyHostToDevice, st), "flag");
                ckl(cudaMemcpyAsync(dact + na, &active.back(), sizeof(int), cudaMemcpyHostToDevice, st), "active");
                if (!dl) C = std::max(C, hm.v);
                ckl(cudaStreamSynchronize(st), "sync");
            }
            drop = false;
            const int na = (int)active.size();
            // equiangular direction: L L^T w = s, w *= AA
            cgd::k_lars_signs<<<(na + tb - 1) / tb, tb, 0, st>>>(c, dact, na, sv);
            ckl(cudaMemcpyAsync(w, sv, sizeof(double) * na, cudaMemcpyDeviceToDevice, st), "w = s");
            trsv64(L, kmax, 1, na, true, w, st);    // L y = s
            trsv64(L, 1, kmax, na, false, w, st);   // L^T w = y
            cgd::k_lars_scale<<<1, cgd::LARS_THREADS, 0, st>>>(sv, w, na, scal + 1);
            cgd::k_lars_direction<<<(n + tb - 1) / tb, tb, 0, st>>>(G, n, dact, w, na, a);
            double AA = 0.0;
            ckl(cudaMemcpyAsync(&AA, scal + 1, sizeof(double), cudaMemcpyDeviceToHost, st), "AA");
            ckl(cudaStreamSynchronize(st), "sync");
            cgd::k_lars_steps<<<1, cgd::LARS_THREADS, 0, st>>>(c, a, flag, n, C, AA, dl ? -1 : dropped, x, dact, w, na,
                                                               mp, dl ? 1.0e-12 : 0.0);
            cgd::MinPos hp[2];
            ckl(cudaMemcpyAsync(hp, mp, sizeof(hp), cudaMemcpyDeviceToHost, st), "steps");
            ckl(cudaStreamSynchronize(st), "sync");
            dropped = -1;
            double gamma = dl ? (na < n ? (hp[0].i >= 0 ? hp[0].v : 1.0e20) : C / AA) : std::min(C / AA, hp[0].v);
            next_add = dl ? hp[0].i : -1;
            int kz = -1;
            if ((!dl || dlasso) && hp[1].i >= 0 && hp[1].v < gamma) {
                gamma = hp[1].v;
                kz = hp[1].i;
                drop = true;
            }
            bool last = false;
            if (!dl && C - gamma * AA < target) {   // land exactly on C / n = alpha
                gamma = (C - target) / AA;
                drop = false;
                kz = -1;
                last = true;
            }
            if (dl && max_norm < 1.0e49)
                ckl(cudaMemcpyAsync(xprev, x, sizeof(double) * n, cudaMemcpyDeviceToDevice, st), "x before the step");
            cgd::k_lars_update<<<(std::max(n, na) + tb - 1) / tb, tb, 0, st>>>(x, c, a, dact, w, na, n, gamma);
            if (!dl) C -= gamma * AA;
            ++steps;
            if (last) break;
            if (drop) {
                const int var = active[kz];
                const double zero = 0.0;
                const int z0 = 0;
                ckl(cudaMemcpyAsync(x + var, &zero, sizeof(double), cudaMemcpyHostToDevice, st), "beta = 0");
                ckl(cudaMemcpyAsync(flag + var, &z0, sizeof(int), cudaMemcpyHostToDevice, st), "flag");
                hflag[var] = 0;
                cgd::k_lars_chol_delete<<<1, cgd::LARS_THREADS, 0, st>>>(L, kmax, na, kz);
                active.erase(active.begin() + kz);
                if (!active.empty())
                    ckl(cudaMemcpyAsync(dact, active.data(), sizeof(int) * active.size(), cudaMemcpyHostToDevice, st),
                        "active");
                dropped = var;
                ckl(cudaStreamSynchronize(st), "sync");
            }
            if (dl && max_norm < 1.0e49) {   // the driver's --max_norm: keep the vertex before this step
                cgd::k_lars_l1<<<1, cgd::LARS_THREADS, 0, st>>>(x, n, scal + 3);
                double l1 = 0.0;
                ckl(cudaMemcpyAsync(&l1, scal + 3, sizeof(double), cudaMemcpyDeviceToHost, st), "l1");
                ckl(cudaStreamSynchronize(st), "sync");
                if (l1 > max_norm) {
                    ckl(cudaMemcpyAsync(x, xprev, sizeof(double) * n, cudaMemcpyDeviceToDevice, st), "revert");
                    stopped_max_norm = true;
                    break;
                }
            }
            ckl(cudaGetLastError(), "lars step");
        }
        ckl(cudaStreamSynchronize(st), "sync");
        // iterations as the reference's driver counts them: it takes the step of the
        // iteration that finds the objective risen before it stops (dlars.C:365-381)
        if (info) {
            info[0] = steps + (stopped_objective ? 1 : 0);
            info[1] = (double)active.size();
            info[2] = dl ? last_obj : C / (double)nsamples;
        }
        (void)stopped_max_norm;
    } catch (...) {
        for (void* p : mem) cudaFreeAsync(p, st);
        cudaStreamSynchronize(st);
        throw;
    }
    for (void* p : mem) cudaFreeAsync(p, st);
}

void dlars_normalized(const double* G, const double* h, const double* colsum, double bsum, int n, int64_t nsamples,
                      double btb, double lambda, int lasso, int max_iter, double* x, double* info, cudaStream_t st,
                      double max_norm, const char* restart_in, const char* restart_out) {
    double *Gc = nullptr, *hc = nullptr, *sigma = nullptr;
    int* bad = nullptr;
    ckl(cudaMallocAsync((void**)&Gc, sizeof(double) * (size_t)n * n, st), "normalised G");
    ckl(cudaMallocAsync((void**)&hc, sizeof(double) * n, st), "normalised h");
    ckl(cudaMallocAsync((void**)&sigma, sizeof(double) * n, st), "column scales");
    ckl(cudaMallocAsync((void**)&bad, sizeof(int), st), "flag");
    auto release = [&]() {
        cudaFreeAsync(Gc, st); cudaFreeAsync(hc, st); cudaFreeAsync(sigma, st); cudaFreeAsync(bad, st);
    };
    try {
        const double N = (double)nsamples, ybar = bsum / N;
        ckl(cudaMemsetAsync(bad, 0, sizeof(int), st), "flag");
        cgd::k_dlars_sigma<<<(n + 255) / 256, 256, 0, st>>>(G, colsum, n, N, sigma, bad);
        int hbad = 0;
        ckl(cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, st), "flag");
        ckl(cudaStreamSynchronize(st), "sync");
        if (hbad) throw std::runtime_error("a column of A is constant: its normalisation scale is 0");
        const int64_t nn = (int64_t)n * n;
        cgd::k_dlars_center<<<(unsigned)((nn + 255) / 256), 256, 0, st>>>(G, h, colsum, sigma, n, N, ybar, Gc, hc);
        ckl(cudaGetLastError(), "normalise");
        lars_lasso(Gc, hc, n, nsamples, lambda, max_iter, x, info, st, lasso ? 2 : 1, btb - N * ybar * ybar, max_norm,
                   restart_in, restart_out);
        cgd::k_dlars_unscale<<<(n + 255) / 256, 256, 0, st>>>(x, sigma, n);
        ckl(cudaGetLastError(), "unscale");
    } catch (...) {
        release();
        throw;
    }
    release();
}

}  // namespace cg
