// FP64 dense kernels of the normal-equations solve (see dense64.h).
//
// The reference solves its least-squares problem with numpy's SVD on the CPU
// (src/chimes_lsq.py:169-214).  On this GPU the FP64 pipe delivers about 1/64 of
// the FP32 rate, so every kernel here is shaped around the FP64 FMA rate rather
// than around bytes: register-blocked tiles (16 FMAs per 8 shared-memory loads in
// the SYRK), and enough independent CTAs per SM to keep the pipe issuing.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <stdexcept>
#include <string>

#include "dense64.h"
#include "gram.h"

namespace cgd {

// ---------------------------------------------------------------- SYRK (X^T X)
constexpr int SY_T = 64, SY_KC = 16, SY_THREADS = 256;

// (ti, tj), ti <= tj, of the linear index t over the upper triangle of ntile x ntile
// tiles stored by rows (row ti holds ntile - ti pairs).
__device__ __forceinline__ void upper_pair(int64_t t, int ntile, int& ti, int& tj) {
    const double b = 2.0 * ntile + 1.0;
    int64_t r = (int64_t)floor((b - sqrt(b * b - 8.0 * (double)t)) * 0.5);
    r = max((int64_t)0, min((int64_t)ntile - 1, r));
    auto start = [&](int64_t x) { return x * ntile - x * (x - 1) / 2; };
    while (r > 0 && start(r) > t) --r;
    while (r + 1 < ntile && start(r + 1) <= t) ++r;
    ti = (int)r;
    tj = (int)(r + (t - start(r)));
}

// grid.x: upper tile pair, grid.y: K slice.  Thread (ty, tx) of a 16 x 16 layout owns
// C rows ty + 16u and columns tx + 16v of the 64 x 64 tile (u, v < 4).
template <bool ATOMIC>
__global__ void __launch_bounds__(SY_THREADS) k_syrk_tn(const double* __restrict__ X, int64_t ldx, int64_t K, int m,
                                                        double alpha, double* __restrict__ C, int64_t ldc, int ntile,
                                                        int64_t kslice) {
    __shared__ double As[SY_KC][SY_T];
    __shared__ double Bs[SY_KC][SY_T];
    int ti, tj;
    upper_pair(blockIdx.x, ntile, ti, tj);
    const bool diag = ti == tj;
    const int64_t kb = (int64_t)blockIdx.y * kslice, ke = min(K, kb + kslice);
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int ci = ti * SY_T, cj = tj * SY_T;
    double acc[4][4];
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] = 0.0;
    for (int64_t k0 = kb; k0 < ke; k0 += SY_KC) {
#pragma unroll
        for (int q = 0; q < SY_KC * SY_T / SY_THREADS; ++q) {
            const int idx = threadIdx.x + q * SY_THREADS;
            const int kk = idx / SY_T, c = idx % SY_T;
            const int64_t k = k0 + kk;
            const bool kin = k < ke;
            As[kk][c] = (kin && ci + c < m) ? X[k * ldx + ci + c] : 0.0;
            if (!diag) Bs[kk][c] = (kin && cj + c < m) ? X[k * ldx + cj + c] : 0.0;
        }
        __syncthreads();
        const double(*Bp)[SY_T] = diag ? As : Bs;
#pragma unroll
        for (int kk = 0; kk < SY_KC; ++kk) {
            double a[4], b[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) a[u] = As[kk][ty + 16 * u];
#pragma unroll
            for (int v = 0; v < 4; ++v) b[v] = Bp[kk][tx + 16 * v];
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int v = 0; v < 4; ++v) acc[u][v] = fma(a[u], b[v], acc[u][v]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        const int i = ci + ty + 16 * u;
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            const int j = cj + tx + 16 * v;
            if (i < m && j < m && j >= i) {
                double* p = C + (int64_t)i * ldc + j;
                if (ATOMIC) atomicAdd(p, alpha * acc[u][v]);
                else *p += alpha * acc[u][v];
            }
        }
    }
}

// ---------------------------------------------------------------- Cholesky
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
    for (int j = 0; j < kb; ++j) {
        if (threadIdx.x == 0) {
            const double d = a[j * kb + j];
            if (!(d > 0.0)) atomicCAS(info, 0, k + j + 1);
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

// Panel solve X L_kk^T = P below the diagonal block at (k, k): rows k+kb+i of the
// columns k..k+kb-1 (column-major, leading dimension n).  A CTA owns TR_R rows;
// four threads share a row (lanes 4r..4r+3 of one warp) and split each row's dot
// products by l mod 4, so a row's forward substitution needs only warp shuffles.
constexpr int TR_R = 64, TR_THREADS = 256, TR_PLD = CH_NB + 4;
__global__ void __launch_bounds__(TR_THREADS, 1) k_trsm_panel(double* __restrict__ G, int n, int k, int kb, int m) {
    extern __shared__ double sm[];
    double* Ls = sm;                    // Ls[j * kb + l] = L(j, l), l <= j
    double* Ps = sm + kb * kb;          // Ps[r * TR_PLD + l]
    double* rdiag = Ps + TR_R * TR_PLD; // 1 / L(j, j)
    const int i0 = blockIdx.x * TR_R;
    const int rows = min(TR_R, m - i0);
    for (int idx = threadIdx.x; idx < kb * kb; idx += blockDim.x) {
        const int j = idx % kb, l = idx / kb;
        Ls[j * kb + l] = l <= j ? G[(int64_t)(k + l) * n + (k + j)] : 0.0;
    }
    for (int idx = threadIdx.x; idx < TR_R * kb; idx += blockDim.x) {
        const int r = idx % TR_R, l = idx / TR_R;
        Ps[r * TR_PLD + l] = r < rows ? G[(int64_t)(k + l) * n + (k + kb + i0 + r)] : 0.0;
    }
    __syncthreads();
    for (int j = threadIdx.x; j < kb; j += blockDim.x) rdiag[j] = 1.0 / Ls[j * kb + j];
    __syncthreads();
    const int r = threadIdx.x >> 2, q = threadIdx.x & 3;
    double* pr = Ps + r * TR_PLD;
    for (int j = 0; j < kb; ++j) {
        const double* lj = Ls + j * kb;
        double s = 0.0;
        for (int l = q; l < j; l += 4) s = fma(pr[l], lj[l], s);
        s += __shfl_xor_sync(0xffffffffu, s, 1);
        s += __shfl_xor_sync(0xffffffffu, s, 2);
        if (q == 0) pr[j] = (pr[j] - s) * rdiag[j];
        __syncwarp();
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < TR_R * kb; idx += blockDim.x) {
        const int rr = idx % TR_R, l = idx / TR_R;
        if (rr < rows) G[(int64_t)(k + l) * n + (k + kb + i0 + rr)] = Ps[rr * TR_PLD + l];
    }
}

// ---------------------------------------------------------------- triangular solves
// T(i, j) = M[i*si + j*sj].  One CTA solves the whole system when n fits its shared
// memory: blocks of 32 in solve order, warp 0 substitutes within the block with
// shuffles, then every warp updates the remaining right-hand sides.
constexpr int TS_THREADS = 1024, TS_SMALL = 1024, TS_BLOCK = 128;
__device__ __forceinline__ double tget(const double* M, int64_t si, int64_t sj, int64_t i, int64_t j) {
    return M[i * si + j * sj];
}

// The bl x bl diagonal block at b0 (bl <= 32), staged by every thread of the CTA into
// tb (32 x 33) so that warp 0's substitution below reads shared memory only.
__device__ void trsv_stage_block(const double* M, int64_t si, int64_t sj, int b0, int bl, double (*tb)[33]) {
    for (int t = threadIdx.x; t < 32 * 32; t += blockDim.x) {
        const int i = si == 1 ? t % 32 : t / 32, j = si == 1 ? t / 32 : t % 32;   // contiguous index fastest
        tb[i][j] = (i < bl && j < bl) ? tget(M, si, sj, b0 + i, b0 + j) : 0.0;
    }
}

__device__ void trsv_block_warp(const double (*tb)[33], int b0, int bl, bool lower, double* xs, int lane) {
    double v = lane < bl ? xs[b0 + lane] : 0.0;
    if (lower) {
        for (int k = 0; k < bl; ++k) {
            if (lane == k) v = v / tb[k][k];
            const double xk = __shfl_sync(0xffffffffu, v, k);
            if (lane > k && lane < bl) v = fma(-tb[lane][k], xk, v);
        }
    } else {
        for (int k = bl - 1; k >= 0; --k) {
            if (lane == k) v = v / tb[k][k];
            const double xk = __shfl_sync(0xffffffffu, v, k);
            if (lane < k) v = fma(-tb[lane][k], xk, v);
        }
    }
    if (lane < bl) xs[b0 + lane] = v;
}

// rows [r0, r1) of xs -= T(rows, b0 .. b0+bl) * xs[b0 .. b0+bl)
__device__ void trsv_update_cta(const double* M, int64_t si, int64_t sj, int b0, int bl, int r0, int r1, double* xs) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (sj == 1) {   // rows contiguous along j: a warp per row
        for (int i = r0 + warp; i < r1; i += nw) {
            double p = 0.0;
            for (int c = lane; c < bl; c += 32) p = fma(M[(int64_t)i * si + b0 + c], xs[b0 + c], p);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) p += __shfl_xor_sync(0xffffffffu, p, o);
            if (lane == 0) xs[i] -= p;
        }
    } else {         // columns contiguous along i (or general): a thread per row
        for (int i = r0 + (int)threadIdx.x; i < r1; i += blockDim.x) {
            double p = 0.0;
#pragma unroll 8   // eight independent loads in flight per thread
            for (int c = 0; c < bl; ++c) p = fma(tget(M, si, sj, i, b0 + c), xs[b0 + c], p);
            xs[i] -= p;
        }
    }
}

__global__ void __launch_bounds__(TS_THREADS) k_trsv_small(const double* __restrict__ M, int64_t si, int64_t sj,
                                                           int n, int lower, double* __restrict__ x) {
    extern __shared__ double xs[];
    __shared__ double tb[32][33];
    for (int i = threadIdx.x; i < n; i += blockDim.x) xs[i] = x[i];
    const int nb = (n + 31) / 32;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int bb = 0; bb < nb; ++bb) {
        const int b = lower ? bb : nb - 1 - bb;
        const int b0 = b * 32, bl = min(32, n - b0);
        trsv_stage_block(M, si, sj, b0, bl, tb);
        __syncthreads();
        if (warp == 0) trsv_block_warp(tb, b0, bl, lower != 0, xs, lane);
        __syncthreads();
        if (lower) trsv_update_cta(M, si, sj, b0, bl, b0 + bl, n, xs);
        else trsv_update_cta(M, si, sj, b0, bl, 0, b0, xs);
        __syncthreads();
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) x[i] = xs[i];
}

// Large systems: after the block [b0, b0+bl) is solved (k_trsv_small on the block),
// every remaining right-hand side row is updated by a grid of CTAs.
__global__ void __launch_bounds__(256) k_trsv_update(const double* __restrict__ M, int64_t si, int64_t sj, int b0,
                                                     int bl, int r0, int r1, double* __restrict__ x) {
    __shared__ double xb[TS_BLOCK];
    for (int c = threadIdx.x; c < bl; c += blockDim.x) xb[c] = x[b0 + c];
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (sj == 1) {
        const int gw = blockIdx.x * (blockDim.x >> 5) + warp, nw = gridDim.x * (blockDim.x >> 5);
        for (int i = r0 + gw; i < r1; i += nw) {
            double p = 0.0;
            for (int c = lane; c < bl; c += 32) p = fma(M[(int64_t)i * si + b0 + c], xb[c], p);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) p += __shfl_xor_sync(0xffffffffu, p, o);
            if (lane == 0) x[i] -= p;
        }
    } else {
        for (int i = r0 + blockIdx.x * blockDim.x + threadIdx.x; i < r1; i += gridDim.x * blockDim.x) {
            double p0 = 0.0, p1 = 0.0;
            int c = 0;
#pragma unroll 8   // sixteen independent loads in flight per thread
            for (; c + 1 < bl; c += 2) {
                p0 = fma(tget(M, si, sj, i, b0 + c), xb[c], p0);
                p1 = fma(tget(M, si, sj, i, b0 + c + 1), xb[c + 1], p1);
            }
            if (c < bl) p0 = fma(tget(M, si, sj, i, b0 + c), xb[c], p0);
            x[i] -= p0 + p1;
        }
    }
}

// ---------------------------------------------------------------- matrix-vector
__global__ void __launch_bounds__(256) k_gemv_rows(const double* __restrict__ A, int64_t lda, int64_t nrows, int ncols,
                                                   const double* __restrict__ v, const double* __restrict__ b,
                                                   const double* __restrict__ w, double* __restrict__ t) {
    const int lane = threadIdx.x & 31;
    const int64_t r = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (r >= nrows) return;
    const double* row = A + r * lda;
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
    int c = lane;
    for (; c + 96 < ncols; c += 128) {
        s0 = fma(row[c], v[c], s0);
        s1 = fma(row[c + 32], v[c + 32], s1);
        s2 = fma(row[c + 64], v[c + 64], s2);
        s3 = fma(row[c + 96], v[c + 96], s3);
    }
    for (; c < ncols; c += 32) s0 = fma(row[c], v[c], s0);
    double s = (s0 + s1) + (s2 + s3);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) {
        if (b) s = b[r] - s;
        if (w) s *= w[r] * w[r];
        t[r] = s;
    }
}

// partial[y][c] = sum over the rows of slice y of A[r][c] t[r]; a block walks its
// slice's rows with its threads across the columns (four columns per thread, four
// rows per step, whole rows read contiguously).
constexpr int ATB_SLICES = 1024, ATB_THREADS = 256;
__global__ void __launch_bounds__(ATB_THREADS) k_atb_partial(const double* __restrict__ A, int64_t lda, int64_t nr,
                                                             int ncols, const double* __restrict__ b,
                                                             double* __restrict__ partial) {
    const int64_t per = (nr + gridDim.y - 1) / gridDim.y;
    const int64_t r0 = (int64_t)blockIdx.y * per, r1 = min(nr, r0 + per);
    for (int c0 = 0; c0 < ncols; c0 += 4 * ATB_THREADS) {
        double s[4] = {0, 0, 0, 0};
        int cc[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) cc[u] = c0 + u * ATB_THREADS + threadIdx.x;
        int64_t r = r0;
        for (; r + 4 <= r1; r += 4) {   // 16 loads in flight per thread
            double v[4][4];
            double br[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                br[q] = b[r + q];
                const double* row = A + (r + q) * lda;
#pragma unroll
                for (int u = 0; u < 4; ++u) v[q][u] = cc[u] < ncols ? row[cc[u]] : 0.0;
            }
#pragma unroll
            for (int q = 0; q < 4; ++q)
#pragma unroll
                for (int u = 0; u < 4; ++u) s[u] = fma(v[q][u], br[q], s[u]);
        }
        for (; r < r1; ++r) {
            const double br = b[r];
            const double* row = A + r * lda;
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (cc[u] < ncols) s[u] = fma(row[cc[u]], br, s[u]);
        }
#pragma unroll
        for (int u = 0; u < 4; ++u)
            if (cc[u] < ncols) partial[(int64_t)blockIdx.y * ncols + cc[u]] = s[u];
    }
}
__global__ void k_atb_reduce(const double* __restrict__ partial, int nslices, int ncols, double* __restrict__ h) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncols) return;
    double s = 0.0;
    for (int y = 0; y < nslices; ++y) s += partial[(int64_t)y * ncols + c];
    h[c] += s;
}

// ---------------------------------------------------------------- vectors
__global__ void __launch_bounds__(1024) k_dot(const double* __restrict__ x, const double* __restrict__ y, int n,
                                              double* __restrict__ out) {
    __shared__ double red[32];
    double s = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) s = fma(x[i], y[i], s);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        s = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (threadIdx.x == 0) *out = s;
    }
}
__global__ void k_axpby(int n, double a, const double* __restrict__ x, double b, double* __restrict__ y) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = a * x[i] + b * y[i];
}
__global__ void k_add_diag(double* G, int n, double v) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) G[(int64_t)i * n + i] += v;
}

// ---------------------------------------------------------------- FP64 FMA rate
// CH independent FMA chains per thread (enough in flight to cover the FP64 pipe's
// latency at the occupancy the launch gets); the result is stored so that the
// chains are not removed.
template <int CH>
__global__ void __launch_bounds__(256) k_fp64_fma(double* out, int iters, double seed) {
    double x[CH];
#pragma unroll
    for (int k = 0; k < CH; ++k) x[k] = seed + 1e-9 * (threadIdx.x + 37 * k);
    const double mul = 0.9999999999, add = 1e-12;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < CH; ++k) x[k] = fma(x[k], mul, add);
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < CH; ++k) s += x[k];
    out[(int64_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace cgd

namespace cg {

static void ckd(cudaError_t e, const char* w) {
    if (e != cudaSuccess) throw std::runtime_error(std::string("CUDA error in ") + w + ": " + cudaGetErrorString(e));
}

static int sm_count() {
    static thread_local int dev_cached = -1, cached = 0;
    int dev = 0;
    ckd(cudaGetDevice(&dev), "cudaGetDevice");
    if (dev != dev_cached) {
        ckd(cudaDeviceGetAttribute(&cached, cudaDevAttrMultiProcessorCount, dev), "SM count");
        cached = std::max(1, cached);
        dev_cached = dev;
    }
    return cached;
}

void syrk_tn(const double* X, int64_t ldx, int64_t K, int m, double alpha, double* C, int64_t ldc, cudaStream_t st) {
    if (K <= 0 || m <= 0) return;
    const int ntile = (m + cgd::SY_T - 1) / cgd::SY_T;
    const int64_t npairs = (int64_t)ntile * (ntile + 1) / 2;
    const int64_t target = (int64_t)sm_count() * 6;   // about six resident CTAs per SM
    const int64_t kchunks = (K + cgd::SY_KC - 1) / cgd::SY_KC;
    int64_t nslice = npairs >= target ? 1 : std::min<int64_t>(kchunks, (target + npairs - 1) / npairs);
    const int64_t kslice = (kchunks + nslice - 1) / nslice * cgd::SY_KC;
    nslice = (K + kslice - 1) / kslice;
    if (npairs > 0x7fffffffLL) throw std::runtime_error("syrk_tn: matrix too large");
    const dim3 grid((unsigned)npairs, (unsigned)nslice);
    if (nslice > 1)
        cgd::k_syrk_tn<true><<<grid, cgd::SY_THREADS, 0, st>>>(X, ldx, K, m, alpha, C, ldc, ntile, kslice);
    else
        cgd::k_syrk_tn<false><<<grid, cgd::SY_THREADS, 0, st>>>(X, ldx, K, m, alpha, C, ldc, ntile, kslice);
    ckd(cudaGetLastError(), "k_syrk_tn");
}

bool cholesky64(double* G, int n, int* d_info, cudaStream_t st, bool tensor_updates) {
    ckd(cudaMemsetAsync(d_info, 0, sizeof(int), st), "info");
    // trailing updates of full 128-wide panels by exact BF16 digit products on the
    // tensor cores (syrk_update_ozaki); the FP64 SYRK otherwise
    void* oz = nullptr;
    const bool use_oz = tensor_updates && cgd::CH_NB == 128 && n > cgd::CH_NB;
    if (use_oz) {
        ckd(cudaMallocAsync(&oz, ozaki_scratch_bytes(n), st), "Ozaki scratch");
        ckd(cudaMemsetAsync(oz, 0, sizeof(int), st), "Ozaki error word");
    }
    const size_t smem_potrf = (size_t)cgd::CH_NB * cgd::CH_NB * sizeof(double);
    const size_t smem_trsm = ((size_t)cgd::CH_NB * cgd::CH_NB + (size_t)cgd::TR_R * cgd::TR_PLD + cgd::CH_NB) *
                             sizeof(double);
    ckd(cudaFuncSetAttribute(cgd::k_potrf_block, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_potrf),
        "potrf smem");
    ckd(cudaFuncSetAttribute(cgd::k_trsm_panel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_trsm),
        "trsm smem");
    for (int k = 0; k < n; k += cgd::CH_NB) {
        const int kb = std::min(cgd::CH_NB, n - k);
        cgd::k_potrf_block<<<1, 512, (size_t)kb * kb * sizeof(double), st>>>(G, n, k, kb, d_info);
        const int m = n - k - kb;
        if (m > 0) {
            const size_t sm = ((size_t)kb * kb + (size_t)cgd::TR_R * cgd::TR_PLD + kb) * sizeof(double);
            cgd::k_trsm_panel<<<(m + cgd::TR_R - 1) / cgd::TR_R, cgd::TR_THREADS, sm, st>>>(G, n, k, kb, m);
            // trailing update: A22 -= P P^T (P: rows k+kb.., columns k..k+kb, column-major)
            if (use_oz && kb == 128)
                syrk_update_ozaki(G + (int64_t)k * n + (k + kb), n, kb, m, -1.0, G + (int64_t)(k + kb) * n + (k + kb),
                                  n, oz, st);
            else
                syrk_tn(G + (int64_t)k * n + (k + kb), n, kb, m, -1.0, G + (int64_t)(k + kb) * n + (k + kb), n, st);
        }
        ckd(cudaGetLastError(), "cholesky step");
    }
    int info = 0, oz_err = 0;
    ckd(cudaMemcpyAsync(&info, d_info, sizeof(int), cudaMemcpyDeviceToHost, st), "info");
    if (use_oz) {
        ckd(cudaMemcpyAsync(&oz_err, oz, sizeof(int), cudaMemcpyDeviceToHost, st), "Ozaki error word");
        ckd(cudaFreeAsync(oz, st), "Ozaki scratch");
    }
    ckd(cudaStreamSynchronize(st), "cholesky");
    if (oz_err) throw std::runtime_error("Cholesky trailing update timed out on its pipeline (code " +
                                         std::to_string(oz_err) + ")");
    return info == 0;
}

void trsv64(const double* M, int64_t si, int64_t sj, int n, bool lower, double* x, cudaStream_t st) {
    if (n <= 0) return;
    if (n <= cgd::TS_SMALL) {
        const size_t smem = (size_t)n * sizeof(double);
        ckd(cudaFuncSetAttribute(cgd::k_trsv_small, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)(cgd::TS_SMALL * sizeof(double))),
            "trsv smem");
        cgd::k_trsv_small<<<1, cgd::TS_THREADS, smem, st>>>(M, si, sj, n, lower ? 1 : 0, x);
        ckd(cudaGetLastError(), "k_trsv_small");
        return;
    }
    const int nb = (n + cgd::TS_BLOCK - 1) / cgd::TS_BLOCK;
    const int grid = sm_count() * 4;
    for (int bb = 0; bb < nb; ++bb) {
        const int b = lower ? bb : nb - 1 - bb;
        const int b0 = b * cgd::TS_BLOCK, bl = std::min(cgd::TS_BLOCK, n - b0);
        // the diagonal block as a small system on x[b0 .. b0+bl)
        cgd::k_trsv_small<<<1, cgd::TS_THREADS, (size_t)bl * sizeof(double), st>>>(M + b0 * si + b0 * sj, si, sj, bl,
                                                                                   lower ? 1 : 0, x + b0);
        const int r0 = lower ? b0 + bl : 0, r1 = lower ? n : b0;
        if (r1 > r0) cgd::k_trsv_update<<<grid, 256, 0, st>>>(M, si, sj, b0, bl, r0, r1, x);
        ckd(cudaGetLastError(), "trsv step");
    }
}

void cholesky_solve64(const double* L, int n, const double* h, double* x, cudaStream_t st) {
    if (x != h) ckd(cudaMemcpyAsync(x, h, sizeof(double) * n, cudaMemcpyDeviceToDevice, st), "x = h");
    trsv64(L, 1, n, n, true, x, st);    // L y = h:   L(i, j) = L[i + j n]
    trsv64(L, n, 1, n, false, x, st);   // L^T x = y: L^T(i, j) = L[j + i n]
}

void gemv_rows64(const double* A, int64_t lda, int64_t nrows, int ncols, const double* v, const double* b,
                 const double* w, double* t, cudaStream_t st) {
    if (nrows <= 0) return;
    cgd::k_gemv_rows<<<(unsigned)((nrows + 7) / 8), 256, 0, st>>>(A, lda, nrows, ncols, v, b, w, t);
    ckd(cudaGetLastError(), "k_gemv_rows");
}

int64_t atb_partial_doubles(int64_t nrows, int ncols) {
    return std::max<int64_t>(1, std::min<int64_t>(nrows, cgd::ATB_SLICES)) * ncols;
}

void gemv_cols64(const double* A, int64_t lda, int64_t nrows, int ncols, const double* t, double* g, double* partial,
                 cudaStream_t st) {
    if (nrows <= 0) return;
    const int ns = (int)std::min<int64_t>(nrows, cgd::ATB_SLICES);
    cgd::k_atb_partial<<<dim3(1, ns), cgd::ATB_THREADS, 0, st>>>(A, lda, nrows, ncols, t, partial);
    cgd::k_atb_reduce<<<(ncols + 127) / 128, 128, 0, st>>>(partial, ns, ncols, g);
    ckd(cudaGetLastError(), "k_atb");
}

void dot64(const double* x, const double* y, int n, double* out, cudaStream_t st) {
    cgd::k_dot<<<1, 1024, 0, st>>>(x, y, n, out);
    ckd(cudaGetLastError(), "k_dot");
}

void axpby64(int n, double a, const double* x, double b, double* y, cudaStream_t st) {
    if (n <= 0) return;
    cgd::k_axpby<<<(n + 255) / 256, 256, 0, st>>>(n, a, x, b, y);
    ckd(cudaGetLastError(), "k_axpby");
}

void add_diag64(double* G, int n, double v, cudaStream_t st) {
    if (n <= 0 || v == 0.0) return;
    cgd::k_add_diag<<<(n + 255) / 256, 256, 0, st>>>(G, n, v);
    ckd(cudaGetLastError(), "k_add_diag");
}

double fp64_fma_tflops(cudaStream_t st) {
    // the best of a few chain counts and occupancies; flops = 2 per FMA
    const int threads = 256, iters = 1 << 13;
    const int sms = sm_count();
    double* out = nullptr;
    ckd(cudaMallocAsync((void**)&out, sizeof(double) * sms * 8 * threads, st), "peak scratch");
    cudaEvent_t e0, e1;
    ckd(cudaEventCreate(&e0), "event");
    ckd(cudaEventCreate(&e1), "event");
    double best = 0.0;
    auto run = [&](auto kernel, int chains, int blocks_per_sm) {
        const int blocks = sms * blocks_per_sm;
        kernel<<<blocks, threads, 0, st>>>(out, iters, 1.0);   // warm-up (clocks settle)
        for (int rep = 0; rep < 3; ++rep) {
            ckd(cudaEventRecord(e0, st), "record");
            kernel<<<blocks, threads, 0, st>>>(out, iters, 1.0 + rep);
            ckd(cudaEventRecord(e1, st), "record");
            ckd(cudaEventSynchronize(e1), "sync");
            float ms = 0.f;
            ckd(cudaEventElapsedTime(&ms, e0, e1), "elapsed");
            best = std::max(best, 2.0 * chains * iters * (double)blocks * threads / (ms * 1e-3) / 1e12);
        }
        ckd(cudaGetLastError(), "k_fp64_fma");
    };
    run(cgd::k_fp64_fma<8>, 8, 8);
    run(cgd::k_fp64_fma<16>, 16, 4);
    run(cgd::k_fp64_fma<32>, 32, 4);
    run(cgd::k_fp64_fma<32>, 32, 2);
    ckd(cudaFreeAsync(out, st), "peak scratch free");
    {   // and the register-blocked SYRK of this file on a 2048 x 4096 operand (FMA bound)
        const int K = 2048, m = 4096;
        double *X = nullptr, *C = nullptr;
        ckd(cudaMallocAsync((void**)&X, sizeof(double) * K * m, st), "peak scratch");
        ckd(cudaMallocAsync((void**)&C, sizeof(double) * m * m, st), "peak scratch");
        ckd(cudaMemsetAsync(X, 0, sizeof(double) * K * m, st), "peak scratch");   // finite operands
        ckd(cudaMemsetAsync(C, 0, sizeof(double) * m * m, st), "peak scratch");
        syrk_tn(X, m, K, m, 1.0, C, m, st);   // warm-up
        for (int rep = 0; rep < 3; ++rep) {
            ckd(cudaEventRecord(e0, st), "record");
            syrk_tn(X, m, K, m, 1.0, C, m, st);
            ckd(cudaEventRecord(e1, st), "record");
            ckd(cudaEventSynchronize(e1), "sync");
            float ms = 0.f;
            ckd(cudaEventElapsedTime(&ms, e0, e1), "elapsed");
            best = std::max(best, (double)K * m * (m + 1.0) / (ms * 1e-3) / 1e12);
        }
        ckd(cudaFreeAsync(X, st), "peak scratch free");
        ckd(cudaFreeAsync(C, st), "peak scratch free");
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    ckd(cudaStreamSynchronize(st), "sync");
    return best;
}

}  // namespace cg
