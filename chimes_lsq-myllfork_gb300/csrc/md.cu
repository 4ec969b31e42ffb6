// MD force kernels: 2-body pairs, dense-tensor triplet / quadruplet contraction,
// the per-frame finish (ZCalc's /V scaling and energy offsets) and the
// velocity-Verlet updates.
//
// Reference arithmetic per cluster (Cheby::Force_3B / Force_4B, src/Cheby.C:2024-2675):
// for every allowed power tuple p with coefficient c_p,
//   E   += perm c_p prod_e f_e T_e[p_e]
//   F_e  = perm c_p (f_e T'_e + f'_e T_e)[p_e] prod_{e' != e} f_e' T_e'[p_e']
// and F_e / r_e times the edge vector is added to the first member and taken
// from the second; the virial collects -F_e r_e and -F_e r_a r_b / r_e.
//
// GB300 formulation: the coefficients of a cluster type are one dense tensor
// C[p_0..p_{n-1}] over the canonical pair slots (zero where a tuple is not
// allowed).  With u_s[k] = f_s T_k(r_s), one depth-first pass over C gives
//   E = sum C prod_s u_s[p_s]   and   G_s[k] = dE / du_s[k]
// (partial sums flow up, prefix products flow down: two FMAs per entry), and
// F_e = perm sum_k G_s[k] (f T' + f' T)_s[k] for the edge e in slot s.  A
// 4-body type of order 4 costs ~11k FMAs per quadruplet this way, against ~80k for
// the power-tuple loop.  One thread owns one cluster; a block shares one
// (frame, cluster type) bucket, so C sits in shared memory and every read of it
// is a broadcast.
#include <algorithm>
#include <cstdio>

#include "basis.cuh"
#include "md.h"

namespace cgd {

constexpr int MDC_THREADS = MDC_TILE;

__device__ __forceinline__ int frame_of_atom(const FramesDev& F, int64_t a) {
    int lo = 0, hi = F.nframes - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (F.atom_ofs[mid] <= a) lo = mid; else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Sum 8 per-thread values over the block and add them to the frame's scalars:
// v = [E, P, Wxx, Wxy, Wxz, Wyy, Wyz, Wzz].
__device__ void block_scalars_add(double* v, double* So, int f) {
    __shared__ double red[8][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        double s = warp_sum(v[k]);
        if (lane == 0) red[k][w] = s;
    }
    __syncthreads();
    if (threadIdx.x < 8) {
        double s = 0.0;
        for (int i = 0; i < nw; ++i) s += red[threadIdx.x][i];
        // tensor slots: xx=2 xy=3 xz=4 yx=5 yy=6 yz=7 zx=8 zy=9 zz=10 (symmetric)
        const int k = threadIdx.x;
        double* o = So + (size_t)f * MD_NSCALAR;
        if (s != 0.0) {
            if (k == 0) atomicAdd(o + 0, s);
            else if (k == 1) atomicAdd(o + 1, s);
            else if (k == 2) atomicAdd(o + 2, s);
            else if (k == 3) { atomicAdd(o + 3, s); atomicAdd(o + 5, s); }
            else if (k == 4) { atomicAdd(o + 4, s); atomicAdd(o + 8, s); }
            else if (k == 5) atomicAdd(o + 6, s);
            else if (k == 6) { atomicAdd(o + 7, s); atomicAdd(o + 9, s); }
            else atomicAdd(o + 10, s);
        }
    }
}

// ------------------------------------------------------------------ 2-body
struct Dot2 {
    const double* c;
    double e = 0.0, g = 0.0;
    __device__ void operator()(int k, double gk, double hk) {
        e = fma(c[k], gk, e);
        g = fma(c[k], hk, g);
    }
};

// One warp per real atom over its 2-body list (pairs i <= PARENT[g] with r < s_max;
// Cheby::Force_all src/Cheby.C:1812-1968).
__global__ void __launch_bounds__(256) k_md2(ModelDev M, MdDev D, FramesDev F, NeighDev NB, double* Fo, double* So) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= NB.n_real) return;
    const int f = frame_of_atom(F, warp);
    const int N = F.natoms[f];
    const int64_t aofs = F.atom_ofs[f];
    const BoxDev& B = F.box[f];
    const int64_t o = NB.ofs2[warp];
    const int n = NB.cnt2[warp];
    const int ord = M.order2;
    double fi[3] = {0.0, 0.0, 0.0}, v[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int t = lane; t < n; t += 32) {
        const int64_t q = o + t;
        const int g = NB.g2[q], pt = NB.pt2[q];
        double r, R[3];
        const PairDev& P = M.pairs[pt];
        if (NB.md == 2) {   // lists reused over steps: this step's distance, exact r < s_max
            const int64_t gb = F.ghost_ofs[f];
            r = dist_exact(B.h, F.scaled + 3 * (gb + (warp - aofs)), F.scaled + 3 * (gb + g), R);
            if (!(r < P.smax)) continue;
        } else {
            r = NB.r2[q];
            R[0] = NB.rab2[3 * q]; R[1] = NB.rab2[3 * q + 1]; R[2] = NB.rab2[3 * q + 2];
        }
        double fc, fd;
        fcut_eval(M, r, P.smax, fc, fd);
        Dot2 acc{D.c2 + (size_t)pt * ord};
        basis_visit(M, P.lambda, P.xavg, P.xdiff, P.smin, r, fc, fd, 1, ord, acc);
        double es = B.perm2 * acc.e, gs = B.perm2 * acc.g;
        if (r - D.pen_dist < P.smin) {   // cubic penalty below s_min + d (src/Cheby.C:1900-1968)
            const double rp = P.smin + D.pen_dist - r;
            if (rp > 0.0) {
                gs += -3.0 * rp * rp * D.pen_scale;
                es += rp * rp * rp * D.pen_scale;
            }
        }
        const double wv = gs / r;
        double* fo = Fo + 3 * (aofs + g % N);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            fi[c] = fma(wv, R[c], fi[c]);
            atomicAdd(fo + c, -wv * R[c]);
        }
        v[0] += es;
        v[1] -= gs * r;
        v[2] -= wv * R[0] * R[0]; v[3] -= wv * R[0] * R[1]; v[4] -= wv * R[0] * R[2];
        v[5] -= wv * R[1] * R[1]; v[6] -= wv * R[1] * R[2]; v[7] -= wv * R[2] * R[2];
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) fi[c] = warp_sum(fi[c]);
#pragma unroll
    for (int k = 0; k < 8; ++k) v[k] = warp_sum(v[k]);
    if (lane == 0) {
        const int i = warp - (int)aofs;
        double* fo = Fo + 3 * (aofs + i);
        if (n > 0) {
            for (int c = 0; c < 3; ++c) atomicAdd(fo + c, fi[c]);
            double* so = So + (size_t)f * MD_NSCALAR;
            atomicAdd(so + 0, v[0]); atomicAdd(so + 1, v[1]);
            atomicAdd(so + 2, v[2]); atomicAdd(so + 3, v[3]); atomicAdd(so + 4, v[4]);
            atomicAdd(so + 5, v[3]); atomicAdd(so + 6, v[5]); atomicAdd(so + 7, v[6]);
            atomicAdd(so + 8, v[4]); atomicAdd(so + 9, v[6]); atomicAdd(so + 10, v[7]);
        }
    }
}

// ------------------------------------------------------------------ grouping
__device__ __forceinline__ int frame_of_cluster(const int64_t* cfo, int nframes, int64_t q) {
    int lo = 0, hi = nframes - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (cfo[mid] <= q) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Warp-aggregated increment: one atomic per distinct key in the warp; returns the
// slot of this lane (order among equal keys within the warp by lane).
__device__ __forceinline__ int warp_agg_inc(int* ctr, int key, bool active) {
    const unsigned act = __ballot_sync(0xffffffffu, active);
    int slot = 0;
    if (active) {
        const unsigned peers = __match_any_sync(act, key);
        const int leader = __ffs(peers) - 1;
        const int lane = threadIdx.x & 31;
        int base = 0;
        if (lane == leader) base = atomicAdd(ctr + key, __popc(peers));
        base = __shfl_sync(peers, base, leader);
        slot = base + __popc(peers & ((1u << lane) - 1u));
    }
    return slot;
}

__global__ void k_md_bucket_count(int64_t n, int nframes, const int64_t* cfo, const int* type, int ntypes,
                                  int* cnt) {
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n; base += (int64_t)gridDim.x * blockDim.x) {
        const int64_t q = base + threadIdx.x;
        const bool ok = q < n && type[q] >= 0;   // -1: filtered out this step
        const int key = ok ? frame_of_cluster(cfo, nframes, q) * ntypes + type[q] : 0;
        warp_agg_inc(cnt, key, ok);
    }
}

// Single block: start[] = exclusive scan of the counts, tile_ofs[] = exclusive scan
// of ceil(count / MDC_TILE).
__global__ void k_md_bucket_scan(const int* cnt, int nkeys, int64_t* start, int* tile_ofs) {
    __shared__ int64_t ps[1024];
    __shared__ int pt[1024];
    const int per = (nkeys + blockDim.x - 1) / blockDim.x;
    const int b = threadIdx.x * per, e = min(nkeys, b + per);
    int64_t s = 0;
    int t = 0;
    for (int i = b; i < e; ++i) { s += cnt[i]; t += (cnt[i] + MDC_TILE - 1) / MDC_TILE; }
    ps[threadIdx.x] = s;
    pt[threadIdx.x] = t;
    __syncthreads();
    for (int off = 1; off < (int)blockDim.x; off <<= 1) {
        int64_t vs = threadIdx.x >= (unsigned)off ? ps[threadIdx.x - off] : 0;
        int vt = threadIdx.x >= (unsigned)off ? pt[threadIdx.x - off] : 0;
        __syncthreads();
        ps[threadIdx.x] += vs;
        pt[threadIdx.x] += vt;
        __syncthreads();
    }
    int64_t rs = ps[threadIdx.x] - s;
    int rt = pt[threadIdx.x] - t;
    for (int i = b; i < e; ++i) {
        start[i] = rs; tile_ofs[i] = rt;
        rs += cnt[i]; rt += (cnt[i] + MDC_TILE - 1) / MDC_TILE;
    }
    if (threadIdx.x == blockDim.x - 1) { start[nkeys] = ps[threadIdx.x]; tile_ofs[nkeys] = pt[threadIdx.x]; }
}

__global__ void k_md_bucket_fill(int64_t n, int nframes, const int64_t* cfo, const int* type, int ntypes,
                                 const int64_t* start, int* cursor, int* val) {
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n; base += (int64_t)gridDim.x * blockDim.x) {
        const int64_t q = base + threadIdx.x;
        const bool ok = q < n && type[q] >= 0;
        const int key = ok ? frame_of_cluster(cfo, nframes, q) * ntypes + type[q] : 0;
        const int slot = warp_agg_inc(cursor, key, ok);
        if (ok) val[start[key] + slot] = (int)q;
    }
}

// Tile -> (key, first grouped cluster); false when the tile is past the last one.
__device__ __forceinline__ bool tile_lookup(const MdBuckets& B, int tile, int& key, int64_t& c0, int64_t& c1) {
    if (tile >= B.tile_ofs[B.nkeys]) return false;
    int lo = 0, hi = B.nkeys - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (B.tile_ofs[mid] <= tile) lo = mid; else hi = mid - 1;
    }
    key = lo;
    c0 = B.start[key] + (int64_t)(tile - B.tile_ofs[key]) * MDC_TILE;
    c1 = B.start[key + 1];
    return c0 < c1;
}

// ------------------------------------------------------------------ clusters
template <int N_, int O>
struct IPow { static constexpr int v = O * IPow<N_ - 1, O>::v; };
template <int O>
struct IPow<0, O> { static constexpr int v = 1; };

template <int O, typename R>
__device__ __forceinline__ R pick(const R (&a)[O], int i) {
    R v = a[0];
#pragma unroll
    for (int k = 1; k < O; ++k) if (k == i) v = a[k];
    return v;
}
template <int O, typename R>
__device__ __forceinline__ void put(R (&a)[O], int i, R v) {
#pragma unroll
    for (int k = 0; k < O; ++k) if (k == i) a[k] = v;
}

// E and G_s[k] = dE/du_s[k] for one cluster: slot 0 is walked at run time, the
// remaining slots fully unrolled (registers only).
template <int O, typename R>
__device__ __forceinline__ R contract3(const R* __restrict__ sC, const R (&u)[3][O], R (&G)[3][O]) {
    R E = R(0);
#pragma unroll 1
    for (int a = 0; a < O; ++a) {
        const R ua = pick<O>(u[0], a);
        const R* Ca = sC + a * O * O;
        R Sa = R(0);
#pragma unroll
        for (int b = 0; b < O; ++b) {
            const R P = ua * u[1][b];
            R Sab = R(0);
#pragma unroll
            for (int c = 0; c < O; ++c) {
                const R cv = Ca[b * O + c];
                Sab = fma(cv, u[2][c], Sab);
                G[2][c] = fma(P, cv, G[2][c]);
            }
            G[1][b] = fma(ua, Sab, G[1][b]);
            Sa = fma(u[1][b], Sab, Sa);
        }
        put<O>(G[0], a, Sa);
        E = fma(ua, Sa, E);
    }
    return E;
}

template <int O, typename R>
__device__ __forceinline__ R contract4(const R* __restrict__ sC, const R (&u)[6][O], R (&G)[6][O]) {
    R E = R(0);
#pragma unroll 1
    for (int a = 0; a < O; ++a) {
        const R ua = pick<O>(u[0], a);
        const R* Ca = sC + a * IPow<5, O>::v;
        R Sa = R(0);
#pragma unroll
        for (int b = 0; b < O; ++b) {
            const R Pb = ua * u[1][b];
            R Sb = R(0);
#pragma unroll
            for (int c = 0; c < O; ++c) {
                const R Pc = Pb * u[2][c];
                R Sc = R(0);
#pragma unroll
                for (int d = 0; d < O; ++d) {
                    const R Pd = Pc * u[3][d];
                    R Sd = R(0);
#pragma unroll
                    for (int e = 0; e < O; ++e) {
                        const R Pe = Pd * u[4][e];
                        const R* Cl = Ca + (((b * O + c) * O + d) * O + e) * O;
                        R Se = R(0);
#pragma unroll
                        for (int g = 0; g < O; ++g) {
                            const R cv = Cl[g];
                            Se = fma(cv, u[5][g], Se);
                            G[5][g] = fma(Pe, cv, G[5][g]);
                        }
                        G[4][e] = fma(Pd, Se, G[4][e]);
                        Sd = fma(u[4][e], Se, Sd);
                    }
                    G[3][d] = fma(Pc, Sd, G[3][d]);
                    Sc = fma(u[3][d], Sd, Sc);
                }
                G[2][c] = fma(Pb, Sc, G[2][c]);
                Sb = fma(u[2][c], Sc, Sb);
            }
            G[1][b] = fma(ua, Sb, G[1][b]);
            Sa = fma(u[1][b], Sb, Sa);
        }
        put<O>(G[0], a, Sa);
        E = fma(ua, Sa, E);
    }
    return E;
}

__device__ __forceinline__ void edge_ab(int NBODY, int e, int& a, int& b) {
    if (NBODY == 3) { a = e == 2 ? 1 : 0; b = e == 0 ? 1 : 2; }
    else {
        a = e < 3 ? 0 : (e < 5 ? 1 : 2);
        b = e == 0 ? 1 : (e == 1 || e == 3) ? 2 : 3;
    }
}

// Per-thread geometry of a cluster, slot by slot (canonical slot s <- actual edge e).
// FP64: the exact H (s_b - s_a) distance of the enumeration; FP32 form: the FP32
// Cartesian copy of the ghosts (the cluster set itself was decided exactly).
template <typename R>
struct SlotGeomT {
    R r, R3[3];
    int a, b, pt;
};

template <int NBODY, typename R>
__device__ __forceinline__ void cluster_geom(const ModelDev& M, const FramesDev& F, int f, int4 mm,
                                             SlotGeomT<R>* sg) {
    constexpr int NP = NBODY == 3 ? 3 : 6;
    const int N = F.natoms[f];
    const int64_t gb = F.ghost_ofs[f];
    const int* typ = F.type + F.atom_ofs[f];
    int id = 0, w = 1;
#pragma unroll
    for (int u = 0; u < NBODY; ++u) { id += w * (typ[member(mm, u) % N] + 1); w *= 10; }
    const int8_t* pm = (NBODY == 3 ? M.pidx3 : M.pidx4) + id * NP;
    const BoxDev& B = F.box[f];
#pragma unroll
    for (int e = 0; e < NP; ++e) {
        const int s = pm[e];
        int a, b;
        edge_ab(NBODY, e, a, b);
        const int ga = member(mm, a), gbm = member(mm, b);
        SlotGeomT<R> g;
        g.a = a; g.b = b;
        if constexpr (sizeof(R) == 8) {
            g.r = dist_exact(B.h, F.scaled + 3 * (gb + ga), F.scaled + 3 * (gb + gbm), g.R3);
        } else {
            const float4* c32 = reinterpret_cast<const float4*>(F.cart32);
            const float4 x = c32[gb + ga], y = c32[gb + gbm];
            g.R3[0] = y.x - x.x; g.R3[1] = y.y - x.y; g.R3[2] = y.z - x.z;
            g.r = sqrtf(g.R3[0] * g.R3[0] + g.R3[1] * g.R3[1] + g.R3[2] * g.R3[2]);
        }
        g.pt = M.int_pair_map[typ[ga % N] * M.natmtyp + typ[gbm % N]];
        sg[s] = g;
    }
}

// FCUT::get_fcut (src/Fcut.C:17-72) in the contraction precision.
template <typename R>
__device__ __forceinline__ void fcut_r(const ModelDev& M, R r, R rmax, R& f, R& fd) {
    if constexpr (sizeof(R) == 8) {
        fcut_eval(M, r, rmax, f, fd);
    } else {
        if (M.fcut == 0) {
            const float irm = 1.0f / rmax;
            const float f0 = 1.0f - r * irm;
            f = f0 * f0 * f0;
            fd = f0 * f0 * (-3.0f * irm);
        } else {
            const float th = rmax - (float)M.fcut_offset * rmax;
            if (r < th) { f = 1.0f; fd = 0.0f; }
            else if (r > rmax) { f = 0.0f; fd = 0.0f; }
            else {
                const float a = (r - th) / (rmax - th) * (float)PI_REF + (float)PI_REF / 2.0f;
                const float ad = (float)PI_REF / (rmax - th);
                f = 0.5f + 0.5f * sinf(a);
                fd = 0.5f * cosf(a) * ad;
            }
        }
    }
}

// basis_regs in FP32 arithmetic (the FP32 form); FP64 uses basis_regs itself.
template <int O, bool WANT_G, bool WANT_H>
__device__ __forceinline__ void basis_regs_f(const ModelDev& M, float lambda, float xavg, float xdiff, float smin,
                                             float r, float fc, float fd, float* g, float* h) {
    const bool out = r < smin;
    const float rr = out ? smin : r;
    float x, ex = 0.0f;
    const float ixd = 1.0f / xdiff;
    if (M.trans == 0) { ex = expf(-rr / lambda); x = (ex - xavg) * ixd; }
    else if (M.trans == 1) { x = (1.0f / rr - xavg) * ixd; }
    else { x = (rr - xavg) * ixd; }
    float dxdr;
    if (M.trans == 0) dxdr = -ex / lambda * ixd;
    else if (M.trans == 1) dxdr = -ixd / (rr * rr);
    else dxdr = ixd;
    dxdr *= (float)M.deriv_const;
    const bool zero_d = out && M.fix == 1;
    float damp = 1.0f, shift = 0.0f;
    if (out && M.fix == 0) { damp = expf((r - smin) / (float)M.smooth); shift = (float)M.smooth * (damp - 1.0f); }
    const float lin = (out && M.fix == 2) ? (r - smin) : 0.0f;
    float t_prev = 1.0f, t_cur = x, u_prev2 = 0.0f, u_prev = 1.0f;
#pragma unroll
    for (int n = 0; n < O; ++n) {
        float tn, un_1;
        if (n == 0) { tn = 1.0f; un_1 = 0.0f; }
        else if (n == 1) { tn = x; un_1 = 1.0f; }
        else {
            tn = 2.0f * x * t_cur - t_prev;
            t_prev = t_cur; t_cur = tn;
            const float un = (n - 1 == 1) ? 2.0f * x : 2.0f * x * u_prev - u_prev2;
            u_prev2 = u_prev; u_prev = un;
            un_1 = un;
        }
        float td = (n == 0 || zero_d) ? 0.0f : n * dxdr * un_1;
        if (out) {
            if (M.fix == 0) { tn += shift * td; td *= damp; }
            else if (M.fix == 2) tn += td * lin;
        }
        if (WANT_G) g[n] = fc * tn;
        if (WANT_H) h[n] = fc * td + fd * tn;
    }
}

template <int O, bool WANT_G, bool WANT_H, typename R>
__device__ __forceinline__ void basis_r(const ModelDev& M, double lambda, double xavg, double xdiff, double smin, R r,
                                        R fc, R fd, R* g, R* h) {
    if constexpr (sizeof(R) == 8)
        basis_regs<O, WANT_G, WANT_H>(M, lambda, xavg, xdiff, smin, r, fc, fd, g, h);
    else
        basis_regs_f<O, WANT_G, WANT_H>(M, (float)lambda, (float)xavg, (float)xdiff, (float)smin, r, fc, fd, g, h);
}

template <int NBODY, int O, typename R>
__global__ void __launch_bounds__(MDC_THREADS) k_mdc(ModelDev M, MdDev D, FramesDev F, ClusterSet CS, MdBuckets MB,
                                                     double* Fo, double* So) {
    constexpr int NP = NBODY == 3 ? 3 : 6;
    constexpr int SZ = IPow<NP, O>::v;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    R* sC = reinterpret_cast<R*>(smem_raw);
    SlotGeomT<R>* sG = reinterpret_cast<SlotGeomT<R>*>(smem_raw + ((SZ * sizeof(R) + 15) & ~size_t(15)));
    int key;
    int64_t cb, t1;
    if (!tile_lookup(MB, blockIdx.x, key, cb, t1)) return;
    const int f = key / MB.ntypes;
    const int T = key % MB.ntypes;
    const R* Cg = (NBODY == 3 ? (sizeof(R) == 8 ? (const R*)D.C3 : (const R*)D.C3f)
                              : (sizeof(R) == 8 ? (const R*)D.C4 : (const R*)D.C4f)) + (size_t)T * SZ;
    for (int i = threadIdx.x; i < SZ; i += blockDim.x) sC[i] = Cg[i];
    __syncthreads();
    const int64_t c = cb + threadIdx.x;
    const bool active = c < t1;
    double v[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (active) {
        const int N = F.natoms[f];
        const int64_t aofs = F.atom_ofs[f];
        const BoxDev& B = F.box[f];
        const R perm = (R)(NBODY == 3 ? B.perm3 : B.perm4);
        const ClusterTypeDev& CT = (NBODY == 3 ? M.types3 : M.types4)[T];
        const int4 mm = CS.m[MB.val[c]];
        SlotGeomT<R>* sg = sG + (size_t)threadIdx.x * NP;
        cluster_geom<NBODY, R>(M, F, f, mm, sg);
        R u[NP][O], G[NP][O];
#pragma unroll
        for (int s = 0; s < NP; ++s) {
            const SlotGeomT<R>& g = sg[s];
            R fc, fd;
            fcut_r<R>(M, g.r, (R)CT.smax[s], fc, fd);
            basis_r<O, true, false, R>(M, M.pairs[g.pt].lambda, CT.xavg[s], CT.xdiff[s], CT.smin[s], g.r, fc, fd, u[s],
                                       (R*)nullptr);
#pragma unroll
            for (int k = 0; k < O; ++k) G[s][k] = R(0);
        }
        R E;
        if constexpr (NBODY == 3) E = contract3<O, R>(sC, u, G);
        else E = contract4<O, R>(sC, u, G);
        v[0] = (double)(perm * E);
        R fm[NBODY][3];
        R w[8] = {0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
        for (int k = 0; k < NBODY; ++k) fm[k][0] = fm[k][1] = fm[k][2] = R(0);
#pragma unroll
        for (int s = 0; s < NP; ++s) {
            const SlotGeomT<R>& g = sg[s];
            R fc, fd;
            fcut_r<R>(M, g.r, (R)CT.smax[s], fc, fd);
            R h[O];
            basis_r<O, false, true, R>(M, M.pairs[g.pt].lambda, CT.xavg[s], CT.xdiff[s], CT.smin[s], g.r, fc, fd,
                                       (R*)nullptr, h);
            R gs = R(0);
#pragma unroll
            for (int k = 0; k < O; ++k) gs = fma(G[s][k], h[k], gs);
            const R ge = perm * gs;
            const R wv = ge / g.r;
#pragma unroll
            for (int k = 0; k < NBODY; ++k) {
                if (k == g.a) { fm[k][0] += wv * g.R3[0]; fm[k][1] += wv * g.R3[1]; fm[k][2] += wv * g.R3[2]; }
                if (k == g.b) { fm[k][0] -= wv * g.R3[0]; fm[k][1] -= wv * g.R3[1]; fm[k][2] -= wv * g.R3[2]; }
            }
            w[1] -= ge * g.r;
            w[2] -= wv * g.R3[0] * g.R3[0]; w[3] -= wv * g.R3[0] * g.R3[1]; w[4] -= wv * g.R3[0] * g.R3[2];
            w[5] -= wv * g.R3[1] * g.R3[1]; w[6] -= wv * g.R3[1] * g.R3[2]; w[7] -= wv * g.R3[2] * g.R3[2];
        }
#pragma unroll
        for (int k = 1; k < 8; ++k) v[k] = (double)w[k];
#pragma unroll
        for (int k = 0; k < NBODY; ++k) {
            double* fo = Fo + 3 * (aofs + member(mm, k) % N);
            atomicAdd(fo + 0, (double)fm[k][0]);
            atomicAdd(fo + 1, (double)fm[k][1]);
            atomicAdd(fo + 2, (double)fm[k][2]);
        }
    }
    block_scalars_add(v, So, f);
}

// Any order: the dense tensor read from global memory, digits decoded at run time,
// leave-one-out products by prefix / suffix.  Used for orders without an unrolled
// instantiation.
constexpr int MDG_MAXO = 16;

template <int NBODY>
__global__ void __launch_bounds__(MDC_THREADS) k_mdc_generic(ModelDev M, MdDev D, FramesDev F, ClusterSet CS,
                                                             MdBuckets MB, int O, double* Fo, double* So) {
    constexpr int NP = NBODY == 3 ? 3 : 6;
    __shared__ SlotGeomT<double> sG[MDC_THREADS * NP];
    int key;
    int64_t cb, t1;
    if (!tile_lookup(MB, blockIdx.x, key, cb, t1)) return;
    const int f = key / MB.ntypes;
    const int T = key % MB.ntypes;
    int SZ = 1;
    for (int k = 0; k < NP; ++k) SZ *= O;
    const double* C = (NBODY == 3 ? D.C3 : D.C4) + (size_t)T * SZ;
    const int64_t c = cb + threadIdx.x;
    double v[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (c < t1) {
        const int N = F.natoms[f];
        const int64_t aofs = F.atom_ofs[f];
        const BoxDev& B = F.box[f];
        const double perm = NBODY == 3 ? B.perm3 : B.perm4;
        const ClusterTypeDev& CT = (NBODY == 3 ? M.types3 : M.types4)[T];
        const int4 mm = CS.m[MB.val[c]];
        SlotGeomT<double>* sg = sG + (size_t)threadIdx.x * NP;
        cluster_geom<NBODY, double>(M, F, f, mm, sg);
        double u[NP][MDG_MAXO], h[NP][MDG_MAXO], G[NP][MDG_MAXO];
        for (int s = 0; s < NP; ++s) {
            const SlotGeomT<double>& g = sg[s];
            double fc, fd;
            fcut_eval(M, g.r, CT.smax[s], fc, fd);
            basis_gh(M, M.pairs[g.pt].lambda, CT.xavg[s], CT.xdiff[s], CT.smin[s], g.r, 0, O, fc, fd, u[s], h[s], 1);
            for (int k = 0; k < O; ++k) G[s][k] = 0.0;
        }
        double E = 0.0;
        for (int idx = 0; idx < SZ; ++idx) {
            const double cv = C[idx];
            if (cv == 0.0) continue;
            int p[NP];
            int rem = idx;
            for (int s = NP - 1; s >= 0; --s) { p[s] = rem % O; rem /= O; }
            double pre[NP + 1], suf[NP + 1];
            pre[0] = 1.0; suf[NP] = 1.0;
            for (int s = 0; s < NP; ++s) pre[s + 1] = pre[s] * u[s][p[s]];
            for (int s = NP - 1; s >= 0; --s) suf[s] = suf[s + 1] * u[s][p[s]];
            E += cv * pre[NP];
            for (int s = 0; s < NP; ++s) G[s][p[s]] += cv * pre[s] * suf[s + 1];
        }
        v[0] = perm * E;
        for (int s = 0; s < NP; ++s) {
            const SlotGeomT<double>& g = sg[s];
            double gs = 0.0;
            for (int k = 0; k < O; ++k) gs += G[s][k] * h[s][k];
            const double ge = perm * gs;
            const double wv = ge / g.r;
            double* fa = Fo + 3 * (aofs + member(mm, g.a) % N);
            double* fb = Fo + 3 * (aofs + member(mm, g.b) % N);
            for (int k = 0; k < 3; ++k) { atomicAdd(fa + k, wv * g.R3[k]); atomicAdd(fb + k, -wv * g.R3[k]); }
            v[1] -= ge * g.r;
            v[2] -= wv * g.R3[0] * g.R3[0]; v[3] -= wv * g.R3[0] * g.R3[1]; v[4] -= wv * g.R3[0] * g.R3[2];
            v[5] -= wv * g.R3[1] * g.R3[1]; v[6] -= wv * g.R3[1] * g.R3[2]; v[7] -= wv * g.R3[2] * g.R3[2];
        }
    }
    block_scalars_add(v, So, f);
}

// ------------------------------------------------------------------ list reuse
// Clusters of lists enumerated with a skin: keep a cluster this step iff every edge
// is inside its slot's s_max (the same FP32-then-exact test as the enumeration);
// type_out[q] = its type or -1.
__device__ __forceinline__ bool within_md(const FramesDev& F, const BoxDev& B, int64_t gb, int a, int b, double smax) {
    const float4* c32 = reinterpret_cast<const float4*>(F.cart32);
    const float4 x = c32[gb + a], y = c32[gb + b];
    const float dx = y.x - x.x, dy = y.y - x.y, dz = y.z - x.z;
    const float r32 = sqrtf(dx * dx + dy * dy + dz * dz);
    if (r32 < (float)smax - 1.0e-2f) return true;
    if (r32 > (float)smax + 1.0e-2f) return false;
    double rab[3];
    return dist_exact(B.h, F.scaled + 3 * (gb + a), F.scaled + 3 * (gb + b), rab) < smax;
}

// The FP32 form of k_md2: geometry from the FP32 Cartesian copy, basis, cut-off,
// penalty and products in FP32; which pairs count (r < s_max) is decided as in
// the FP64 form (FP32 with a margin, exact FP64 near s_max); FP64 accumulation.
__global__ void __launch_bounds__(256) k_md2f(ModelDev M, MdDev D, FramesDev F, NeighDev NB, double* Fo, double* So) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= NB.n_real) return;
    const int f = frame_of_atom(F, warp);
    const int N = F.natoms[f];
    const int64_t aofs = F.atom_ofs[f];
    const BoxDev& B = F.box[f];
    const int64_t o = NB.ofs2[warp];
    const int n = NB.cnt2[warp];
    const int ord = M.order2;
    const float4* c32 = reinterpret_cast<const float4*>(F.cart32);
    const int64_t gb = F.ghost_ofs[f];
    const float4 xi = c32[gb + (warp - aofs)];
    float fi[3] = {0.f, 0.f, 0.f}, v[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int t = lane; t < n; t += 32) {
        const int64_t q = o + t;
        const int g = NB.g2[q], pt = NB.pt2[q];
        const PairDev& P = M.pairs[pt];
        float r, R[3];
        if (NB.md == 2) {   // lists reused over steps: this step's geometry
            const float4 xg = c32[gb + g];
            R[0] = xg.x - xi.x; R[1] = xg.y - xi.y; R[2] = xg.z - xi.z;
            r = sqrtf(R[0] * R[0] + R[1] * R[1] + R[2] * R[2]);
            if (!within_md(F, B, gb, (int)(warp - aofs), g, P.smax)) continue;
        } else {
            r = (float)NB.r2[q];
            R[0] = (float)NB.rab2[3 * q]; R[1] = (float)NB.rab2[3 * q + 1]; R[2] = (float)NB.rab2[3 * q + 2];
        }
        float fc, fd;
        fcut_r<float>(M, r, (float)P.smax, fc, fd);
        // Chebyshev basis with a run-time order (as basis_regs_f)
        const float smin = (float)P.smin, lam = (float)P.lambda;
        const bool out = r < smin;
        const float rr = out ? smin : r;
        const float ixd = 1.0f / (float)P.xdiff;
        float x, ex = 0.0f, dxdr;
        if (M.trans == 0) { ex = expf(-rr / lam); x = (ex - (float)P.xavg) * ixd; dxdr = -ex / lam * ixd; }
        else if (M.trans == 1) { x = (1.0f / rr - (float)P.xavg) * ixd; dxdr = -ixd / (rr * rr); }
        else { x = (rr - (float)P.xavg) * ixd; dxdr = ixd; }
        dxdr *= (float)M.deriv_const;
        const bool zero_d = out && M.fix == 1;
        float damp = 1.0f, shift = 0.0f;
        if (out && M.fix == 0) { damp = expf((r - smin) / (float)M.smooth); shift = (float)M.smooth * (damp - 1.0f); }
        const float lin = (out && M.fix == 2) ? (r - smin) : 0.0f;
        const double* c = D.c2 + (size_t)pt * ord;
        float t_prev = 1.0f, t_cur = x, u_prev2 = 0.0f, u_prev = 1.0f, e = 0.0f, gsum = 0.0f;
        for (int k = 1; k <= ord; ++k) {   // 2-body columns use T_1 .. T_order
            float tn, un_1;
            if (k == 1) { tn = x; un_1 = 1.0f; }
            else {
                tn = 2.0f * x * t_cur - t_prev;
                t_prev = t_cur; t_cur = tn;
                const float un = (k - 1 == 1) ? 2.0f * x : 2.0f * x * u_prev - u_prev2;
                u_prev2 = u_prev; u_prev = un;
                un_1 = un;
            }
            float td = zero_d ? 0.0f : k * dxdr * un_1;
            if (out) {
                if (M.fix == 0) { tn += shift * td; td *= damp; }
                else if (M.fix == 2) tn += td * lin;
            }
            const float ck = (float)c[k - 1];
            e = fmaf(ck, fc * tn, e);
            gsum = fmaf(ck, fc * td + fd * tn, gsum);
        }
        const float perm = (float)B.perm2;
        float es = perm * e, gs = perm * gsum;
        if (r - (float)D.pen_dist < smin) {   // cubic penalty below s_min + d (src/Cheby.C:1900-1968)
            const float rp = smin + (float)D.pen_dist - r;
            if (rp > 0.0f) {
                gs += -3.0f * rp * rp * (float)D.pen_scale;
                es += rp * rp * rp * (float)D.pen_scale;
            }
        }
        const float wv = gs / r;
        double* fo = Fo + 3 * (aofs + g % N);
#pragma unroll
        for (int cc = 0; cc < 3; ++cc) {
            fi[cc] = fmaf(wv, R[cc], fi[cc]);
            atomicAdd(fo + cc, (double)(-wv * R[cc]));
        }
        v[0] += es;
        v[1] -= gs * r;
        v[2] -= wv * R[0] * R[0]; v[3] -= wv * R[0] * R[1]; v[4] -= wv * R[0] * R[2];
        v[5] -= wv * R[1] * R[1]; v[6] -= wv * R[1] * R[2]; v[7] -= wv * R[2] * R[2];
    }
    double fd3[3], vd[8];
#pragma unroll
    for (int cc = 0; cc < 3; ++cc) fd3[cc] = warp_sum((double)fi[cc]);
#pragma unroll
    for (int k = 0; k < 8; ++k) vd[k] = warp_sum((double)v[k]);
    if (lane == 0 && n > 0) {
        double* fo = Fo + 3 * warp;
        for (int cc = 0; cc < 3; ++cc) atomicAdd(fo + cc, fd3[cc]);
        double* so = So + (size_t)f * MD_NSCALAR;
        atomicAdd(so + 0, vd[0]); atomicAdd(so + 1, vd[1]);
        atomicAdd(so + 2, vd[2]); atomicAdd(so + 3, vd[3]); atomicAdd(so + 4, vd[4]);
        atomicAdd(so + 5, vd[3]); atomicAdd(so + 6, vd[5]); atomicAdd(so + 7, vd[6]);
        atomicAdd(so + 8, vd[4]); atomicAdd(so + 9, vd[6]); atomicAdd(so + 10, vd[7]);
    }
}

template <int NBODY>
__global__ void k_md_filter(ModelDev M, FramesDev F, ClusterSet CS, const int64_t* cfo, int64_t n, int* type_out) {
    constexpr int NP = NBODY == 3 ? 3 : 6;
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    const int f = frame_of_cluster(cfo, F.nframes, q);
    const int4 mm = CS.m[q];
    const int T = CS.type[q];
    const int N = F.natoms[f];
    const int64_t gb = F.ghost_ofs[f];
    const int* typ = F.type + F.atom_ofs[f];
    int id = 0, w = 1;
#pragma unroll
    for (int u = 0; u < NBODY; ++u) { id += w * (typ[member(mm, u) % N] + 1); w *= 10; }
    const int8_t* pm = (NBODY == 3 ? M.pidx3 : M.pidx4) + id * NP;
    const ClusterTypeDev& CT = (NBODY == 3 ? M.types3 : M.types4)[T];
    const BoxDev& B = F.box[f];
    bool ok = true;
#pragma unroll
    for (int e = 0; e < NP; ++e) {
        int a, b;
        edge_ab(NBODY, e, a, b);
        ok = ok && within_md(F, B, gb, member(mm, a), member(mm, b), CT.smax[pm[e]]);
    }
    type_out[q] = ok ? T : -1;
}

// Largest squared displacement since the lists were built (as ordered bits of a
// non-negative double).
__global__ void k_md_maxdisp(const double* x, const double* xref, int64_t n, unsigned long long* out) {
    double m = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double dx = x[3 * i] - xref[3 * i], dy = x[3 * i + 1] - xref[3 * i + 1], dz = x[3 * i + 2] - xref[3 * i + 2];
        m = fmax(m, dx * dx + dy * dy + dz * dz);
    }
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0 && m > 0.0) atomicMax(out, (unsigned long long)__double_as_longlong(m));
}

// ------------------------------------------------------------------ finish
// ZCalc (src/functions.C:838-887): per-atom energy offsets, PRESSURE_XYZ / 3V,
// tensor / V.
__global__ void k_md_finalize(ModelDev M, MdDev D, FramesDev F, double* So) {
    const int f = blockIdx.x;
    const int N = F.natoms[f];
    double e = 0.0;
    if (D.eoff) {
        const int* typ = F.type + F.atom_ofs[f];
        for (int a = threadIdx.x; a < N; a += blockDim.x) e += D.eoff[typ[a]];
    }
    __shared__ double red[32];
    e = warp_sum(e);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = e;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int i = 0; i < (int)((blockDim.x + 31) >> 5); ++i) s += red[i];
        double* o = So + (size_t)f * MD_NSCALAR;
        const double V = F.box[f].vol;
        o[0] += s;
        o[1] /= 3.0 * V;
        for (int k = 2; k < MD_NSCALAR; ++k) o[k] /= V;
    }
}

// ------------------------------------------------------------------ integration
__global__ void k_md_drift(FramesDev F, const unsigned char* first, int64_t n3, double* x, double* v, const double* a,
                           double dt) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n3) return;
    if (first && first[frame_of_atom(F, i / 3)]) return;   // a frame's step 0 only evaluates forces
    x[i] += v[i] * dt + 0.5 * a[i] * dt * dt;
    v[i] = v[i] + 0.5 * a[i] * dt;
}

__global__ void k_md_kick(FramesDev F, const double* Fo, const double* inv_mass_type, const double* mass_type,
                          double* acc, double* v, double dt, int half, const unsigned char* first, double* ke) {
    const int f = blockIdx.x;
    if (first && first[f]) half = 0;
    const int N = F.natoms[f];
    const int64_t aofs = F.atom_ofs[f];
    double k = 0.0;
    for (int i = threadIdx.x; i < 3 * N; i += blockDim.x) {
        const int64_t g = 3 * aofs + i;
        const int t = F.type[aofs + i / 3];
        const double a = Fo[g] * inv_mass_type[t];
        acc[g] = a;
        if (half) v[g] = v[g] + 0.5 * a * dt;
        k += 0.5 * mass_type[t] * v[g] * v[g];
    }
    if (!ke) return;
    __shared__ double red[32];
    k = warp_sum(k);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = k;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int i = 0; i < (int)((blockDim.x + 31) >> 5); ++i) s += red[i];
        ke[f] = s;
    }
}

// ------------------------------------------------------------------ thermostats
// Per-frame state th[f * MD_TH_STRIDE + TH_*] (md.h);
// CONSTRAINT::UPDATE_COORDS / UPDATE_VELOCS_HALF_1 / _2, src/ClassDefs.C:867-1352.

__device__ __forceinline__ double block_sum(double v, double* red) {
    v = warp_sum(v);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = 0.0;
    for (int i = 0; i < (int)((blockDim.x + 31) >> 5); ++i) s += red[i];
    return s;
}

// NVT-MTK first half (one block per frame): the kinetic energy of v(t), then
// x += v dt + a dt^2 / 2 - zeta0 v dt^2 / 2 and v_iter = v + a dt / 2 - zeta0 v dt / 2,
// and the thermostat position.
__global__ void k_md_mtk_half1(FramesDev F, const double* mass_type, double* x, double* v, const double* a, double dt,
                               double* th) {
    __shared__ double red[32];
    const int f = blockIdx.x;
    const int N = F.natoms[f];
    const int64_t aofs = F.atom_ofs[f];
    double* t = th + (size_t)f * MD_TH_STRIDE;
    double k = 0.0;
    for (int i = threadIdx.x; i < 3 * N; i += blockDim.x) {
        const int64_t g = 3 * aofs + i;
        k += 0.5 * mass_type[F.type[aofs + i / 3]] * v[g] * v[g];
    }
    k = block_sum(k, red);
    const double z0 = t[TH_ZETA], f0 = t[TH_FORCE];
    for (int i = threadIdx.x; i < 3 * N; i += blockDim.x) {
        const int64_t g = 3 * aofs + i;
        const double vi = v[g], ai = a[g];
        double xi = x[g] + (vi * dt + 0.5 * ai * dt * dt);
        xi -= 0.5 * z0 * vi * dt * dt;
        x[g] = xi;
        double vn = vi + 0.5 * ai * dt;
        vn -= 0.5 * z0 * vi * dt;
        v[g] = vn;
    }
    if (threadIdx.x == 0) {
        t[TH_KCUR] = k;
        t[TH_ZETA0] = z0;
        t[TH_FORCE0] = f0;
        t[TH_POSIT0] = t[TH_POSIT];
        t[TH_POSIT] = t[TH_POSIT] + z0 * dt + 0.5 * dt * dt * f0;
    }
}

// NVT-MTK second half (one block per frame): a = F/m; the thermostat velocity and
// the velocity scale by the reference's 10-step fixed point (Martyna, Tobias, Klein
// 1994, appendix D), the kinetic energy of (v_iter + a dt/2) / s being that of
// v_iter + a dt/2 over s^2; then v = (v_iter + a dt / 2) / s.
__global__ void k_md_mtk_half2(FramesDev F, const double* Fo, const double* inv_mass_type, const double* mass_type,
                               double* acc, double* v, double dt, double* th, double* ke) {
    __shared__ double red[32];
    const int f = blockIdx.x;
    const int N = F.natoms[f];
    const int64_t aofs = F.atom_ofs[f];
    double* t = th + (size_t)f * MD_TH_STRIDE;
    double k0 = 0.0;
    for (int i = threadIdx.x; i < 3 * N; i += blockDim.x) {
        const int64_t g = 3 * aofs + i;
        const int ty = F.type[aofs + i / 3];
        const double ai = Fo[g] * inv_mass_type[ty];
        acc[g] = ai;
        const double u = v[g] + 0.5 * ai * dt;
        k0 += 0.5 * mass_type[ty] * u * u;
    }
    k0 = block_sum(k0, red);
    const double Q = t[TH_Q], nkt = t[TH_NDOFKT], z0 = t[TH_ZETA0], f0 = t[TH_FORCE0];
    double fT = (2.0 * t[TH_KCUR] - nkt) / Q;
    double zT = z0, s = 1.0;
    for (int itr = 0; itr < 10; ++itr) {
        zT = z0 + (f0 + fT) * 0.5 * dt;
        s = 1.0 + 0.5 * dt * zT;
        fT = (2.0 * (k0 / (s * s)) - nkt) / Q;
    }
    double k = 0.0;
    for (int i = threadIdx.x; i < 3 * N; i += blockDim.x) {
        const int64_t g = 3 * aofs + i;
        const double vn = (v[g] + 0.5 * acc[g] * dt) / s;
        v[g] = vn;
        k += 0.5 * mass_type[F.type[aofs + i / 3]] * vn * vn;
    }
    k = block_sum(k, red);
    if (threadIdx.x == 0) {
        t[TH_ZETA] = zT;
        t[TH_FORCE] = fT;
        t[TH_VSCALE] = s;
        if (ke) ke[f] = k;
    }
}

// NVT-BEREND: after the plain second half, v *= sqrt(1 + dt/tau (T0/T - 1)) with T
// from the current kinetic energy and N_DOF = 3N - 3 (one block per frame).
__global__ void k_md_berend(FramesDev F, const double* mass_type, double* v, double dt, double tau, double T0,
                            double kb, double* ke, int* bad) {
    __shared__ double red[32];
    const int f = blockIdx.x;
    const int N = F.natoms[f];
    const int64_t aofs = F.atom_ofs[f];
    double k = 0.0;
    for (int i = threadIdx.x; i < 3 * N; i += blockDim.x) {
        const int64_t g = 3 * aofs + i;
        k += 0.5 * mass_type[F.type[aofs + i / 3]] * v[g] * v[g];
    }
    k = block_sum(k, red);
    const double T = 2.0 * k / ((3.0 * N - 3.0) * kb);
    const double fac = 1.0 + dt / tau * (T0 / T - 1.0);
    if (!(fac > 0.0)) {
        if (threadIdx.x == 0) atomicExch(bad, 1);
        return;
    }
    const double eta = pow(fac, 0.5);
    double k2 = 0.0;
    for (int i = threadIdx.x; i < 3 * N; i += blockDim.x) {
        const int64_t g = 3 * aofs + i;
        v[g] *= eta;
        k2 += 0.5 * mass_type[F.type[aofs + i / 3]] * v[g] * v[g];
    }
    k2 = block_sum(k2, red);
    if (threadIdx.x == 0 && ke) ke[f] = k2;
}

// ------------------------------------------------------------------ launchers
bool md_fast_order(int nbody, int order) {
    if (nbody == 3) return order >= 2 && order <= 8;
    return order >= 2 && order <= 4;
}

void launch_md2(const ModelDev& M, const MdDev& D, const FramesDev& F, const NeighDev& NB, double* Fo, double* So,
                cudaStream_t st, int prec) {
    if (NB.n_real == 0 || M.order2 == 0) return;
    const int threads = 256;
    const int64_t blocks = ((int64_t)NB.n_real * 32 + threads - 1) / threads;
    if (prec == 1) k_md2f<<<(unsigned)blocks, threads, 0, st>>>(M, D, F, NB, Fo, So);
    else k_md2<<<(unsigned)blocks, threads, 0, st>>>(M, D, F, NB, Fo, So);
}

void launch_md_bucket(int64_t n, int nframes, const int64_t* cfo, const int* type, const MdBuckets& B,
                      cudaStream_t st) {
    if (n <= 0) return;
    int* cnt = B.cursor;   // counts first, then reused as fill cursors
    cudaMemsetAsync(cnt, 0, sizeof(int) * B.nkeys, st);
    const int blocks = (int)std::min<int64_t>(4 * 152, (n + 255) / 256);
    k_md_bucket_count<<<blocks, 256, 0, st>>>(n, nframes, cfo, type, B.ntypes, cnt);
    k_md_bucket_scan<<<1, 1024, 0, st>>>(cnt, B.nkeys, B.start, B.tile_ofs);
    cudaMemsetAsync(B.cursor, 0, sizeof(int) * B.nkeys, st);
    k_md_bucket_fill<<<blocks, 256, 0, st>>>(n, nframes, cfo, type, B.ntypes, B.start, B.cursor, B.val);
}

template <int NBODY, int O, typename R>
static void run_mdc(unsigned grid, const ModelDev& M, const MdDev& D, const FramesDev& F, const ClusterSet& CS,
                    const MdBuckets& B, double* Fo, double* So, cudaStream_t st) {
    constexpr int NP = NBODY == 3 ? 3 : 6;
    const size_t smem = ((IPow<NP, O>::v * sizeof(R) + 15) & ~size_t(15)) + sizeof(SlotGeomT<R>) * NP * MDC_THREADS;
    static thread_local int attr_dev = -1;   // the attribute is per device
    int dev = 0;
    cudaGetDevice(&dev);
    if (attr_dev != dev) {
        cudaFuncSetAttribute(k_mdc<NBODY, O, R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        attr_dev = dev;
    }
    k_mdc<NBODY, O, R><<<grid, MDC_THREADS, smem, st>>>(M, D, F, CS, B, Fo, So);
}

template <int NBODY, typename R>
static bool dispatch_mdc(int order, unsigned grid, const ModelDev& M, const MdDev& D, const FramesDev& F,
                         const ClusterSet& CS, const MdBuckets& B, double* Fo, double* So, cudaStream_t st) {
#define MDC_CASE(O)                                          \
    case O:                                                  \
        run_mdc<NBODY, O, R>(grid, M, D, F, CS, B, Fo, So, st); \
        return true;
    if constexpr (NBODY == 3) {
        switch (order) { MDC_CASE(2) MDC_CASE(3) MDC_CASE(4) MDC_CASE(5) MDC_CASE(6) MDC_CASE(7) MDC_CASE(8) }
    } else {
        switch (order) { MDC_CASE(2) MDC_CASE(3) MDC_CASE(4) }
    }
#undef MDC_CASE
    return false;
}

void launch_mdc(int nbody, int prec, int order, int64_t max_tiles, const ModelDev& M, const MdDev& D,
                const FramesDev& F, const ClusterSet& CS, const MdBuckets& B, double* Fo, double* So,
                cudaStream_t st) {
    if (max_tiles <= 0) return;
    const unsigned grid = (unsigned)max_tiles;
    bool done;
    if (nbody == 3)
        done = prec == 1 ? dispatch_mdc<3, float>(order, grid, M, D, F, CS, B, Fo, So, st)
                         : dispatch_mdc<3, double>(order, grid, M, D, F, CS, B, Fo, So, st);
    else
        done = prec == 1 ? dispatch_mdc<4, float>(order, grid, M, D, F, CS, B, Fo, So, st)
                         : dispatch_mdc<4, double>(order, grid, M, D, F, CS, B, Fo, So, st);
    if (done) return;
    if (nbody == 3) k_mdc_generic<3><<<grid, MDC_THREADS, 0, st>>>(M, D, F, CS, B, order, Fo, So);
    else k_mdc_generic<4><<<grid, MDC_THREADS, 0, st>>>(M, D, F, CS, B, order, Fo, So);
}

void launch_md_filter(int nbody, const ModelDev& M, const FramesDev& F, const ClusterSet& CS, const int64_t* cfo,
                      int64_t n, int* type_out, cudaStream_t st) {
    if (n <= 0) return;
    const unsigned g = (unsigned)((n + 255) / 256);
    if (nbody == 3) k_md_filter<3><<<g, 256, 0, st>>>(M, F, CS, cfo, n, type_out);
    else k_md_filter<4><<<g, 256, 0, st>>>(M, F, CS, cfo, n, type_out);
}

void launch_md_maxdisp(const double* x, const double* xref, int64_t n, unsigned long long* out, cudaStream_t st) {
    if (n > 0) k_md_maxdisp<<<(unsigned)std::min<int64_t>(1024, (n + 255) / 256), 256, 0, st>>>(x, xref, n, out);
}

void launch_md_finalize(int nframes, const ModelDev& M, const MdDev& D, const FramesDev& F, double* So,
                        cudaStream_t st) {
    if (nframes > 0) k_md_finalize<<<nframes, 256, 0, st>>>(M, D, F, So);
}

void launch_md_drift(int64_t natoms, const FramesDev& F, const unsigned char* first, double* xyz, double* v,
                     const double* acc, double dt, cudaStream_t st) {
    const int64_t n3 = 3 * natoms;
    if (n3 > 0) k_md_drift<<<(unsigned)((n3 + 255) / 256), 256, 0, st>>>(F, first, n3, xyz, v, acc, dt);
}

void launch_md_kick(int nframes, const FramesDev& F, const double* Fo, const double* inv_mass_type,
                    const double* mass_type, double* acc, double* v, double dt, int half, const unsigned char* first,
                    double* ke, cudaStream_t st) {
    if (nframes > 0)
        k_md_kick<<<nframes, 256, 0, st>>>(F, Fo, inv_mass_type, mass_type, acc, v, dt, half, first, ke);
}

void launch_md_mtk_half1(int nframes, const FramesDev& F, const double* mass_type, double* x, double* v,
                         const double* acc, double dt, double* th, cudaStream_t st) {
    if (nframes > 0) k_md_mtk_half1<<<nframes, 256, 0, st>>>(F, mass_type, x, v, acc, dt, th);
}

void launch_md_mtk_half2(int nframes, const FramesDev& F, const double* Fo, const double* inv_mass_type,
                         const double* mass_type, double* acc, double* v, double dt, double* th, double* ke,
                         cudaStream_t st) {
    if (nframes > 0) k_md_mtk_half2<<<nframes, 256, 0, st>>>(F, Fo, inv_mass_type, mass_type, acc, v, dt, th, ke);
}

void launch_md_berend(int nframes, const FramesDev& F, const double* mass_type, double* v, double dt, double tau,
                      double T0, double kb, double* ke, int* bad, cudaStream_t st) {
    if (nframes > 0) k_md_berend<<<nframes, 256, 0, st>>>(F, mass_type, v, dt, tau, T0, kb, ke, bad);
}

// CONSTRAINT::CONSERVED_QUANT src/ClassDefs.C:1481-1511.
__global__ void k_md_conserved(int nframes, const double* th, int mode, double p0, const BoxDev* box, double* out) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nframes) return;
    const double* t = th + (size_t)f * MD_TH_STRIDE;
    if (mode == 1) {
        out[f] = 0.5 * t[TH_ZETA] * t[TH_ZETA] * t[TH_Q] + t[TH_NDOFKT] * t[TH_POSIT];
    } else if (mode == 2) {
        const double tke = 0.5 * t[TH_ZETA] * t[TH_ZETA] * t[TH_Q];
        const double bke = 0.5 * t[TH_BVEL] * t[TH_BVEL] * t[TH_W];
        const double tpe = t[TH_NDOF1KT] * t[TH_POSIT];
        const double bpe = p0 * box[f].vol;
        out[f] = tke + tpe + bke + bpe;
    } else {
        out[f] = 0.0;
    }
}

void launch_md_conserved(int nframes, const double* th, int mode, double p0, const BoxDev* box, double* out,
                         cudaStream_t st) {
    if (nframes > 0) k_md_conserved<<<(nframes + 127) / 128, 128, 0, st>>>(nframes, th, mode, p0, box, out);
}

// ------------------------------------------------------------------ barostats
// An orthorhombic cell scaled by (sx, sy, sz): H, H^-1, lengths, volume (BOX::UPDATE_CELL
// for CELL_AX / BY / CZ only; the neighbour convention of the frame is kept).
__device__ void box_scale(BoxDev& B, double sx, double sy, double sz) {
    B.h[0] *= sx; B.h[4] *= sy; B.h[8] *= sz;
    B.inv[0] = 1.0 / B.h[0]; B.inv[4] = 1.0 / B.h[4]; B.inv[8] = 1.0 / B.h[8];
    B.lx = B.h[0]; B.ly = B.h[4]; B.lz = B.h[8];
    B.vol = B.h[0] * B.h[4] * B.h[8];
}

// NPT-BEREND (-ANISO), CONSTRAINT::UPDATE_COORDS src/ClassDefs.C:883-1001 with the plain
// first velocity half: K of v(t), x += v dt + a dt^2 / 2, v += a dt / 2, then
// mu = (1 - dt / kp (P0 - P))^(1/3) with P = PRESSURE_XYZ + 2 K / (3 V) (or the tensor
// diagonal + 2 K / (3 V) per axis), x *= mu and the cell *= mu.
__global__ void k_md_npt_berend(FramesDev F, BoxDev* box, const double* mass_type, double* x, double* v,
                                const double* a, double dt, const double* so_prev, double p0, double kp, int aniso,
                                int* bad) {
    __shared__ double red[32];
    const int f = blockIdx.x;
    const int N = F.natoms[f];
    const int64_t aofs = F.atom_ofs[f];
    double k = 0.0;
    for (int i = threadIdx.x; i < 3 * N; i += blockDim.x) {
        const int64_t g = 3 * aofs + i;
        k += 0.5 * mass_type[F.type[aofs + i / 3]] * v[g] * v[g];
    }
    k = block_sum(k, red);
    BoxDev& B = box[f];
    const double v0 = B.vol;
    const double* so = so_prev + (size_t)f * MD_NSCALAR;
    double mu[3];
    bool ok = true;
    if (!aniso) {
        const double P = so[1] + 2.0 * k / (3.0 * v0);
        const double fac = 1.0 - dt / kp * (p0 - P);
        ok = fac >= 0.0;
        mu[0] = mu[1] = mu[2] = pow(fac, 1.0 / 3.0);
    } else {
        for (int d = 0; d < 3; ++d) {
            const double pd = so[2 + 4 * d] + 2.0 / 3.0 * k / v0;
            const double fac = 1.0 - dt / kp * (p0 - pd);
            ok = ok && fac >= 0.0;
            mu[d] = pow(fac, 1.0 / 3.0);
        }
    }
    if (!ok) {   // the reference stops: negative Berendsen scaling factor
        if (threadIdx.x == 0) atomicExch(bad, 1);
        return;
    }
    for (int i = threadIdx.x; i < 3 * N; i += blockDim.x) {
        const int64_t g = 3 * aofs + i;
        double xi = x[g];
        xi += v[g] * dt + 0.5 * a[g] * dt * dt;
        v[g] = v[g] + 0.5 * a[g] * dt;
        x[g] = xi * mu[i % 3];
    }
    __syncthreads();
    if (threadIdx.x == 0) box_scale(B, mu[0], mu[1], mu[2]);
}

// NPT-MTK first half (one block per frame): the state shift of UPDATE_COORDS, K of
// v(t); x += v dt + a dt^2/2 - zeta0 v dt^2/2; the thermostat position; barostat
// position eps = eps0 + veps0 dt + dt^2/2 (Feps0 / W - veps0 zeta0), scale
// s = exp(eps - eps0); x -= dt^2/2 (2 + 3/N_DOF) veps0 v, then x = s (x - com) + com and
// the cell *= s; v_iter = (v + a dt/2 - zeta0 v dt/2 - (2 + 3/N_DOF) veps0 v dt/2) s.
__global__ void k_md_nptmtk_half1(FramesDev F, BoxDev* box, const double* mass_type, double* x, double* v,
                                  const double* a, double dt, double* th) {
    __shared__ double red[32];
    const int f = blockIdx.x;
    const int N = F.natoms[f];
    const int64_t aofs = F.atom_ofs[f];
    double* t = th + (size_t)f * MD_TH_STRIDE;
    double k = 0.0, mt = 0.0;
    for (int i = threadIdx.x; i < 3 * N; i += blockDim.x) {
        const int64_t g = 3 * aofs + i;
        const double m = mass_type[F.type[aofs + i / 3]];
        k += 0.5 * m * v[g] * v[g];
        if (i % 3 == 0) mt += m;
    }
    k = block_sum(k, red);
    mt = block_sum(mt, red);
    const double z0 = t[TH_ZETA], f0 = t[TH_FORCE];
    const double bp0 = t[TH_BPOS], bv0 = t[TH_BVEL], bf0 = t[TH_BFORCE], W = t[TH_W];
    const double cdof = 2.0 + 3.0 / t[TH_NDOF];
    const double bpT = bp0 + bv0 * dt + 0.5 * dt * dt * bf0 / W - 0.5 * dt * dt * bv0 * z0;
    const double sc = exp(bpT - bp0);
    // drift and thermostat, then the centre of mass of those positions
    double cm[3] = {0.0, 0.0, 0.0};
    for (int i = threadIdx.x; i < 3 * N; i += blockDim.x) {
        const int64_t g = 3 * aofs + i;
        const double vi = v[g], ai = a[g];
        double xi = x[g] + (vi * dt + 0.5 * ai * dt * dt);
        xi -= 0.5 * z0 * vi * dt * dt;
        x[g] = xi;
        cm[i % 3] += mass_type[F.type[aofs + i / 3]] * xi;
    }
    double com[3];
    for (int d = 0; d < 3; ++d) com[d] = block_sum(cm[d], red) / mt;
    for (int i = threadIdx.x; i < 3 * N; i += blockDim.x) {
        const int64_t g = 3 * aofs + i;
        const double vi = v[g], ai = a[g];
        double xi = x[g];
        xi -= 0.5 * dt * dt * cdof * bv0 * vi;
        x[g] = sc * (xi - com[i % 3]) + com[i % 3];
        double vn = vi + 0.5 * ai * dt;
        vn -= 0.5 * z0 * vi * dt;
        vn -= 0.5 * cdof * bv0 * vi * dt;
        v[g] = vn * sc;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        t[TH_KCUR] = k;
        t[TH_ZETA0] = z0;
        t[TH_FORCE0] = f0;
        t[TH_BVEL0] = bv0;
        t[TH_BFORCE0] = bf0;
        t[TH_POSIT0] = t[TH_POSIT];
        t[TH_POSIT] = t[TH_POSIT] + z0 * dt + 0.5 * dt * dt * f0;
        t[TH_BPOS0] = bp0;
        t[TH_BPOS] = bpT;
        t[TH_SCALE] = sc;
        t[TH_VOL0] = t[TH_VOL];
        box_scale(box[f], sc, sc, sc);
        t[TH_VOL] = box[f].vol;
    }
}

// NPT-MTK second half (one block per frame), UPDATE_VELOCS_HALF_2 src/ClassDefs.C:1262-1419:
// u = v_iter + a dt/2; initial guess from K(v(t)); then 10 rounds of v = u / s,
// K = K(u) / s^2, barostat force 3/N_DOF 2K + 3 V (P + 2K/(3V) - P0), thermostat
// force (2K + W veps^2 - (N_DOF+1) kB T) / Q, zeta, veps and s; v keeps the last
// round's u / s.
__global__ void k_md_nptmtk_half2(FramesDev F, const double* Fo, const double* inv_mass_type,
                                  const double* mass_type, const double* so, double p0, double* acc, double* v,
                                  double dt, double* th, double* ke) {
    __shared__ double red[32];
    const int f = blockIdx.x;
    const int N = F.natoms[f];
    const int64_t aofs = F.atom_ofs[f];
    double* t = th + (size_t)f * MD_TH_STRIDE;
    double ku = 0.0;
    for (int i = threadIdx.x; i < 3 * N; i += blockDim.x) {
        const int64_t g = 3 * aofs + i;
        const int ty = F.type[aofs + i / 3];
        const double ai = Fo[g] * inv_mass_type[ty];
        acc[g] = ai;
        const double u = v[g] + 0.5 * ai * dt;
        v[g] = u;
        ku += 0.5 * mass_type[ty] * u * u;
    }
    ku = block_sum(ku, red);
    const double Q = t[TH_Q], W = t[TH_W], ndof = t[TH_NDOF], n1kt = t[TH_NDOF1KT];
    const double z0 = t[TH_ZETA0], f0 = t[TH_FORCE0], bv0 = t[TH_BVEL0], bf0 = t[TH_BFORCE0];
    const double VT = t[TH_VOL], P = so[(size_t)f * MD_NSCALAR + 1];
    const double cdof = 2.0 + 3.0 / ndof;
    double K = t[TH_KCUR];
    double dP = P + 2.0 * K / (3.0 * VT) - p0;
    double bfT = 3.0 / ndof * 2.0 * K + 3.0 * VT * dP;
    double tfT = (2.0 * K + W * bv0 * bv0 - n1kt) / Q;
    double zT = z0 + (f0 + tfT) * 0.5 * dt;
    double bvT = bv0 + 0.5 * dt * (bf0 / W - bv0 * z0 + bfT / W - bv0 * zT);
    double s = 1.0 + 0.5 * dt * (zT + cdof * bvT);
    double s_used = s;
    for (int itr = 0; itr < 10; ++itr) {
        s_used = s;
        K = ku / (s_used * s_used);
        dP = P + 2.0 * K / (3.0 * VT) - p0;
        bfT = 3.0 / ndof * 2.0 * K + 3.0 * VT * dP;
        tfT = (2.0 * K + W * bvT * bvT - n1kt) / Q;
        zT = z0 + (f0 + tfT) * 0.5 * dt;
        bvT = bv0 + 0.5 * dt * (bf0 / W - bv0 * z0 + bfT / W - bvT * zT);
        s = 1.0 + 0.5 * dt * (zT + cdof * bvT);
    }
    double k = 0.0;
    for (int i = threadIdx.x; i < 3 * N; i += blockDim.x) {
        const int64_t g = 3 * aofs + i;
        const double vn = v[g] / s_used;
        v[g] = vn;
        k += 0.5 * mass_type[F.type[aofs + i / 3]] * vn * vn;
    }
    k = block_sum(k, red);
    if (threadIdx.x == 0) {
        t[TH_ZETA] = zT;
        t[TH_FORCE] = tfT;
        t[TH_BVEL] = bvT;
        t[TH_BFORCE] = bfT;
        t[TH_VSCALE] = s;
        if (ke) ke[f] = k;
    }
}

__global__ void k_md_vscale(FramesDev F, const double* mass_type, double* v, double* th, int step, int freq,
                            double T0, double kb) {
    __shared__ double red[32];
    const int f = blockIdx.x;
    const int N = F.natoms[f];
    const int64_t aofs = F.atom_ofs[f];
    double* t = th + (size_t)f * MD_TH_STRIDE;
    double k = 0.0;
    for (int i = threadIdx.x; i < 3 * N; i += blockDim.x) {
        const int64_t g = 3 * aofs + i;
        k += 0.5 * mass_type[F.type[aofs + i / 3]] * v[g] * v[g];
    }
    k = block_sum(k, red);
    const double T = 2.0 * k / (t[TH_NDOF] * kb);
    if ((step + 1) % freq != 0) {
        if (threadIdx.x == 0) t[TH_TAVG] += T;
        return;
    }
    double avg = t[TH_TAVG] + T;
    avg /= freq;
    const double s = sqrt(T0 / avg);
    for (int i = threadIdx.x; i < 3 * N; i += blockDim.x) v[3 * aofs + i] *= s;
    if (threadIdx.x == 0) t[TH_TAVG] = 0.0;
}

void launch_md_vscale(int nframes, const FramesDev& F, const double* mass_type, double* v, double* th, int step,
                      int freq, double T0, double kb, cudaStream_t st) {
    if (nframes > 0) k_md_vscale<<<nframes, 256, 0, st>>>(F, mass_type, v, th, step, freq, T0, kb);
}

__global__ void k_md_volume(int nframes, const BoxDev* box, double* out) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f < nframes) out[f] = box[f].vol;
}

void launch_md_npt_berend(int nframes, const FramesDev& F, BoxDev* box, const double* mass_type, double* x,
                          double* v, const double* acc, double dt, const double* so_prev, double p0, double kp,
                          int aniso, int* bad, cudaStream_t st) {
    if (nframes > 0)
        k_md_npt_berend<<<nframes, 256, 0, st>>>(F, box, mass_type, x, v, acc, dt, so_prev, p0, kp, aniso, bad);
}

void launch_md_nptmtk_half1(int nframes, const FramesDev& F, BoxDev* box, const double* mass_type, double* x,
                            double* v, const double* acc, double dt, double* th, cudaStream_t st) {
    if (nframes > 0) k_md_nptmtk_half1<<<nframes, 256, 0, st>>>(F, box, mass_type, x, v, acc, dt, th);
}

void launch_md_nptmtk_half2(int nframes, const FramesDev& F, const double* Fo, const double* inv_mass_type,
                            const double* mass_type, const double* so, double p0, double* acc, double* v, double dt,
                            double* th, double* ke, cudaStream_t st) {
    if (nframes > 0)
        k_md_nptmtk_half2<<<nframes, 256, 0, st>>>(F, Fo, inv_mass_type, mass_type, so, p0, acc, v, dt, th, ke);
}

void launch_md_volume(int nframes, const BoxDev* box, double* out, cudaStream_t st) {
    if (nframes > 0) k_md_volume<<<(nframes + 127) / 128, 128, 0, st>>>(nframes, box, out);
}

}  // namespace cgd
