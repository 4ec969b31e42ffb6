// Ewald charge columns of the force rows (FITCOUL): ZCalc_Ewald_Deriv,
// src/Ewald.C:477-750.  Column p of atom a's x/y/z rows holds the Coulomb force
// on a per unit q_i q_j of pair type p (charges in electron units, ke = 1).
//
// Real space: the reference walks its half neighbour list (i <= PARENT[g], or the
// unordered small-cell list with PERM_SCALE 1/2) and adds each pair term to both
// atoms.  Summed per atom that is, for either list convention, the sum over every
// image g != a within the cut-off of t(r) (r_g - r_a); the images of a itself
// cancel in pairs.  One warp gathers it per atom (no atomics, fixed order).
//
// k space: the reference sums over all atom pairs and k vectors (O(N^2 K)).  With
// species structure factors S_t(k) = sum_{b of type t} exp(i k.r_b) the same sum
// for atom a is sum_k C_k k Im(exp(-i k.r_a) S_t(k)) (the b = a term is sin 0),
// O(N K) per frame.  The k set, weights and constants are the reference's: k
// components 0..kmax with 0 < |k|^2 < 50, the sign variants (kx,-ky,kz),
// (kx,-ky,-kz), (kx,ky,-kz), a factor 2 for kx > 0, phases with M_PI and k vectors
// and prefactors with the truncated PI = 3.14159265359 of that function.
// Every sum is FP64.  Orthorhombic cells only (as the reference).
#include <cuda_runtime.h>

#include <cstdint>

#include "kernels.h"
#include "md.h"

namespace cgd {

constexpr double EW_PI = 3.14159265359;   // src/Ewald.C:489
constexpr int EW_KD = 8;                  // k components 0..7 (|k|^2 < 50)
constexpr int EW_NQ = EW_KD * EW_KD * EW_KD;
constexpr int EW_MAXT = 10;               // atom types (make_id_int is base 10)

__device__ __forceinline__ int ew_frame_of_atom(const FramesDev& F, int64_t a) {
    int lo = 0, hi = F.nframes - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (F.atom_ofs[mid] <= a) lo = mid; else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ double ew_warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// k index q = (kx, ky, kz) in loop order; false when the reference skips it.
__device__ __forceinline__ bool ew_kvec(int q, int kmax, int& kx, int& ky, int& kz) {
    kx = q / (EW_KD * EW_KD); ky = (q / EW_KD) % EW_KD; kz = q % EW_KD;
    const int ksq = kx * kx + ky * ky + kz * kz;
    return kx <= kmax && ky <= kmax && kz <= kmax && ksq != 0 && ksq < 50;
}

// exp(i phi) of the four sign variants from the three axis phases:
// v0 (a+b+c), v1 (a-b+c), v2 (a-b-c), v3 (a+b-c)  (add_sines src/Ewald.C:752-795)
__device__ __forceinline__ void ew_phases(double sa, double ca, double sb, double cb, double sc, double cc,
                                          double (&s)[4], double (&c)[4]) {
    // e^{i(b+c)}, e^{i(-b+c)}, e^{i(-b-c)}, e^{i(b-c)}
    const double spp = sb * cc + cb * sc, cpp = cb * cc - sb * sc;
    const double smp = -sb * cc + cb * sc, cmp = cb * cc + sb * sc;
    const double syz[4] = {spp, smp, -spp, -smp};
    const double cyz[4] = {cpp, cmp, cpp, cmp};
#pragma unroll
    for (int v = 0; v < 4; ++v) {
        s[v] = sa * cyz[v] + ca * syz[v];
        c[v] = ca * cyz[v] - sa * syz[v];
    }
}

// ---------------------------------------------------------------- real space
__global__ void __launch_bounds__(256) k_ewald_real(ModelDev M, FramesDev F, int nreal, void* A, int64_t lda,
                                                    int is_double) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= nreal) return;
    const int f = ew_frame_of_atom(F, warp);
    const int N = F.natoms[f];
    const int64_t aofs = F.atom_ofs[f];
    const int i = warp - (int)aofs;
    const int64_t gb = F.ghost_ofs[f];
    const BoxDev& B = F.box[f];
    const double alpha = B.ew_alpha, rc = B.ew_rc;
    const float4* c32 = reinterpret_cast<const float4*>(F.cart32);
    const float4 xi = c32[gb + i];
    const int* typ = F.type + aofs;
    double acc[EW_MAXT][3];
#pragma unroll
    for (int t = 0; t < EW_MAXT; ++t) acc[t][0] = acc[t][1] = acc[t][2] = 0.0;
    const int nimg_n = F.nimg * N;
    for (int j = lane; j < nimg_n; j += 32) {
        if (j == i) continue;
        const float4 xj = c32[gb + j];
        const float dx = xj.x - xi.x, dy = xj.y - xi.y, dz = xj.z - xi.z;
        if (sqrtf(dx * dx + dy * dy + dz * dz) > (float)rc + 1.0e-2f) continue;
        double R[3];
        const double r = dist_exact(B.h, F.scaled + 3 * (gb + i), F.scaled + 3 * (gb + j), R);
        if (!(r < rc)) continue;
        double t = ((-2.0 / sqrt(EW_PI)) * exp(-1 * alpha * alpha * r * r) * r * alpha - erfc(alpha * r)) / (r * r);
        t *= -1.0;
        t *= 2.0;
        t *= 0.5 / r;
        t *= B.perm2;
        const int ty = typ[j % N];
#pragma unroll
        for (int tt = 0; tt < EW_MAXT; ++tt)
            if (tt == ty) { acc[tt][0] += t * R[0]; acc[tt][1] += t * R[1]; acc[tt][2] += t * R[2]; }
    }
    const int ti = typ[i];
    const int64_t row = F.row_ofs[f] + 3 * (int64_t)i;
    for (int tt = 0; tt < M.natmtyp && tt < EW_MAXT; ++tt) {
        const double s0 = ew_warp_sum(acc[tt][0]), s1 = ew_warp_sum(acc[tt][1]), s2 = ew_warp_sum(acc[tt][2]);
        if (lane == 0) {
            const int64_t col = M.tot_short + M.int_pair_map[ti * M.natmtyp + tt];
            const double v[3] = {-s0, -s1, -s2};   // the final sign flip of src/Ewald.C:738-747
            for (int q = 0; q < 3; ++q) {
                const int64_t idx = (row + q) * lda + col;
                if (is_double) reinterpret_cast<double*>(A)[idx] += v[q];
                else reinterpret_cast<float*>(A)[idx] += (float)v[q];
            }
        }
    }
}

// ---------------------------------------------------------------- k space
// S[((f * EW_NQ + q) * 4 + v) * natmtyp + t] for the valid k of each frame.
__global__ void __launch_bounds__(128) k_ewald_sfac(ModelDev M, FramesDev F, double2* S) {
    const int f = blockIdx.y;
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= EW_NQ) return;
    const BoxDev& B = F.box[f];
    int kx, ky, kz;
    if (!ew_kvec(q, B.ew_kmax, kx, ky, kz)) return;
    const int N = F.natoms[f];
    const int64_t aofs = F.atom_ofs[f], gb = F.ghost_ofs[f];
    const int* typ = F.type + aofs;
    const int nt = M.natmtyp;
    for (int t = 0; t < nt; ++t) {
        double sr[4] = {0, 0, 0, 0}, si[4] = {0, 0, 0, 0};
        for (int b = 0; b < N; ++b) {
            if (typ[b] != t) continue;
            const double* sb = F.scaled + 3 * (gb + b);   // fractional coordinates (r / L)
            double sa_, ca_, sb_, cb_, sc_, cc_;
            sincos(2.0 * M_PI * sb[0] * kx, &sa_, &ca_);
            sincos(2.0 * M_PI * sb[1] * ky, &sb_, &cb_);
            sincos(2.0 * M_PI * sb[2] * kz, &sc_, &cc_);
            double s[4], c[4];
            ew_phases(sa_, ca_, sb_, cb_, sc_, cc_, s, c);
#pragma unroll
            for (int v = 0; v < 4; ++v) { sr[v] += c[v]; si[v] += s[v]; }
        }
        for (int v = 0; v < 4; ++v) S[(((int64_t)f * EW_NQ + q) * 4 + v) * nt + t] = make_double2(sr[v], si[v]);
    }
}

__global__ void __launch_bounds__(256) k_ewald_kspace(ModelDev M, FramesDev F, int nreal, const double2* S, void* A,
                                                      int64_t lda, int is_double) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= nreal) return;
    const int f = ew_frame_of_atom(F, warp);
    const int64_t aofs = F.atom_ofs[f], gb = F.ghost_ofs[f];
    const int i = warp - (int)aofs;
    const BoxDev& B = F.box[f];
    const int nt = M.natmtyp;
    const double L[3] = {B.h[0], B.h[4], B.h[8]};
    const double alphasq = B.ew_alpha * B.ew_alpha;
    const double* sa = F.scaled + 3 * (gb + i);
    double acc[EW_MAXT][3];
#pragma unroll
    for (int t = 0; t < EW_MAXT; ++t) acc[t][0] = acc[t][1] = acc[t][2] = 0.0;
    for (int q = lane; q < EW_NQ; q += 32) {
        int kx, ky, kz;
        if (!ew_kvec(q, B.ew_kmax, kx, ky, kz)) continue;
        const double rk[3] = {(2.0 * EW_PI / L[0]) * kx, (2.0 * EW_PI / L[1]) * ky, (2.0 * EW_PI / L[2]) * kz};
        const double rksq = rk[0] * rk[0] + rk[1] * rk[1] + rk[2] * rk[2];
        const double kfac = exp(-rksq / (4.0 * alphasq)) / rksq;
        double w = 2.0 * kfac * 0.5 * (4 * EW_PI / B.vol);
        if (kx > 0) w *= 2.0;
        double s_, c_, s2, c2, s3, c3;
        sincos(2.0 * M_PI * sa[0] * kx, &s_, &c_);
        sincos(2.0 * M_PI * sa[1] * ky, &s2, &c2);
        sincos(2.0 * M_PI * sa[2] * kz, &s3, &c3);
        double sp[4], cp[4];
        ew_phases(s_, c_, s2, c2, s3, c3, sp, cp);
        const bool has[4] = {true, ky > 0, ky > 0 && kz > 0, kz > 0};
        const double sy[4] = {1.0, -1.0, -1.0, 1.0}, sz[4] = {1.0, 1.0, -1.0, -1.0};
        for (int v = 0; v < 4; ++v) {
            if (!has[v]) continue;
            const double2* Sv = S + (((int64_t)f * EW_NQ + q) * 4 + v) * nt;
            for (int t = 0; t < nt && t < EW_MAXT; ++t) {
                // Im(exp(-i phi_a) S_t) = sum_b sin(k.(r_b - r_a))
                const double im = Sv[t].y * cp[v] - Sv[t].x * sp[v];
                const double g = w * im;
#pragma unroll
                for (int tt = 0; tt < EW_MAXT; ++tt)
                    if (tt == t) {
                        acc[tt][0] += g * rk[0];
                        acc[tt][1] += g * (sy[v] * rk[1]);
                        acc[tt][2] += g * (sz[v] * rk[2]);
                    }
            }
        }
    }
    const int ti = F.type[aofs + i];
    const int64_t row = F.row_ofs[f] + 3 * (int64_t)i;
    for (int tt = 0; tt < nt && tt < EW_MAXT; ++tt) {
        const double s0 = ew_warp_sum(acc[tt][0]), s1 = ew_warp_sum(acc[tt][1]), s2v = ew_warp_sum(acc[tt][2]);
        if (lane == 0) {
            const int64_t col = M.tot_short + M.int_pair_map[ti * nt + tt];
            const double v[3] = {-s0, -s1, -s2v};
            for (int c = 0; c < 3; ++c) {
                const int64_t idx = (row + c) * lda + col;
                if (is_double) reinterpret_cast<double*>(A)[idx] += v[c];
                else reinterpret_cast<float*>(A)[idx] += (float)v[c];
            }
        }
    }
}

// ---------------------------------------------------------------- MD (fixed charges)
// ZCalc_Ewald / Ewald_K_Space_New (src/Ewald.C:28-426) with ke = 332.0637157615209
// (src/functions.h:40).  Real space: each atom gathers the pair force of every image
// g != a within r_c (the reference's half-list updates of both atoms sum to that);
// energy and virial take the half list's entries, i.e. the images with parent >= a
// (big cells) or all images with PERM_SCALE 1/2 (small cells).  k space over the full
// sphere |k|^2 < k_cut^2 of integer k in [-k_cut, k_cut]^3: S(k) = sum_b q_b exp(i k.r_b),
// energy ke (2 pi / V) sum_k Kfac |S|^2 - ke alpha / sqrt(pi) sum q^2, the Heyes
// virial tensor, forces -4 pi ke Kfac q_a (C sin - S cos) / V k.  The pressure term is
// the Coulomb energy (Hummer et al.).
constexpr double MD_KE = 332.0637157615209;

__global__ void __launch_bounds__(256) k_md_ewald_real(MdDev D, FramesDev F, int nreal, double* Fo, double* So) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= nreal) return;
    const int f = ew_frame_of_atom(F, warp);
    const int N = F.natoms[f];
    const int64_t aofs = F.atom_ofs[f];
    const int i = warp - (int)aofs;
    const int64_t gb = F.ghost_ofs[f];
    const BoxDev& B = F.box[f];
    const double alpha = B.ew_alpha, rc = B.ew_rc;
    const float4* c32 = reinterpret_cast<const float4*>(F.cart32);
    const float4 xi = c32[gb + i];
    const int* typ = F.type + aofs;
    const double qi = D.qtype[typ[i]];
    const bool small = B.small != 0;
    const double perm = B.perm2;
    double fx = 0, fy = 0, fz = 0, u = 0, w[6] = {0, 0, 0, 0, 0, 0};
    const int nimg_n = F.nimg * N;
    for (int j = lane; j < nimg_n; j += 32) {
        if (j == i) continue;
        const float4 xj = c32[gb + j];
        const float dx = xj.x - xi.x, dy = xj.y - xi.y, dz = xj.z - xi.z;
        if (sqrtf(dx * dx + dy * dy + dz * dz) > (float)rc + 1.0e-2f) continue;
        double R[3];
        const double r = dist_exact(B.h, F.scaled + 3 * (gb + i), F.scaled + 3 * (gb + j), R);
        if (!(r < rc)) continue;
        const double qq = qi * D.qtype[typ[j % N]];
        const double ef = erfc(alpha * r);
        const double td = ((-2.0 / sqrt(M_PI)) * exp(-1.0 * alpha * alpha * r * r) * r * alpha - ef) / (r * r * r);
        const double tx = -td * qq * MD_KE;   // the pair force on a is R * tx (R = r_g - r_a) with a minus sign
        fx -= R[0] * tx; fy -= R[1] * tx; fz -= R[2] * tx;
        const bool listed = small || (j % N) >= i;   // the reference's half list
        if (listed) {
            const double wgt = small ? perm : 1.0;
            u += MD_KE * qq * (ef / r) * wgt;
            const double t = tx * wgt;
            w[0] += t * R[0] * R[0]; w[1] += t * R[0] * R[1]; w[2] += t * R[0] * R[2];
            w[3] += t * R[1] * R[1]; w[4] += t * R[1] * R[2]; w[5] += t * R[2] * R[2];
        }
    }
    fx = ew_warp_sum(fx); fy = ew_warp_sum(fy); fz = ew_warp_sum(fz); u = ew_warp_sum(u);
    for (int k = 0; k < 6; ++k) w[k] = ew_warp_sum(w[k]);
    if (lane == 0) {
        double* fo = Fo + 3 * (aofs + i);
        fo[0] += fx; fo[1] += fy; fo[2] += fz;   // one warp owns atom a
        double* so = So + (size_t)f * MD_NSCALAR;
        atomicAdd(so + 0, u);
        atomicAdd(so + 1, u);
        atomicAdd(so + 2, w[0]); atomicAdd(so + 3, w[1]); atomicAdd(so + 4, w[2]);
        atomicAdd(so + 5, w[1]); atomicAdd(so + 6, w[3]); atomicAdd(so + 7, w[4]);
        atomicAdd(so + 8, w[2]); atomicAdd(so + 9, w[4]); atomicAdd(so + 10, w[5]);
    }
}

__device__ __forceinline__ bool md_kvec(int q, int kmax, int& kx, int& ky, int& kz) {
    const int side = 2 * kmax + 1;
    kx = q / (side * side) - kmax; ky = (q / side) % side - kmax; kz = q % side - kmax;
    const int ksq = kx * kx + ky * ky + kz * kz;
    return ksq != 0 && ksq < kmax * kmax;
}

// Per frame and k: S(k) (cos and sin sums); energy and virial of that k.
__global__ void __launch_bounds__(128) k_md_ewald_sfac(MdDev D, FramesDev F, int kmax_max, double2* Sk, double* So) {
    const int f = blockIdx.y;
    const BoxDev& B = F.box[f];
    const int kmax = B.ew_kmax;
    const int side = 2 * kmax + 1, nq = side * side * side;
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    const int side_max = 2 * kmax_max + 1;
    double e = 0, w[6] = {0, 0, 0, 0, 0, 0};
    int kx, ky, kz;
    if (q < nq && md_kvec(q, kmax, kx, ky, kz)) {
        const int N = F.natoms[f];
        const int64_t aofs = F.atom_ofs[f];
        const double L[3] = {B.h[0], B.h[4], B.h[8]};
        const double kv[3] = {(2.0 * M_PI / L[0]) * kx, (2.0 * M_PI / L[1]) * ky, (2.0 * M_PI / L[2]) * kz};
        const double alphasq = B.ew_alpha * B.ew_alpha;
        const double rksq = kv[0] * kv[0] + kv[1] * kv[1] + kv[2] * kv[2];
        const double kfac = exp(-rksq / (4.0 * alphasq)) / rksq;
        double cs = 0.0, sn = 0.0;
        for (int b = 0; b < N; ++b) {
            const double* x = F.xyz + 3 * (aofs + b);
            const double kr = x[0] * kv[0] + x[1] * kv[1] + x[2] * kv[2];
            double sv, cv;
            sincos(kr, &sv, &cv);
            const double qb = D.qtype[F.type[aofs + b]];
            cs += qb * cv;
            sn += qb * sv;
        }
        Sk[(size_t)f * side_max * side_max * side_max + q] = make_double2(cs, sn);
        const double kw = kfac * (cs * cs + sn * sn);
        const double V = (B.h[0] * B.h[4] * B.h[8]);
        const double pre = 2 * M_PI * MD_KE / V;
        e = kw;
        w[0] = pre * kw * (1.0 - 2.0 * kv[0] * kv[0] / rksq - 0.5 * kv[0] * kv[0] / alphasq);
        w[3] = pre * kw * (1.0 - 2.0 * kv[1] * kv[1] / rksq - 0.5 * kv[1] * kv[1] / alphasq);
        w[5] = pre * kw * (1.0 - 2.0 * kv[2] * kv[2] / rksq - 0.5 * kv[2] * kv[2] / alphasq);
        w[1] = pre * kw * (-2.0 * kv[0] * kv[1] / rksq - 0.5 * kv[0] * kv[1] / alphasq);
        w[2] = pre * kw * (-2.0 * kv[0] * kv[2] / rksq - 0.5 * kv[0] * kv[2] / alphasq);
        w[4] = pre * kw * (-2.0 * kv[1] * kv[2] / rksq - 0.5 * kv[1] * kv[2] / alphasq);
    } else if (q < side_max * side_max * side_max) {
        Sk[(size_t)f * side_max * side_max * side_max + q] = make_double2(0.0, 0.0);
    }
    // block sums -> frame scalars: energy ke (2 pi / V) sum kw (pressure term the same)
    __shared__ double red[7][4];
    double vals[7] = {e, w[0], w[1], w[2], w[3], w[4], w[5]};
    for (int k = 0; k < 7; ++k) {
        double v = ew_warp_sum(vals[k]);
        if ((threadIdx.x & 31) == 0) red[k][threadIdx.x >> 5] = v;
    }
    __syncthreads();
    if (threadIdx.x < 7) {
        double s = 0.0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += red[threadIdx.x][i];
        double* so = So + (size_t)f * MD_NSCALAR;
        if (s != 0.0) {
            const int k = threadIdx.x;
            if (k == 0) {
                const double uk = MD_KE * (2 * M_PI / (F.box[f].h[0] * F.box[f].h[4] * F.box[f].h[8])) * s;
                atomicAdd(so + 0, uk);
                atomicAdd(so + 1, uk);
            } else if (k == 1) atomicAdd(so + 2, s);
            else if (k == 2) { atomicAdd(so + 3, s); atomicAdd(so + 5, s); }
            else if (k == 3) { atomicAdd(so + 4, s); atomicAdd(so + 8, s); }
            else if (k == 4) atomicAdd(so + 6, s);
            else if (k == 5) { atomicAdd(so + 7, s); atomicAdd(so + 9, s); }
            else atomicAdd(so + 10, s);
        }
    }
}

// Per atom: the k-space force, and the self-energy term (one warp per atom).
__global__ void __launch_bounds__(256) k_md_ewald_kforce(MdDev D, FramesDev F, int nreal, int kmax_max,
                                                         const double2* Sk, double* Fo, double* So) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= nreal) return;
    const int f = ew_frame_of_atom(F, warp);
    const int64_t aofs = F.atom_ofs[f];
    const int i = warp - (int)aofs;
    const BoxDev& B = F.box[f];
    const int kmax = B.ew_kmax;
    const int side = 2 * kmax + 1, nq = side * side * side;
    const int side_max = 2 * kmax_max + 1;
    const double L[3] = {B.h[0], B.h[4], B.h[8]};
    const double alphasq = B.ew_alpha * B.ew_alpha;
    const double V = (B.h[0] * B.h[4] * B.h[8]);
    const double* x = F.xyz + 3 * (aofs + i);
    const double qa = D.qtype[F.type[aofs + i]];
    double fx = 0, fy = 0, fz = 0;
    for (int q = lane; q < nq; q += 32) {
        int kx, ky, kz;
        if (!md_kvec(q, kmax, kx, ky, kz)) continue;
        const double kv[3] = {(2.0 * M_PI / L[0]) * kx, (2.0 * M_PI / L[1]) * ky, (2.0 * M_PI / L[2]) * kz};
        const double rksq = kv[0] * kv[0] + kv[1] * kv[1] + kv[2] * kv[2];
        const double kfac = exp(-rksq / (4.0 * alphasq)) / rksq;
        const double2 s = Sk[(size_t)f * side_max * side_max * side_max + q];
        double sv, cv;
        sincos(x[0] * kv[0] + x[1] * kv[1] + x[2] * kv[2], &sv, &cv);
        const double td = -4.0 * M_PI * kfac * MD_KE * qa * (s.x * sv - s.y * cv) / V;
        fx -= kv[0] * td; fy -= kv[1] * td; fz -= kv[2] * td;   // ACCEL -= TMP_EWALD
    }
    fx = ew_warp_sum(fx); fy = ew_warp_sum(fy); fz = ew_warp_sum(fz);
    if (lane == 0) {
        double* fo = Fo + 3 * (aofs + i);
        fo[0] += fx; fo[1] += fy; fo[2] += fz;
        const double self = -MD_KE * B.ew_alpha / sqrt(M_PI) * qa * qa;
        double* so = So + (size_t)f * MD_NSCALAR;
        atomicAdd(so + 0, self);
        atomicAdd(so + 1, self);
    }
}

size_t md_ewald_scratch_bytes(int nframes, int kmax_max) {
    const size_t side = 2 * (size_t)kmax_max + 1;
    return sizeof(double2) * (size_t)nframes * side * side * side;
}

void launch_md_ewald(int nframes, int nreal, int kmax_max, const ModelDev& M, const MdDev& D, const FramesDev& F,
                     void* S, double* Fo, double* So, cudaStream_t st) {
    (void)M;
    if (!D.coulomb || nreal == 0) return;
    const unsigned wb = (unsigned)(((int64_t)nreal * 32 + 255) / 256);
    k_md_ewald_real<<<wb, 256, 0, st>>>(D, F, nreal, Fo, So);
    const int side = 2 * kmax_max + 1, nq = side * side * side;
    k_md_ewald_sfac<<<dim3((nq + 127) / 128, (unsigned)nframes), 128, 0, st>>>(D, F, kmax_max, (double2*)S, So);
    k_md_ewald_kforce<<<wb, 256, 0, st>>>(D, F, nreal, kmax_max, (const double2*)S, Fo, So);
}

size_t ewald_scratch_bytes(int nframes, int natmtyp) {
    return sizeof(double2) * (size_t)nframes * EW_NQ * 4 * (size_t)natmtyp;
}

void launch_ewald(int prec, int nframes, int nreal, const ModelDev& M, const FramesDev& F, void* S, void* A,
                  int64_t lda, cudaStream_t st) {
    if (M.ncoul == 0 || nreal == 0) return;
    const unsigned wb = (unsigned)(((int64_t)nreal * 32 + 255) / 256);
    k_ewald_real<<<wb, 256, 0, st>>>(M, F, nreal, A, lda, prec == 0);
    k_ewald_sfac<<<dim3((EW_NQ + 127) / 128, (unsigned)nframes), 128, 0, st>>>(M, F, (double2*)S);
    k_ewald_kspace<<<wb, 256, 0, st>>>(M, F, nreal, (const double2*)S, A, lda, prec == 0);
}

}  // namespace cgd
